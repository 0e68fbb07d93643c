// lj/cut/gpu and eam/gpu (see pair_gpu.h).
#include "pair_gpu.h"

#include <stdio.h>

#include "atom.h"
#include "cacg_shim.h"
#include "element.h"

using namespace CAC_NS;

// ---- lj/cut/gpu

PairLJCutGPU::PairLJCutGPU(CAC *cac) : PairLJCut(cac) {}

PairLJCutGPU::~PairLJCutGPU() {}

void PairLJCutGPU::init_style() {
  PairLJCut::init_style();
  char line[64];
  snprintf(line, sizeof(line), "pair_style lj/cut %.17g", cut_global);
  CacgShim::of(cac)->begin(line);
}

// the base forms lj1, lj2, cutsq (pair_lj_cut.cpp:140-198); they are handed
// over at the next compute
double PairLJCutGPU::init_one(int i, int j) {
  const double c = PairLJCut::init_one(i, j);
  CacgShim::of(cac)->tables_pending = 1;
  return c;
}

void PairLJCutGPU::compute(int eflag, int vflag) {
  CacgShim *g = CacgShim::of(cac);
  if (g->tables_pending) {
    const int nt = atom->ntypes;
    // row and column 0 are unused; the contiguous (nt + 1)^2 arrays are passed
    g->check(cacg_set_lj(g->h, nt, &lj1[0][0], &lj2[0][0], &cutsq[0][0]));
    g->finish_init();
  }
  g->put_state();
  g->check(cacg_pair_compute(g->h, eflag, vflag));
  if (atom->nlocal) g->check(cacg_get_atoms(g->h, 0, NULL, NULL, &atom->f[0][0], NULL));
}

void PairLJCutGPU::ecompute() {
  CacgShim *g = CacgShim::of(cac);
  g->put_state();
  g->check(cacg_pair_ecompute(g->h));
  if (element->nlocal)
    g->check(cacg_get_elements(g->h, 0, NULL, NULL, NULL, &element->nodef[0][0][0], NULL));
}

// ---- eam/gpu

PairEAMGPU::PairEAMGPU(CAC *cac) : PairEAM(cac) {}

PairEAMGPU::~PairEAMGPU() {}

// the base reads the file and builds the splines (file2array, array2spline,
// pair_eam.cpp:274-282); the one species' splines are handed over as built
void PairEAMGPU::init_style() {
  PairEAM::init_style();
  CacgShim *g = CacgShim::of(cac);
  g->begin("pair_style eam");
  g->check(cacg_set_eam(g->h, nr, dr, nrho, drho, &frho_spline[type2frho[1]][0][0],
                        &rhor_spline[type2rhor[1][1]][0][0], &z2r_spline[type2z2r[1][1]][0][0],
                        cutforcesq, atom->mass[1]));
  g->finish_init();
}

void PairEAMGPU::compute(int eflag, int vflag) {
  CacgShim *g = CacgShim::of(cac);
  g->put_state();
  g->check(cacg_pair_compute(g->h, eflag, vflag));
  if (atom->nlocal) g->check(cacg_get_atoms(g->h, 0, NULL, NULL, &atom->f[0][0], NULL));
}

void PairEAMGPU::ecompute() {
  CacgShim *g = CacgShim::of(cac);
  g->put_state();
  g->check(cacg_pair_ecompute(g->h));
  if (element->nlocal)
    g->check(cacg_get_elements(g->h, 0, NULL, NULL, NULL, &element->nodef[0][0][0], NULL));
}
