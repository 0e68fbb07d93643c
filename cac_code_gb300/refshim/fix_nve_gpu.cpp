// fix nve/gpu (see fix_nve_gpu.h).
#include "fix_nve_gpu.h"

#include "atom.h"
#include "cacg_shim.h"
#include "element.h"

using namespace CAC_NS;

FixNVEGPU::FixNVEGPU(CAC *cac, int narg, char **arg) : FixNVE(cac, narg, arg) {}

FixNVEGPU::~FixNVEGPU() {}

void FixNVEGPU::initial_integrate(int) {
  CacgShim *g = CacgShim::of(cac);
  g->put_state();
  g->check(cacg_fix_nve_initial_integrate(g->h));
  g->get_state();
}

void FixNVEGPU::einitial_integrate(int) {}

// the forces of the last Pair::compute / ecompute are on the device
void FixNVEGPU::final_integrate() {
  CacgShim *g = CacgShim::of(cac);
  g->check(cacg_fix_nve_final_integrate(g->h));
  g->get_state();
}

void FixNVEGPU::efinal_integrate() {}
