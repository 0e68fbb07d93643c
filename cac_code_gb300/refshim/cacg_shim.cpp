// One libcacg handle per CAC instance and the transfer of the reference's
// host state into it (see cacg_shim.h).
#include "cacg_shim.h"

#include <stdio.h>
#include <string.h>

#include <map>
#include <vector>

#include "atom.h"
#include "cac.h"
#include "domain.h"
#include "element.h"
#include "error.h"
#include "neighbor.h"
#include "update.h"

using namespace CAC_NS;

namespace {
std::map<CAC *, CacgShim *> &shims() {
  static std::map<CAC *, CacgShim *> m;
  return m;
}
}  // namespace

CacgShim::CacgShim(CAC *cac) : Pointers(cac), h(NULL), tables_pending(1), ready(0) {
  if (cacg_create(&h, 0) != CACG_OK) error->all(FLERR, "libcacg: no usable GPU");
}

CacgShim::~CacgShim() { cacg_destroy(h); }

CacgShim *CacgShim::of(CAC *cac) {
  std::map<CAC *, CacgShim *> &m = shims();
  std::map<CAC *, CacgShim *>::iterator it = m.find(cac);
  if (it != m.end()) return it->second;
  CacgShim *s = new CacgShim(cac);
  m[cac] = s;
  return s;
}

void CacgShim::release(CAC *cac) {
  std::map<CAC *, CacgShim *> &m = shims();
  std::map<CAC *, CacgShim *>::iterator it = m.find(cac);
  if (it == m.end()) return;
  delete it->second;
  m.erase(it);
}

void CacgShim::check(int rc) {
  if (rc != CACG_OK) error->all(FLERR, cacg_error(h));
}

void CacgShim::begin(const char *pair_style_line) {
  char line[256];
  snprintf(line, sizeof(line), "units %s", update->unit_style);
  check(cacg_command(h, line));
  snprintf(line, sizeof(line), "boundary %s %s %s", domain->periodicity[0] ? "p" : "f",
           domain->periodicity[1] ? "p" : "f", domain->periodicity[2] ? "p" : "f");
  check(cacg_command(h, line));
  snprintf(line, sizeof(line), "timestep %.17g", update->dt);
  check(cacg_command(h, line));
  check(cacg_set_box(h, domain->boxlo, domain->boxhi, domain->periodicity));
  check(cacg_set_masses(h, atom->ntypes, atom->mass + 1));
  const int n = atom->nlocal;
  check(cacg_set_atoms(h, n, n ? &atom->x[0][0] : NULL, n ? &atom->v[0][0] : NULL, atom->type));
  const int ne = element->nlocal;
  if (element->ntypes > 0) {
    std::vector<int> nae, numint, intp;
    std::vector<double> w;
    for (int t = 1; t <= element->ntypes; t++) {
      for (int d = 0; d < 3; d++) nae.push_back(element->nae[t][d]);
      numint.push_back(element->numint[t]);
      for (int m = 0; m < element->numint[t]; m++) {
        for (int d = 0; d < 3; d++) intp.push_back(element->intp[t][m][d]);
        w.push_back(element->weight[t][m]);
      }
    }
    check(cacg_set_element_types(h, element->ntypes, &nae[0], &numint[0],
                                 intp.empty() ? NULL : &intp[0], w.empty() ? NULL : &w[0]));
  }
  check(cacg_set_elements(h, ne, element->type, ne ? &element->x[0][0] : NULL,
                          ne ? &element->nodex[0][0][0] : NULL,
                          ne ? &element->nodev[0][0][0] : NULL));
  check(cacg_command(h, pair_style_line));
  snprintf(line, sizeof(line), "neighbor %.17g bin", neighbor->skin);
  check(cacg_command(h, line));
  snprintf(line, sizeof(line), "neigh_modify every %d delay %d check %s", neighbor->every,
           neighbor->delay, neighbor->dist_check ? "yes" : "no");
  check(cacg_command(h, line));
  check(cacg_command(h, "fix 1 all nve"));
  tables_pending = 1;
  ready = 0;
}

void CacgShim::finish_init() {
  check(cacg_init(h));
  check(cacg_setup(h));
  tables_pending = 0;
  ready = 1;
}

void CacgShim::put_state() {
  if (atom->nlocal) check(cacg_put_atoms(h, &atom->x[0][0], &atom->v[0][0]));
  if (element->nlocal) check(cacg_put_nodes(h, &element->nodex[0][0][0], &element->nodev[0][0][0]));
}

void CacgShim::get_state() {
  if (atom->nlocal) check(cacg_get_atoms(h, 0, &atom->x[0][0], &atom->v[0][0], NULL, NULL));
  if (element->nlocal)
    check(cacg_get_elements(h, 0, &element->x[0][0], &element->nodex[0][0][0],
                            &element->nodev[0][0][0], NULL, NULL));
}
