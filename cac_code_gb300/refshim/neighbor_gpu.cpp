// The GPU neighbor builds (see neighbor_gpu.h).
#include "neighbor_gpu.h"

#include "cacg_shim.h"

using namespace CAC_NS;

NeighborGPU::NeighborGPU(CAC *cac) : Neighbor(cac) {}

NeighborGPU::~NeighborGPU() {}

// Neighbor::build after comm->exchange/borders (verlet.cpp:184-198): the
// current positions in, ghosts and bins from them (cacg_setup), then the list
void NeighborGPU::build(int) {
  CacgShim *g = CacgShim::of(cac);
  if (!g->ready) return;  // before the pair style's init: nothing to list yet
  ncalls++;
  g->put_state();
  g->check(cacg_setup(g->h));
  g->check(cacg_neighbor_build(g->h));
}

void NeighborGPU::ebuild(int) {
  CacgShim *g = CacgShim::of(cac);
  if (!g->ready) return;
  g->check(cacg_neighbor_ebuild(g->h));
}

void NeighborGPU::nbuild(int) {
  CacgShim *g = CacgShim::of(cac);
  if (!g->ready) return;
  g->check(cacg_neighbor_nbuild(g->h));
}
