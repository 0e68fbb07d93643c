// Link check of the reference-side plug-ins (cac_code_gb300/refshim): a
// program that names every GPU style, so that linking it against the
// reference's objects and libcacg.so resolves every symbol they use.  It
// constructs nothing unless given many arguments (it is linked, not run).
#include "mpi.h"

#include "cac.h"
#include "fix_nve_gpu.h"
#include "neighbor_gpu.h"
#include "pair_gpu.h"

int main(int argc, char **argv) {
  if (argc < 1000) return 0;
  CAC_NS::CAC *cac = 0;
  CAC_NS::Pair *a = new CAC_NS::PairLJCutGPU(cac);
  CAC_NS::Pair *b = new CAC_NS::PairEAMGPU(cac);
  CAC_NS::Neighbor *n = new CAC_NS::NeighborGPU(cac);
  CAC_NS::Fix *f = new CAC_NS::FixNVEGPU(cac, argc, argv);
  delete a;
  delete b;
  delete n;
  delete f;
  return 0;
}
