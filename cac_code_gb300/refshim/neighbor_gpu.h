// Neighbor with build/ebuild/nbuild (neighbor.h:74-76, virtual) on the GPU:
// the lists of half_bin_no_newton, element_neighbor and node_neighbor are
// built and kept on the device for the GPU pair styles.  Constructed in place
// of Neighbor (cac.cpp:161).
#ifndef CACG_NEIGHBOR_GPU_H
#define CACG_NEIGHBOR_GPU_H

#include "neighbor.h"

namespace CAC_NS {

class NeighborGPU : public Neighbor {
 public:
  NeighborGPU(class CAC *);
  virtual ~NeighborGPU();
  virtual void build(int topoflag = 1);
  virtual void ebuild(int topoflag = 1);
  virtual void nbuild(int topoflag = 1);
};

}  // namespace CAC_NS

#endif
