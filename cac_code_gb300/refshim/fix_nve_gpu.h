// fix nve/gpu: FixNVE whose velocity-Verlet half-steps of atoms and nodes
// (fix_nve.cpp:54-242) run on the GPU; positions and velocities cross to the
// reference's host arrays around each call.
#ifdef FIX_CLASS

FixStyle(nve/gpu, FixNVEGPU)

#else

#ifndef CACG_FIX_NVE_GPU_H
#define CACG_FIX_NVE_GPU_H

#include "fix_nve.h"

namespace CAC_NS {

class FixNVEGPU : public FixNVE {
 public:
  FixNVEGPU(class CAC *, int, char **);
  virtual ~FixNVEGPU();
  // atoms and nodes in one call each (the element halves do nothing)
  virtual void initial_integrate(int);
  virtual void einitial_integrate(int);
  virtual void final_integrate();
  virtual void efinal_integrate();
};

}  // namespace CAC_NS

#endif
#endif
