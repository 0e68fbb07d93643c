// Pair styles lj/cut/gpu and eam/gpu: PairLJCut and PairEAM whose compute()
// and ecompute() (pair.h:82-105) run on the GPU through libcacg.  The base
// classes read the coefficients or the potential file and build their tables
// as the reference does (pair_lj_cut.cpp:140-198, pair_eam.cpp:197-580); the
// tables are handed to the library as built (cacg_set_lj, cacg_set_eam).
#ifdef PAIR_CLASS

PairStyle(lj/cut/gpu, PairLJCutGPU)
PairStyle(eam/gpu, PairEAMGPU)

#else

#ifndef CACG_PAIR_GPU_H
#define CACG_PAIR_GPU_H

#include "pair_eam.h"
#include "pair_lj_cut.h"

namespace CAC_NS {

class PairLJCutGPU : public PairLJCut {
 public:
  PairLJCutGPU(class CAC *);
  virtual ~PairLJCutGPU();
  virtual void init_style();
  virtual double init_one(int, int);
  virtual void compute(int, int);
  virtual void ecompute();
};

class PairEAMGPU : public PairEAM {
 public:
  PairEAMGPU(class CAC *);
  virtual ~PairEAMGPU();
  virtual void init_style();
  virtual void compute(int, int);
  virtual void ecompute();
};

}  // namespace CAC_NS

#endif
#endif
