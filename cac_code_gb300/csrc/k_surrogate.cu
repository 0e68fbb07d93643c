// Per-step use of the nodal-force surrogate inside the element force pass.
//
// For the elements far from the atomistic region (a list fixed when the
// surrogate is attached), each step:
//   features  -> 24 nodal displacements about their mean, relative to the
//                ideal node positions, then the 8 nodal densities, normalised
//                and rounded to bf16 [n][64] (zero padded) for the GEMMs;
//   due       -> the far elements tested this step: an element whose spread
//                exceeded the threshold is re-tested after 1, 3, 7, ... 127
//                steps (the quadrature evaluates it meanwhile); an accepted
//                element is tested every step.  The list is compacted on the
//                device, with its length in a device counter;
//   accept    -> skip[e] = (ensemble spread <= threshold); counts evaluated
//                and accepted elements on the device;
//   write     -> nodef[e] = ensemble mean for the accepted elements, after the
//                quadrature's nodal gather (which skipped their force rows).
// The reference has no counterpart: it evaluates every element by quadrature.
#include <cuda_bf16.h>

#include <algorithm>

#include "internal.h"

namespace cacg {
namespace surrogate {

namespace {

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

__device__ __forceinline__ void element_features(const double *__restrict__ nodex,
                                                 const double *__restrict__ nodex0,
                                                 const double *__restrict__ erho, int e,
                                                 float (&f)[MLP_IN]) {
  double u[24], m[3] = {0.0, 0.0, 0.0};
#pragma unroll
  for (int k = 0; k < 24; k++) {
    u[k] = nodex[24 * (size_t) e + k] - nodex0[24 * (size_t) e + k];
    m[k % 3] += u[k];
  }
#pragma unroll
  for (int k = 0; k < 24; k++) f[k] = (float) (u[k] - m[k % 3] * 0.125);
#pragma unroll
  for (int q = 0; q < NPE; q++) f[24 + q] = erho ? (float) erho[NPE * (size_t) e + q] : 0.f;
}

__global__ void k_features(const double *__restrict__ nodex, const double *__restrict__ nodex0,
                           const double *__restrict__ erho, const int *__restrict__ elems, int n,
                           const int *__restrict__ count, const float *__restrict__ norm,
                           __nv_bfloat16 *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (count ? *count : n)) return;
  float f[MLP_IN];
  element_features(nodex, nodex0, erho, elems[i], f);
  __nv_bfloat16 *o = out + 64 * (size_t) i;
#pragma unroll
  for (int c = 0; c < MLP_IN; c++) o[c] = __float2bfloat16((f[c] - norm[c]) * norm[MLP_IN + c]);
#pragma unroll
  for (int c = MLP_IN; c < 64; c++) o[c] = __float2bfloat16(0.f);
}

__global__ void k_raw_features(const double *__restrict__ nodex, const double *__restrict__ nodex0,
                               const double *__restrict__ erho, int n, float *__restrict__ out) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  float f[MLP_IN];
  element_features(nodex, nodex0, erho, e, f);
#pragma unroll
  for (int c = 0; c < MLP_IN; c++) out[(size_t) e * MLP_IN + c] = f[c];
}

// The far elements due for a test this step, compacted into due[] (indices
// into far) with *count; every far element starts the step on the quadrature
__global__ void k_due(int nfar, const int *__restrict__ far, unsigned char *__restrict__ wait,
                      unsigned char *__restrict__ skip, int *__restrict__ due,
                      int *__restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool d = false;
  if (i < nfar) {
    skip[far[i]] = 0;
    const unsigned char w = wait[i];
    d = w == 0;
    if (!d) wait[i] = (unsigned char) (w - 1);
  }
  const unsigned b = __ballot_sync(0xffffffffu, d);
  int base = 0;
  if ((threadIdx.x & 31) == 0 && b) base = atomicAdd(count, __popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (d) due[base + __popc(b & ((1u << (threadIdx.x & 31)) - 1u))] = i;
}

// due[] indexes far[]; the features, means and spreads are in due order.  A
// rejection doubles the element's re-test interval (1, 3, 7, ... 127 steps),
// an acceptance resets it
__global__ void k_accept(const float *__restrict__ spread, const int *__restrict__ far,
                         const int *__restrict__ due, const int *__restrict__ count, int nfar,
                         float thr, unsigned char *__restrict__ skip,
                         unsigned char *__restrict__ wait, unsigned char *__restrict__ streak,
                         unsigned long long *__restrict__ counters) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = count ? *count : nfar;
  bool acc = false;
  if (i < n) {
    const int f = due ? due[i] : i;
    acc = spread[i] <= thr;
    skip[far[f]] = acc ? 1 : 0;
    if (wait) {
      const unsigned char st = acc ? 0 : (unsigned char) min(streak[f] + 1, 7);
      streak[f] = st;
      wait[f] = (unsigned char) ((1u << st) - 1u);
    }
  }
  unsigned b = __ballot_sync(0xffffffffu, acc);
  unsigned v = __ballot_sync(0xffffffffu, i < n);
  if ((threadIdx.x & 31) == 0) {
    if (v) atomicAdd(counters, (unsigned long long) __popc(v));
    if (b) atomicAdd(counters + 1, (unsigned long long) __popc(b));
  }
}

// a grid-stride loop over the device count (most steps test few elements)
__global__ void k_write(const float *__restrict__ mean, const int *__restrict__ far,
                        const int *__restrict__ due, const int *__restrict__ count, int nfar,
                        const unsigned char *__restrict__ skip, double *__restrict__ nodef) {
  const long n = (long) (count ? *count : nfar) * MLP_OUT;
  for (long i = blockIdx.x * (long) blockDim.x + threadIdx.x; i < n;
       i += (long) gridDim.x * blockDim.x) {
    const int r = (int) (i / MLP_OUT), c = (int) (i % MLP_OUT);
    const int e = far[due ? due[r] : r];
    if (skip[e]) nodef[(size_t) MLP_OUT * e + c] = (double) mean[i];
  }
}

__global__ void k_gather_far(const int *__restrict__ far, const int *__restrict__ due,
                             const int *__restrict__ count, int *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < *count) out[i] = far[due[i]];
}

__global__ void k_to_float(const double *__restrict__ src, long n, float *__restrict__ dst) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float) src[i];
}

}  // namespace

void features(const double *nodex, const double *nodex0, const double *erho, const int *elems,
              int n, const int *count, const float *norm, void *xf, cudaStream_t s) {
  if (n <= 0) return;
  k_features<<<nblk(n, 128), 128, 0, s>>>(nodex, nodex0, erho, elems, n, count, norm,
                                          static_cast<__nv_bfloat16 *>(xf));
  check(cudaGetLastError(), "surrogate features");
}

void raw_features(const double *nodex, const double *nodex0, const double *erho, int n, float *x,
                  cudaStream_t s) {
  if (n <= 0) return;
  k_raw_features<<<nblk(n, 128), 128, 0, s>>>(nodex, nodex0, erho, n, x);
  check(cudaGetLastError(), "surrogate raw features");
}

void due(int nfar, const int *far, unsigned char *wait, unsigned char *skip, int *due_list,
         int *count, cudaStream_t s) {
  check(cudaMemsetAsync(count, 0, sizeof(int), s), "surrogate due");
  if (nfar <= 0) return;
  k_due<<<nblk(nfar, 256), 256, 0, s>>>(nfar, far, wait, skip, due_list, count);
  check(cudaGetLastError(), "surrogate due");
}

void accept(const float *spread, const int *far, const int *due_list, const int *count, int nfar,
            float thr, unsigned char *skip, unsigned char *wait, unsigned char *streak,
            unsigned long long *counters, cudaStream_t s) {
  if (nfar <= 0) return;
  k_accept<<<nblk(nfar, 256), 256, 0, s>>>(spread, far, due_list, count, nfar, thr, skip, wait,
                                           streak, counters);
  check(cudaGetLastError(), "surrogate accept");
}

void write_forces(const float *mean, const int *far, const int *due_list, const int *count,
                  int nfar, const unsigned char *skip, double *nodef, cudaStream_t s) {
  if (nfar <= 0) return;
  int dev = 0, nsm = 0;
  check(cudaGetDevice(&dev), "device");
  check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "sm count");
  const int grid = std::min(nblk((long long) nfar * MLP_OUT, 256), 8 * nsm);
  k_write<<<grid, 256, 0, s>>>(mean, far, due_list, count, nfar,
                                                                 skip, nodef);
  check(cudaGetLastError(), "surrogate write");
}

void gather_far(const int *far, const int *due_list, const int *count, int nfar, int *out,
                cudaStream_t s) {
  if (nfar <= 0) return;
  k_gather_far<<<nblk(nfar, 256), 256, 0, s>>>(far, due_list, count, out);
  check(cudaGetLastError(), "surrogate gather_far");
}

void to_float(const double *src, long long n, float *dst, cudaStream_t s) {
  if (n <= 0) return;
  k_to_float<<<nblk(n, 256), 256, 0, s>>>(src, n, dst);
  check(cudaGetLastError(), "to_float");
}

}  // namespace surrogate
}  // namespace cacg
