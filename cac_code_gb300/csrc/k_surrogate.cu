// Per-step use of the nodal-force surrogate inside the element force pass.
//
// For the elements far from the atomistic region (a list fixed when the
// surrogate is attached), each step:
//   features  -> 24 nodal displacements about their mean, relative to the
//                ideal node positions, then the 8 nodal densities, normalised
//                and rounded to bf16 [n][64] (zero padded) for the GEMMs;
//   accept    -> skip[e] = (ensemble spread <= threshold); counts evaluated
//                and accepted elements on the device;
//   write     -> nodef[e] = ensemble mean for the accepted elements, after the
//                quadrature's nodal gather (which skipped their force rows).
// The reference has no counterpart: it evaluates every element by quadrature.
#include <cuda_bf16.h>

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
                           const float *__restrict__ norm, __nv_bfloat16 *__restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
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

__global__ void k_accept(const float *__restrict__ spread, const int *__restrict__ far, int nfar,
                         float thr, unsigned char *__restrict__ skip,
                         unsigned long long *__restrict__ counters) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool acc = false;
  if (i < nfar) {
    acc = spread[i] <= thr;
    skip[far[i]] = acc ? 1 : 0;
  }
  unsigned b = __ballot_sync(0xffffffffu, acc);
  unsigned v = __ballot_sync(0xffffffffu, i < nfar);
  if ((threadIdx.x & 31) == 0) {
    if (v) atomicAdd(counters, (unsigned long long) __popc(v));
    if (b) atomicAdd(counters + 1, (unsigned long long) __popc(b));
  }
}

__global__ void k_write(const float *__restrict__ mean, const int *__restrict__ far, int nfar,
                        const unsigned char *__restrict__ skip, double *__restrict__ nodef) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= (long) nfar * MLP_OUT) return;
  int r = (int) (i / MLP_OUT), c = (int) (i % MLP_OUT);
  int e = far[r];
  if (skip[e]) nodef[(size_t) MLP_OUT * e + c] = (double) mean[i];
}

__global__ void k_to_float(const double *__restrict__ src, long n, float *__restrict__ dst) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i < n) dst[i] = (float) src[i];
}

}  // namespace

void features(const double *nodex, const double *nodex0, const double *erho, const int *elems,
              int n, const float *norm, void *xf, cudaStream_t s) {
  if (n <= 0) return;
  k_features<<<nblk(n, 128), 128, 0, s>>>(nodex, nodex0, erho, elems, n, norm,
                                          static_cast<__nv_bfloat16 *>(xf));
  check(cudaGetLastError(), "surrogate features");
}

void raw_features(const double *nodex, const double *nodex0, const double *erho, int n, float *x,
                  cudaStream_t s) {
  if (n <= 0) return;
  k_raw_features<<<nblk(n, 128), 128, 0, s>>>(nodex, nodex0, erho, n, x);
  check(cudaGetLastError(), "surrogate raw features");
}

void accept(const float *spread, const int *far, int nfar, float thr, unsigned char *skip,
            unsigned long long *counters, cudaStream_t s) {
  if (nfar <= 0) return;
  k_accept<<<nblk(nfar, 256), 256, 0, s>>>(spread, far, nfar, thr, skip, counters);
  check(cudaGetLastError(), "surrogate accept");
}

void write_forces(const float *mean, const int *far, int nfar, const unsigned char *skip,
                  double *nodef, cudaStream_t s) {
  if (nfar <= 0) return;
  k_write<<<nblk((long long) nfar * MLP_OUT, 256), 256, 0, s>>>(mean, far, nfar, skip, nodef);
  check(cudaGetLastError(), "surrogate write");
}

void to_float(const double *src, long long n, float *dst, cudaStream_t s) {
  if (n <= 0) return;
  k_to_float<<<nblk(n, 256), 256, 0, s>>>(src, n, dst);
  check(cudaGetLastError(), "to_float");
}

}  // namespace surrogate
}  // namespace cacg
