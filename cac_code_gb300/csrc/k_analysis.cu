// Centro-symmetry of the atoms over the full atom list (Output::centro_atom,
// output.cpp:352-447), built without contraction (-fmad=false) so that every
// value is the reference's bit for bit.
//
// One thread per local atom.  Its in-range neighbors (rsq < cutneighmax^2)
// go to a column-major scratch slice (entry k of thread t at k * chunk + t,
// coalesced across the warp); the 12 nearest are moved to the front by the
// Numerical-Recipes partial quickselect the reference uses (select2 with the
// index array, output.cpp:499-554), the 66 pair vectors R_j + R_k - 2 R_i
// are formed in that order, and the 6 smallest of their squared lengths
// (select, output.cpp:458-497) are summed.  Atoms with fewer than 12
// neighbors get 0.  The partition steps are the published routine's, kept so
// the same neighbors are chosen among equal distances and the sum adds in the
// same order.
#include "internal.h"

namespace cacg {
namespace analysis {

namespace {

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

// k smallest of arr[1..n] (1-based positions, element p at base[(p-1)*str])
// into the first k positions; iarr (optional) follows the same swaps
template <class T>
__device__ void nr_select(int k, int n, T *arr, int *iarr, int str) {
#define A(p) arr[(size_t) ((p) - 1) * str]
#define IA(p) iarr[(size_t) ((p) - 1) * str]
#define SWAP_AT(p, q)                                           \
  {                                                             \
    T t_ = A(p);                                                \
    A(p) = A(q);                                                \
    A(q) = t_;                                                  \
    if (iarr) {                                                 \
      int u_ = IA(p);                                           \
      IA(p) = IA(q);                                            \
      IA(q) = u_;                                               \
    }                                                           \
  }
  int l = 1, ir = n;
  for (;;) {
    if (ir <= l + 1) {
      if (ir == l + 1 && A(ir) < A(l)) SWAP_AT(l, ir);
      return;
    }
    const int mid = (l + ir) >> 1;
    SWAP_AT(mid, l + 1);
    if (A(l) > A(ir)) SWAP_AT(l, ir);
    if (A(l + 1) > A(ir)) SWAP_AT(l + 1, ir);
    if (A(l) > A(l + 1)) SWAP_AT(l, l + 1);
    int i = l + 1, j = ir;
    const T piv = A(l + 1);
    const int ipiv = iarr ? IA(l + 1) : 0;
    for (;;) {
      do i++; while (A(i) < piv);
      do j--; while (A(j) > piv);
      if (j < i) break;
      SWAP_AT(i, j);
    }
    A(l + 1) = A(j);
    A(j) = piv;
    if (iarr) {
      IA(l + 1) = IA(j);
      IA(j) = ipiv;
    }
    if (j >= k) ir = j - 1;
    if (j <= k) l = i;
  }
#undef A
#undef IA
#undef SWAP_AT
}

__global__ void __launch_bounds__(128)
k_centro(const double4 *__restrict__ x, const int *__restrict__ num, const int *__restrict__ list,
         int stride, int i0, int n, double cutsq, double *__restrict__ dsq,
         int *__restrict__ near, int chunk, double *__restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const int i = i0 + t;
  const double4 xi = x[i];
  double *ds = dsq + t;
  int *nr = near + t;
  int m = 0;
  for (int k = 0; k < num[i]; k++) {
    const int j = list[(size_t) k * stride + i];
    const double4 xj = x[j];
    const double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    const double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < cutsq) {
      ds[(size_t) m * chunk] = rsq;
      nr[(size_t) m * chunk] = j;
      m++;
    }
  }
  constexpr int NNN = 12, NHALF = NNN / 2, NPAIRS = NNN * (NNN - 1) / 2;
  if (m < NNN) {
    out[i] = 0.0;
    return;
  }
  nr_select<double>(NNN, m, ds, nr, chunk);
  double pairs[NPAIRS];
  int q = 0;
  for (int a = 0; a < NNN; a++) {
    const double4 xa = x[nr[(size_t) a * chunk]];
    for (int b = a + 1; b < NNN; b++) {
      const double4 xb = x[nr[(size_t) b * chunk]];
      const double dx = xa.x + xb.x - 2.0 * xi.x;
      const double dy = xa.y + xb.y - 2.0 * xi.y;
      const double dz = xa.z + xb.z - 2.0 * xi.z;
      pairs[q++] = dx * dx + dy * dy + dz * dz;
    }
  }
  nr_select<double>(NHALF, NPAIRS, pairs, nullptr, 1);
  double v = 0.0;
  for (int a = 0; a < NHALF; a++) v += pairs[a];
  out[i] = v;
}

}  // namespace

void centro(const double4 *x, const int *num, const int *list, int stride, int i0, int n,
            double cutsq, double *dsq, int *near, int chunk, double *out, cudaStream_t s) {
  if (n <= 0) return;
  k_centro<<<nblk(n, 128), 128, 0, s>>>(x, num, list, stride, i0, n, cutsq, dsq, near, chunk, out);
  check(cudaGetLastError(), "centro");
}

}  // namespace analysis
}  // namespace cacg
