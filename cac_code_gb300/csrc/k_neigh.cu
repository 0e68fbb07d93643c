// Neighbor lists on the device (sm_103a), compiled without FMA contraction so
// every distance predicate is the reference's own arithmetic:
//   * atom list: Neighbor::half_bin_no_newton (neighbor.cpp:546-625), a FULL list,
//     rsq <= cutneighmaxsq, j over stencil bins in stencil order and bin members
//     in index order -- so each row equals the reference's row entry for entry;
//   * element list: Neighbor::element_neighbor (element_neighbor.cpp:11-75) over
//     element centres with the same bins/stencil and rsq <= cut_allsq;
//   * integration-point list: Neighbor::node_neighbor (full_node_neighbor.cpp:19-239),
//     one warp per integration point; lanes test 32 lattice sites of a sub-element
//     at once and a ballot compacts the hits in the reference's site order.
// Lists are column-major (entry k of row i at k*stride + i) so that the force
// kernels, one thread per row, read them coalesced.
#include "internal.h"

namespace cacg {

namespace {

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

__global__ void __launch_bounds__(128)
k_atom_list(const double4 *__restrict__ x, const int *__restrict__ bin,
            const int *__restrict__ bstart, const int *__restrict__ bmem,
            const double4 *__restrict__ bx, const int *__restrict__ stencil, int nstencil,
            int mbins, int nlocal, double cutsq, int maxneigh, int stride,
            int *__restrict__ num, int *__restrict__ list, int *__restrict__ overflow) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const int ib = bin[i];
  int n = 0;
  for (int k = 0; k < nstencil; k++) {
    int b = ib + __ldg(stencil + k);
    if (b < 0 || b >= mbins) continue;
    int p1 = __ldg(bstart + b + 1);
    for (int p = __ldg(bstart + b); p < p1; p++) {
      int j = __ldg(bmem + p);
      if (j == i) continue;
      double4 xj = bx[p];
      double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq <= cutsq) {
        if (n < maxneigh) list[(size_t) n * stride + i] = j;
        n++;
      }
    }
  }
  num[i] = n;
  if (n > maxneigh) atomicMax(overflow, n);
}

__global__ void __launch_bounds__(128)
k_elem_list(const double *__restrict__ ex, const int *__restrict__ bin,
            const int *__restrict__ bstart, const int *__restrict__ bmem,
            const double4 *__restrict__ bx, const int *__restrict__ stencil, int nstencil,
            int mbins, int nlocal, double cutsq, int maxneigh, int stride,
            int *__restrict__ num, int *__restrict__ list, int *__restrict__ overflow) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double xt = ex[3 * i], yt = ex[3 * i + 1], zt = ex[3 * i + 2];
  const int ib = bin[i];
  int n = 0;
  for (int k = 0; k < nstencil; k++) {
    int b = ib + __ldg(stencil + k);
    if (b < 0 || b >= mbins) continue;
    int p1 = __ldg(bstart + b + 1);
    for (int p = __ldg(bstart + b); p < p1; p++) {
      int j = __ldg(bmem + p);
      if (j == i) continue;
      double4 xj = bx[p];
      double dx = xt - xj.x, dy = yt - xj.y, dz = zt - xj.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq <= cutsq) {
        if (n < maxneigh) list[(size_t) n * stride + i] = j;
        n++;
      }
    }
  }
  num[i] = n;
  if (n > maxneigh) atomicMax(overflow, n);
}

// Interpolated lattice sites of every element (Element::interpolate_atom_vec,
// element.cpp:1226-1272): x = sum_k N_k x_k in node order.  One block per element.
__global__ void k_sites(const double *__restrict__ nodex, const int *__restrict__ etype,
                        const int *__restrict__ site_base, ElemTables t,
                        double4 *__restrict__ site_x, float4 *__restrict__ site_h) {
  __shared__ double nx[24];
  const int e = blockIdx.x;
  if (threadIdx.x < 24) nx[threadIdx.x] = nodex[24 * (size_t) e + threadIdx.x];
  __syncthreads();
  const int ty = etype[e];
  const int nint = t.inter_num[ty];
  const double *S0 = t.spa_inter + (size_t) t.inter_off[ty] * NPE;
  const int base = site_base[e];
  for (int nj = threadIdx.x; nj < nint; nj += blockDim.x) {
    const double *S = S0 + (size_t) nj * NPE;
    double a = 0, b = 0, c = 0;
#pragma unroll
    for (int k = 0; k < NPE; k++) {
      double s = S[k];
      a += s * nx[3 * k];
      b += s * nx[3 * k + 1];
      c += s * nx[3 * k + 2];
    }
    site_x[base + nj] = make_double4(a, b, c, 0.0);
    if (site_h) site_h[base + nj] = make_float4((float) a, (float) b, (float) c, 0.f);
  }
}

__global__ void k_split_hi(const double4 *__restrict__ x, float4 *__restrict__ xh, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = x[i];
  xh[i] = make_float4((float) p.x, (float) p.y, (float) p.z, 0.f);
}

// Sub-element centres (full_node_neighbor.cpp:137-143)
__global__ void k_sub_centres(const double *__restrict__ nodex, int nelem, ElemTables t,
                              double4 *__restrict__ subc) {
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nelem * t.nsub) return;
  int e = tid / t.nsub, isub = tid % t.nsub;
  const double *C = t.spa_center_sub + (size_t) isub * NPE;
  const double *nx = nodex + 24 * (size_t) e;
  double a = 0.0, b = 0.0, c = 0.0;
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    a += C[k] * nx[3 * k];
    b += C[k] * nx[3 * k + 1];
    c += C[k] * nx[3 * k + 2];
  }
  subc[tid] = make_double4(a, b, c, 0.0);
}

// One warp per integration point row.
__global__ void __launch_bounds__(128)
k_ip_list(const double *__restrict__ nodex, const double *__restrict__ ex,
          const int *__restrict__ etype, const int *__restrict__ row_elem,
          const int *__restrict__ row_jj, int nrows, const int *__restrict__ enum_,
          const int *__restrict__ elist, int estride, const double4 *__restrict__ subc,
          const double4 *__restrict__ site_x, const int *__restrict__ site_base, ElemTables t,
          double cut_elesq, double cut_subelesq, double cutsq, int maxip, int rowstride,
          int *__restrict__ ipnum, int *__restrict__ ipent, int *__restrict__ overflow) {
  const int r = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= nrows) return;
  const unsigned lt_mask = (1u << lane) - 1u;
  const int e = row_elem[r], jj = row_jj[r], ty = etype[e];
  const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
  const double *nxe = nodex + 24 * (size_t) e;
  double ix = 0, iy = 0, iz = 0;
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    ix += N[k] * nxe[3 * k];
    iy += N[k] * nxe[3 * k + 1];
    iz += N[k] * nxe[3 * k + 2];
  }
  int n = 0;
  const int nsub = t.nsub;
  const int ne = enum_[e];
  // neighbor elements first, then the element itself (self: rsq > 1e-4)
  for (int ll = 0; ll <= ne; ll++) {
    const bool self = ll == ne;
    const int j = self ? e : elist[(size_t) ll * estride + e];
    if (!self) {
      const double cx = ex[3 * j], cy = ex[3 * j + 1], cz = ex[3 * j + 2];
      double npdis = (ix - cx) * (ix - cx) + (iy - cy) * (iy - cy) + (iz - cz) * (iz - cz);
      if (!(npdis <= cut_elesq)) continue;
    }
    // sub-element centre test, lanes over sub-elements
    unsigned submask = 0;
    for (int s0 = 0; s0 < nsub; s0 += 32) {
      int isub = s0 + lane;
      bool pass = false;
      if (isub < nsub) {
        double4 sc = subc[(size_t) j * nsub + isub];
        double nps = (ix - sc.x) * (ix - sc.x) + (iy - sc.y) * (iy - sc.y) +
                     (iz - sc.z) * (iz - sc.z);
        pass = nps <= cut_subelesq;
      }
      unsigned b = __ballot_sync(0xffffffffu, pass);
      // process passing sub-elements of this chunk in order
      while (b) {
        int bit = __ffs(b) - 1;
        b &= b - 1;
        int isub2 = s0 + bit;
        int first = t.sub_first[isub2], cnt = t.sub_first[isub2 + 1] - first;
        const int sb = site_base[j];
        for (int m0 = 0; m0 < cnt; m0 += 32) {
          int mm = m0 + lane;
          bool hit = false;
          int sid = 0;
          if (mm < cnt) {
            int nj = t.list_inter_sub[first + mm];
            sid = sb + nj;
            double4 sx = site_x[sid];
            double dx = sx.x - ix, dy = sx.y - iy, dz = sx.z - iz;
            double rsq = dx * dx + dy * dy + dz * dz;
            hit = self ? (rsq <= cutsq && rsq > 1.0e-4) : (rsq <= cutsq);
          }
          unsigned hb = __ballot_sync(0xffffffffu, hit);
          if (hit) {
            int slot = n + __popc(hb & lt_mask);
            if (slot < maxip) ipent[(size_t) slot * rowstride + r] = sid;
          }
          n += __popc(hb);
        }
      }
      (void) submask;
    }
  }
  if (lane == 0) {
    ipnum[r] = n;
    if (n > maxip) atomicMax(overflow, n);
  }
}

}  // namespace

void launch_atom_list(const double4 *x, const int *bin, const int *bstart, const int *bmem,
                      const double4 *bx, const int *stencil, int nstencil, int mbins,
                      int nlocal, double cutsq, int maxneigh, int stride, int *num, int *list,
                      int *overflow, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_atom_list<<<nblk(nlocal, 128), 128, 0, s>>>(x, bin, bstart, bmem, bx, stencil, nstencil,
                                                 mbins, nlocal, cutsq, maxneigh, stride, num,
                                                 list, overflow);
  check(cudaGetLastError(), "atom_list");
}

void launch_elem_list(const double *ex, const int *bin, const int *bstart, const int *bmem,
                      const double4 *bx, const int *stencil, int nstencil, int mbins,
                      int nlocal, double cutsq, int maxneigh, int stride, int *num, int *list,
                      int *overflow, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_elem_list<<<nblk(nlocal, 128), 128, 0, s>>>(ex, bin, bstart, bmem, bx, stencil, nstencil,
                                                 mbins, nlocal, cutsq, maxneigh, stride, num,
                                                 list, overflow);
  check(cudaGetLastError(), "elem_list");
}

void launch_sites(const double *nodex, const int *etype, const int *site_base, int nelem,
                  ElemTables t, double4 *site_x, float4 *site_h, cudaStream_t s) {
  if (nelem <= 0) return;
  k_sites<<<nelem, 128, 0, s>>>(nodex, etype, site_base, t, site_x, site_h);
  check(cudaGetLastError(), "sites");
}

void launch_split_hi(const double4 *x, float4 *xh, int n, cudaStream_t s) {
  if (n <= 0) return;
  k_split_hi<<<nblk(n, 256), 256, 0, s>>>(x, xh, n);
  check(cudaGetLastError(), "split_hi");
}

void launch_sub_centres(const double *nodex, int nelem, ElemTables t, double4 *subc,
                        cudaStream_t s) {
  if (nelem <= 0) return;
  k_sub_centres<<<nblk((long long) nelem * t.nsub, 128), 128, 0, s>>>(nodex, nelem, t, subc);
  check(cudaGetLastError(), "sub_centres");
}

void launch_ip_list(const double *nodex, const double *ex, const int *etype,
                    const int *row_elem, const int *row_jj, int nrows, const int *enum_,
                    const int *elist, int estride, const double4 *subc, const double4 *site_x,
                    const int *site_base, ElemTables t, double cut_elesq, double cut_subelesq,
                    double cutsq, int maxip, int rowstride, int *ipnum, int *ipent,
                    int *overflow, cudaStream_t s) {
  if (nrows <= 0) return;
  k_ip_list<<<nblk((long long) nrows * 32, 128), 128, 0, s>>>(
      nodex, ex, etype, row_elem, row_jj, nrows, enum_, elist, estride, subc, site_x,
      site_base, t, cut_elesq, cut_subelesq, cutsq, maxip, rowstride, ipnum, ipent, overflow);
  check(cudaGetLastError(), "ip_list");
}

}  // namespace cacg
