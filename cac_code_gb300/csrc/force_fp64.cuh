// FP64 pair kernels for atoms and element integration points (sm_103a).
//
// Included by two translation units: k_force_exact.cu is compiled with
// -fmad=false, so each expression is the reference's own sequence of IEEE
// multiplies and adds and the forces are bit-identical to the CPU code;
// k_force_fma.cu is compiled with contraction on (the fast FP64 mode).  The
// arithmetic follows, line by line:
//   PairLJCut::compute   pair_lj_cut.cpp:227-288
//   PairLJCut::ecompute  pair_lj_cut.cpp:295-442
//   PairEAM::compute     pair_eam.cpp:584-746
//   PairEAM::ecompute    pair_eam.cpp:761-1141
// One thread per atom / integration point accumulates its row in list order.
// Element-site positions come from the per-step site table (k_sites), which
// holds exactly the sum the reference recomputes for every list entry.
#pragma once
#include "internal.h"

namespace cacg {
namespace FP64NS {  // defined per translation unit

struct LJTab {
  double lj1[(MAXT + 1) * (MAXT + 1)];
  double lj2[(MAXT + 1) * (MAXT + 1)];
  double cutsq[(MAXT + 1) * (MAXT + 1)];
};

__global__ void __launch_bounds__(128)
k_lj_atoms(const double4 *__restrict__ x, const int *__restrict__ type,
           const int *__restrict__ num, const int *__restrict__ list, int stride, int nlocal,
           const LJTab *__restrict__ tab, double *__restrict__ f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const int it = type[i];
  const int n = num[i];
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    double4 xj = x[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    int jt = type[j];
    int ij = it * (MAXT + 1) + jt;
    if (rsq < tab->cutsq[ij]) {
      double r2inv = 1.0 / rsq;
      double r6inv = r2inv * r2inv * r2inv;
      double forcelj = r6inv * (tab->lj1[ij] * r6inv - tab->lj2[ij]);
      double fpair = forcelj * r2inv;
      fx += dx * fpair;
      fy += dy * fpair;
      fz += dz * fpair;
    }
  }
  f[3 * i] = fx;
  f[3 * i + 1] = fy;
  f[3 * i + 2] = fz;
}

__device__ __forceinline__ double spline_value(const double *__restrict__ c, double p) {
  return ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
}

__device__ __forceinline__ double spline_deriv(const double *__restrict__ c, double p) {
  return (c[0] * p + c[1]) * p + c[2];
}

// r-table index: p = r*rdr + 1, m = min(int(p), nr-1), p = min(p - m, 1)
__device__ __forceinline__ int rindex(double r, const EamTables &e, double &p) {
  p = r * e.rdr + 1.0;
  int m = (int) p;
  m = m < e.nr - 1 ? m : e.nr - 1;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  return m;
}

// rho-table index with m clamped to [1, nrho-1] (pair_eam.cpp:672-676)
__device__ __forceinline__ int rhoindex(double rho, const EamTables &e, double &p) {
  p = rho * e.rdrho + 1.0;
  int m = (int) p;
  m = m < e.nrho - 1 ? m : e.nrho - 1;
  m = 1 > m ? 1 : m;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  return m;
}

__global__ void __launch_bounds__(128)
k_eam_rho_atoms(const double4 *__restrict__ x, const int *__restrict__ num,
                const int *__restrict__ list, int stride, int nlocal, EamTables e,
                double *__restrict__ rho, double *__restrict__ fp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const int n = num[i];
  double r = 0.0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    double4 xj = x[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < e.cutforcesq) {
      double p;
      int m = rindex(sqrt(rsq), e, p);
      r += spline_value(e.rhor + 7 * m, p);
    }
  }
  rho[i] = r;
  double p;
  int m = rhoindex(r, e, p);
  fp[i] = spline_deriv(e.frho + 7 * m, p);
}

__global__ void __launch_bounds__(128)
k_eam_force_atoms(const double4 *__restrict__ x, const int *__restrict__ num,
                  const int *__restrict__ list, int stride, int nlocal, EamTables e,
                  const double *__restrict__ fp, double *__restrict__ f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const double fpi = fp[i];
  const int n = num[i];
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    double4 xj = x[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < e.cutforcesq) {
      double r = sqrt(rsq);
      double p;
      int m = rindex(r, e, p);
      double rhoip = spline_deriv(e.rhor + 7 * m, p);
      double rhojp = rhoip;  // same table for every type pair (single funcfl file)
      const double *z = e.z2r + 7 * m;
      double z2p = spline_deriv(z, p);
      double z2 = spline_value(z, p);
      double recip = 1.0 / r;
      double phi = z2 * recip;
      double phip = z2p * recip - phi * recip;
      double psip = fpi * rhojp + __ldg(fp + j) * rhoip + phip;
      double fpair = -psip * recip;
      fx += dx * fpair;
      fy += dy * fpair;
      fz += dz * fpair;
    }
  }
  f[3 * i] = fx;
  f[3 * i + 1] = fy;
  f[3 * i + 2] = fz;
}

// integration-point position: sum_k N_k x_k (pair_lj_cut.cpp:363-367)
__device__ __forceinline__ void ip_position(const double *__restrict__ N,
                                            const double *__restrict__ nx, double &ix,
                                            double &iy, double &iz) {
  ix = 0;
  iy = 0;
  iz = 0;
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    ix += N[k] * nx[3 * k];
    iy += N[k] * nx[3 * k + 1];
    iz += N[k] * nx[3 * k + 2];
  }
}

__global__ void __launch_bounds__(128)
k_lj_ip(const double *__restrict__ nodex, const int *__restrict__ etype,
        const int *__restrict__ row_elem, const int *__restrict__ row_jj, int nrows,
        const int *__restrict__ ipnum, const int *__restrict__ ipent, int rowstride,
        const double4 *__restrict__ site_x, ElemTables t, double lj1, double lj2, double cutsq,
        double *__restrict__ fip) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int e = row_elem[r], jj = row_jj[r], ty = etype[e];
  const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
  double ix, iy, iz;
  ip_position(N, nodex + 24 * (size_t) e, ix, iy, iz);
  double fx = 0, fy = 0, fz = 0;
  const int n = ipnum[r];
  for (int k = 0; k < n; k++) {
    int sid = __ldg(ipent + (size_t) k * rowstride + r);
    double4 s = site_x[sid];
    double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < cutsq) {
      double r2inv = 1.0 / rsq;
      double r6inv = r2inv * r2inv * r2inv;
      double forcelj = r6inv * (lj1 * r6inv - lj2);
      double fpair = forcelj * r2inv;
      fx += dx * fpair;
      fy += dy * fpair;
      fz += dz * fpair;
    }
  }
  fip[3 * r] = fx;
  fip[3 * r + 1] = fy;
  fip[3 * r + 2] = fz;
}

// Nodal densities erho[e][q] from the row of the integration point at node q
// (pair_eam.cpp:927-986).  One thread per (element, node).
__global__ void __launch_bounds__(128)
k_eam_erho(const double *__restrict__ nodex, const int *__restrict__ etype,
           const int *__restrict__ row_first, int nlocal_e, const int *__restrict__ ipnum,
           const int *__restrict__ ipent, int rowstride, const double4 *__restrict__ site_x,
           ElemTables t, EamTables eam, double *__restrict__ erho) {
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nlocal_e * NPE) return;
  int e = tid / NPE, q = tid % NPE;
  int ty = etype[e];
  int r = row_first[e] + t.node_list[ty * NPE + q];
  const double *nx = nodex + 24 * (size_t) e + 3 * q;
  const double ix = nx[0], iy = nx[1], iz = nx[2];
  double acc = 0.0;
  const int n = ipnum[r];
  for (int k = 0; k < n; k++) {
    int sid = __ldg(ipent + (size_t) k * rowstride + r);
    double4 s = site_x[sid];
    double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < eam.cutforcesq) {
      double p;
      int m = rindex(sqrt(rsq), eam, p);
      acc += spline_value(eam.rhor + 7 * m, p);
    }
  }
  erho[tid] = acc;
}

// F'(rho) at every interpolated site, rho = sum_k N_k erho_k (pair_eam.cpp:1060-1076)
__global__ void k_eam_site_fp(const double *__restrict__ erho, const int *__restrict__ etype,
                              const int *__restrict__ site_base, ElemTables t, EamTables eam,
                              double *__restrict__ site_fp) {
  __shared__ double er[NPE];
  const int e = blockIdx.x;
  if (threadIdx.x < NPE) er[threadIdx.x] = erho[NPE * (size_t) e + threadIdx.x];
  __syncthreads();
  const int ty = etype[e];
  const int nint = t.inter_num[ty];
  const double *S0 = t.spa_inter + (size_t) t.inter_off[ty] * NPE;
  const int base = site_base[e];
  for (int nj = threadIdx.x; nj < nint; nj += blockDim.x) {
    const double *S = S0 + (size_t) nj * NPE;
    double rho = 0;
#pragma unroll
    for (int k = 0; k < NPE; k++) rho += S[k] * er[k];
    double p;
    int m = rhoindex(rho, eam, p);
    site_fp[base + nj] = spline_deriv(eam.frho + 7 * m, p);
  }
}

__global__ void __launch_bounds__(128)
k_eam_ip(const double *__restrict__ nodex, const double *__restrict__ erho,
         const int *__restrict__ etype, const int *__restrict__ row_elem,
         const int *__restrict__ row_jj, int nrows, const int *__restrict__ ipnum,
         const int *__restrict__ ipent, int rowstride, const double4 *__restrict__ site_x,
         const double *__restrict__ site_fp, ElemTables t, EamTables eam,
         double *__restrict__ fip) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int e = row_elem[r], jj = row_jj[r], ty = etype[e];
  const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
  const double *nx = nodex + 24 * (size_t) e;
  const double *er = erho + NPE * (size_t) e;
  double ix = 0, iy = 0, iz = 0, rhoi = 0;
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    ix += N[k] * nx[3 * k];
    iy += N[k] * nx[3 * k + 1];
    iz += N[k] * nx[3 * k + 2];
    rhoi += N[k] * er[k];
  }
  double p;
  int m = rhoindex(rhoi, eam, p);
  const double fpi = spline_deriv(eam.frho + 7 * m, p);
  double fx = 0, fy = 0, fz = 0;
  const int n = ipnum[r];
  for (int k = 0; k < n; k++) {
    int sid = __ldg(ipent + (size_t) k * rowstride + r);
    double4 s = site_x[sid];
    double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < eam.cutforcesq) {
      double fpj = __ldg(site_fp + sid);
      double rr = sqrt(rsq);
      double pr;
      int mr = rindex(rr, eam, pr);
      double rhoip = spline_deriv(eam.rhor + 7 * mr, pr);
      const double *z = eam.z2r + 7 * mr;
      double z2p = spline_deriv(z, pr);
      double z2 = spline_value(z, pr);
      double recip = 1.0 / rr;
      double phi = z2 * recip;
      double phip = z2p * recip - phi * recip;
      double psip = (fpi + fpj) * rhoip + phip;
      double fpair = -psip * recip;
      fx += dx * fpair;
      fy += dy * fpair;
      fz += dz * fpair;
    }
  }
  fip[3 * r] = fx;
  fip[3 * r + 1] = fy;
  fip[3 * r + 2] = fz;
}

// nodef[e][q] = sum over integration points jj of (w_jj N_jj,q) F_jj, in jj
// order, as the reference's += sequence into a cleared array
// (pair_lj_cut.cpp:424-428).  One thread per (element, node, component).
__global__ void k_gather_nodef(const double *__restrict__ fip, const int *__restrict__ etype,
                               const int *__restrict__ row_first, int nlocal_e, ElemTables t,
                               double *__restrict__ nodef) {
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nlocal_e * 24) return;
  int e = tid / 24, rem = tid % 24, q = rem / 3, c = rem % 3;
  int ty = etype[e];
  int nint = t.numint[ty];
  int r0 = row_first[e];
  const double *N = t.spa_int + (size_t) t.int_off[ty] * NPE;
  const double *w = t.weight + t.int_off[ty];
  double acc = 0.0;
  for (int jj = 0; jj < nint; jj++) acc += w[jj] * N[jj * NPE + q] * fip[3 * (r0 + jj) + c];
  nodef[tid] = acc;
}

}  // namespace FP64NS (per translation unit)
}  // namespace cacg
