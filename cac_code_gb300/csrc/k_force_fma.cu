// Fast FP64 pair kernels (sm_103a), compiled with contraction.
//
// Same arithmetic as force_fp64.cuh (the reference's formulas, file:line cited
// there) with three changes that cut FP64 instructions, the binding resource
// on GB300 (FP64 ~1/60 of the FP32 rate):
//  * an FP32 pre-test of each list entry against cutoff + a guard band proven
//    from the float rounding of the coordinates -- an entry it rejects is
//    outside the cutoff in exact arithmetic too, so it contributes nothing;
//  * 1/sqrt(r^2) and 1/r^2 from the FP32 hardware estimate refined by two FP64
//    Newton-Raphson steps (y <- y(3 - x y^2)/2 and y <- y(2 - x y)), which
//    reach full double precision instead of IEEE sqrt and divide;
//  * integration points of weight 0 (the EAM node rows) get no force pass:
//    their contribution to the nodal gather is 0 * N * F = 0.
// Forces agree with the exact mode to ~1e-15 relative (tested at 1e-12).
#include "internal.h"

namespace cacg {
namespace fp64_fma {

namespace {

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

struct LJTab {
  double lj1[(MAXT + 1) * (MAXT + 1)];
  double lj2[(MAXT + 1) * (MAXT + 1)];
  double cutsq[(MAXT + 1) * (MAXT + 1)];
};

__device__ __forceinline__ double rsqrt_nr(double x) {
  double y = (double) rsqrtf((float) x);
  const double hx = 0.5 * x;
  y = y * fma(-hx * y, y, 1.5);
  y = y * fma(-hx * y, y, 1.5);
  return y;
}

__device__ __forceinline__ double rcp_nr(double x) {
  double y = (double) __frcp_rn((float) x);
  double e = fma(-x, y, 1.0);
  y = fma(y, e, y);
  e = fma(-x, y, 1.0);
  return fma(y, e, y);
}

__device__ __forceinline__ double spline_value(const double *__restrict__ c, double p) {
  return ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
}

__device__ __forceinline__ double spline_deriv(const double *__restrict__ c, double p) {
  return (c[0] * p + c[1]) * p + c[2];
}

__device__ __forceinline__ int rindex(double r, const EamTables &e, double &p) {
  p = r * e.rdr + 1.0;
  int m = (int) p;
  m = m < e.nr - 1 ? m : e.nr - 1;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  return m;
}

__device__ __forceinline__ int rhoindex(double rho, const EamTables &e, double &p) {
  p = rho * e.rdrho + 1.0;
  int m = (int) p;
  m = m < e.nrho - 1 ? m : e.nrho - 1;
  m = 1 > m ? 1 : m;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  return m;
}

__device__ __forceinline__ float rsq_f(float4 a, float4 b) {
  float dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return dx * dx + dy * dy + dz * dz;
}

__global__ void __launch_bounds__(128)
k_lj_atoms(const double4 *__restrict__ x, const float4 *__restrict__ xh,
           const int *__restrict__ type, const int *__restrict__ num,
           const int *__restrict__ list, int stride, int nlocal, const LJTab *__restrict__ tab,
           float cut_pass, double *__restrict__ f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const float4 hi = xh[i];
  const int it = type[i];
  const int n = num[i];
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    double4 xj = x[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    int ij = it * (MAXT + 1) + type[j];
    if (rsq < tab->cutsq[ij]) {
      double r2inv = rcp_nr(rsq);
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

__global__ void __launch_bounds__(128)
k_eam_rho_atoms(const double4 *__restrict__ x, const float4 *__restrict__ xh,
                const int *__restrict__ num, const int *__restrict__ list, int stride,
                int nlocal, EamTables e, float cut_pass, double *__restrict__ rho,
                double *__restrict__ fp) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const float4 hi = xh[i];
  const int n = num[i];
  double r = 0.0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    double4 xj = x[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < e.cutforcesq) {
      double p;
      int m = rindex(rsq * rsqrt_nr(rsq), e, p);
      r += spline_value(e.rhor + 7 * m, p);
    }
  }
  rho[i] = r;
  double p;
  int m = rhoindex(r, e, p);
  fp[i] = spline_deriv(e.frho + 7 * m, p);
}

__global__ void __launch_bounds__(128)
k_eam_force_atoms(const double4 *__restrict__ x, const float4 *__restrict__ xh,
                  const int *__restrict__ num, const int *__restrict__ list, int stride,
                  int nlocal, EamTables e, float cut_pass, const double *__restrict__ fp,
                  double *__restrict__ f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const double4 xi = x[i];
  const float4 hi = xh[i];
  const double fpi = fp[i];
  const int n = num[i];
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    double4 xj = x[j];
    double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < e.cutforcesq) {
      double recip = rsqrt_nr(rsq);
      double r = rsq * recip;
      double p;
      int m = rindex(r, e, p);
      double rhoip = spline_deriv(e.rhor + 7 * m, p);
      const double *z = e.z2r + 7 * m;
      double z2p = spline_deriv(z, p);
      double z2 = spline_value(z, p);
      double phi = z2 * recip;
      double phip = z2p * recip - phi * recip;
      double psip = fpi * rhoip + __ldg(fp + j) * rhoip + phip;
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

// Positions are interpolated without contraction (explicit round-to-nearest
// multiply and add), exactly as the exact mode: element coordinates reach
// |x| ~ 1e3, and a fused rounding there would move a site by ~1e-13, which the
// stiff pair forces amplify beyond the 1e-12 FP64 tolerance.
__device__ __forceinline__ void ip_position(const double *__restrict__ N,
                                            const double *__restrict__ nx, double &ix,
                                            double &iy, double &iz) {
  ix = 0;
  iy = 0;
  iz = 0;
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    ix = __dadd_rn(ix, __dmul_rn(N[k], nx[3 * k]));
    iy = __dadd_rn(iy, __dmul_rn(N[k], nx[3 * k + 1]));
    iz = __dadd_rn(iz, __dmul_rn(N[k], nx[3 * k + 2]));
  }
}

__global__ void __launch_bounds__(128)
k_lj_ip(const double *__restrict__ nodex, const int *__restrict__ etype,
        const int *__restrict__ row_elem, const int *__restrict__ row_jj, int nrows,
        const int *__restrict__ ipnum, const int *__restrict__ ipent, int rowstride,
        const double4 *__restrict__ site_x, const float4 *__restrict__ site_h, ElemTables t,
        double lj1, double lj2, double cutsq, float cut_pass, const int *__restrict__ rows,
        double *__restrict__ fip) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  if (rows) r = rows[r];
  const int e = row_elem[r], jj = row_jj[r], ty = etype[e];
  double fx = 0, fy = 0, fz = 0;
  if (t.weight[t.int_off[ty] + jj] != 0.0) {
    const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
    double ix, iy, iz;
    ip_position(N, nodex + 24 * (size_t) e, ix, iy, iz);
    const float4 hi = make_float4((float) ix, (float) iy, (float) iz, 0.f);
    const int n = ipnum[r];
    for (int k = 0; k < n; k++) {
      int sid = __ldg(ipent + (size_t) k * rowstride + r);
      double4 s = site_x[sid];
      double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < cutsq) {
        double r2inv = rcp_nr(rsq);
        double r6inv = r2inv * r2inv * r2inv;
        double forcelj = r6inv * (lj1 * r6inv - lj2);
        double fpair = forcelj * r2inv;
        fx += dx * fpair;
        fy += dy * fpair;
        fz += dz * fpair;
      }
    }
  }
  fip[3 * r] = fx;
  fip[3 * r + 1] = fy;
  fip[3 * r + 2] = fz;
}

__global__ void __launch_bounds__(128)
k_eam_erho(const double *__restrict__ nodex, const int *__restrict__ etype,
           const int *__restrict__ row_first, int nlocal_e, const int *__restrict__ ipnum,
           const int *__restrict__ ipent, int rowstride, const double4 *__restrict__ site_x,
           const float4 *__restrict__ site_h, ElemTables t, EamTables eam, float cut_pass,
           double *__restrict__ erho) {
  int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nlocal_e * NPE) return;
  int e = tid / NPE, q = tid % NPE;
  int ty = etype[e];
  int r = row_first[e] + t.node_list[ty * NPE + q];
  const double *nx = nodex + 24 * (size_t) e + 3 * q;
  const double ix = nx[0], iy = nx[1], iz = nx[2];
  const float4 hi = make_float4((float) ix, (float) iy, (float) iz, 0.f);
  double acc = 0.0;
  const int n = ipnum[r];
  for (int k = 0; k < n; k++) {
    int sid = __ldg(ipent + (size_t) k * rowstride + r);
    double4 s = site_x[sid];
    double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
    double rsq = dx * dx + dy * dy + dz * dz;
    if (rsq < eam.cutforcesq) {
      double p;
      int m = rindex(rsq * rsqrt_nr(rsq), eam, p);
      acc += spline_value(eam.rhor + 7 * m, p);
    }
  }
  erho[tid] = acc;
}

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
         const float4 *__restrict__ site_h, const double *__restrict__ site_fp, ElemTables t,
         EamTables eam, float cut_pass, const int *__restrict__ rows, double *__restrict__ fip) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  if (rows) r = rows[r];
  const int e = row_elem[r], jj = row_jj[r], ty = etype[e];
  double fx = 0, fy = 0, fz = 0;
  if (t.weight[t.int_off[ty] + jj] != 0.0) {
    const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
    const double *nx = nodex + 24 * (size_t) e;
    const double *er = erho + NPE * (size_t) e;
    double ix, iy, iz, rhoi = 0;
    ip_position(N, nx, ix, iy, iz);
#pragma unroll
    for (int k = 0; k < NPE; k++) rhoi += N[k] * er[k];
    double p;
    int m = rhoindex(rhoi, eam, p);
    const double fpi = spline_deriv(eam.frho + 7 * m, p);
    const float4 hi = make_float4((float) ix, (float) iy, (float) iz, 0.f);
    const int n = ipnum[r];
    for (int k = 0; k < n; k++) {
      int sid = __ldg(ipent + (size_t) k * rowstride + r);
      double4 s = site_x[sid];
      double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < eam.cutforcesq) {
        double fpj = __ldg(site_fp + sid);
        double recip = rsqrt_nr(rsq);
        double rr = rsq * recip;
        double pr;
        int mr = rindex(rr, eam, pr);
        double rhoip = spline_deriv(eam.rhor + 7 * mr, pr);
        const double *z = eam.z2r + 7 * mr;
        double z2p = spline_deriv(z, pr);
        double z2 = spline_value(z, pr);
        double phi = z2 * recip;
        double phip = z2p * recip - phi * recip;
        double psip = (fpi + fpj) * rhoip + phip;
        double fpair = -psip * recip;
        fx += dx * fpair;
        fy += dy * fpair;
        fz += dz * fpair;
      }
    }
  }
  fip[3 * r] = fx;
  fip[3 * r + 1] = fy;
  fip[3 * r + 2] = fz;
}

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

// Per-step short lists: the entries of a row whose FP32 distance passes the
// guarded cutoff test (any entry inside the cutoff in exact arithmetic passes),
// in list order.  Both EAM passes and the element passes then iterate mostly
// interacting pairs, so the FP64 branch seldom diverges inside a warp.
__global__ void __launch_bounds__(128)
k_filter_atoms(const float4 *__restrict__ xh, const int *__restrict__ num,
               const int *__restrict__ list, int stride, int nlocal, float cut_pass,
               int *__restrict__ snum, int *__restrict__ slist) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlocal) return;
  const float4 hi = xh[i];
  const int n = num[i];
  int m = 0;
  for (int k = 0; k < n; k++) {
    int j = __ldg(list + (size_t) k * stride + i);
    if (rsq_f(hi, __ldg(xh + j)) <= cut_pass) slist[(size_t) m++ * stride + i] = j;
  }
  snum[i] = m;
}

// rows: all rows (mode 0), rows of nonzero weight or node rows (mode 1)
__global__ void __launch_bounds__(128)
k_filter_rows(const double *__restrict__ nodex, const int *__restrict__ etype,
              const int *__restrict__ row_elem, const int *__restrict__ row_jj, int nrows,
              const int *__restrict__ ipnum, const int *__restrict__ ipent, int rowstride,
              const float4 *__restrict__ site_h, ElemTables t, float cut_pass, int only_needed,
              int *__restrict__ snum, int *__restrict__ sent, const int *__restrict__ row_list,
              const unsigned char *__restrict__ skip) {
  int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nrows) return;
  const int r = row_list ? row_list[it] : it;
  const int e = row_elem[r], jj = row_jj[r], ty = etype[e];
  // rows of nonzero weight of an element whose forces come from elsewhere
  if (skip && skip[e] && t.weight[t.int_off[ty] + jj] != 0.0) {
    snum[r] = 0;
    return;
  }
  if (only_needed && t.weight[t.int_off[ty] + jj] == 0.0) {
    bool node = false;
    for (int q = 0; q < NPE; q++) node = node || t.node_list[ty * NPE + q] == jj;
    if (!node) {
      snum[r] = 0;
      return;
    }
  }
  const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
  double ix, iy, iz;
  ip_position(N, nodex + 24 * (size_t) e, ix, iy, iz);
  const float4 hi = make_float4((float) ix, (float) iy, (float) iz, 0.f);
  const int n = ipnum[r];
  int m = 0;
  for (int k = 0; k < n; k++) {
    int sid = __ldg(ipent + (size_t) k * rowstride + r);
    if (rsq_f(hi, __ldg(site_h + sid)) <= cut_pass) sent[(size_t) m++ * rowstride + r] = sid;
  }
  snum[r] = m;
}

// Sites referenced by any integration-point list (built once per rebuild):
// flag every entry's site, then the host compacts the flags into `need` and the
// owning element of each needed site into `need_elem`.
__global__ void k_mark_sites(const int *__restrict__ ipnum, const int *__restrict__ ipent,
                             int nrows, int rowstride, int *__restrict__ flag) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int n = ipnum[r];
  for (int k = 0; k < n; k++) flag[__ldg(ipent + (size_t) k * rowstride + r)] = 1;
}

__global__ void k_need_compact(const int *__restrict__ flag, const int *__restrict__ pos,
                               int nsites, const int *__restrict__ site_base, int nall,
                               int *__restrict__ need, int *__restrict__ need_elem) {
  int sid = blockIdx.x * blockDim.x + threadIdx.x;
  if (sid >= nsites || !flag[sid]) return;
  int lo = 0, hi = nall;  // site_base[lo] <= sid < site_base[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (site_base[mid] <= sid) lo = mid;
    else hi = mid;
  }
  need[pos[sid]] = sid;
  need_elem[pos[sid]] = lo;
}

// positions of the needed sites, contraction-free (both FP64 modes), one thread
// per site; consecutive needed sites mostly share their element's nodes in L1
__global__ void k_sites_needed(const double *__restrict__ nodex, const int *__restrict__ etype,
                               const int *__restrict__ site_base, const int *__restrict__ need,
                               const int *__restrict__ need_elem, int nneed, ElemTables t,
                               double4 *__restrict__ site_x, float4 *__restrict__ site_h) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nneed) return;
  const int sid = need[q], j = need_elem[q];
  const int nj = sid - site_base[j];
  const double *S = t.spa_inter + ((size_t) t.inter_off[etype[j]] + nj) * NPE;
  double a, b, c;
  ip_position(S, nodex + 24 * (size_t) j, a, b, c);
  site_x[sid] = make_double4(a, b, c, 0.0);
  site_h[sid] = make_float4((float) a, (float) b, (float) c, 0.f);
}

// F'(rho) of the needed sites (pair_eam.cpp:1060-1076)
__global__ void k_site_fp_needed(const double *__restrict__ erho, const int *__restrict__ etype,
                                 const int *__restrict__ site_base, const int *__restrict__ need,
                                 const int *__restrict__ need_elem, int nneed, ElemTables t,
                                 EamTables eam, double *__restrict__ site_fp) {
  int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nneed) return;
  const int sid = need[q], j = need_elem[q];
  const int nj = sid - site_base[j];
  const double *S = t.spa_inter + ((size_t) t.inter_off[etype[j]] + nj) * NPE;
  const double *er = erho + NPE * (size_t) j;
  double rho = 0;
#pragma unroll
  for (int k = 0; k < NPE; k++) rho += S[k] * er[k];
  double p;
  int m = rhoindex(rho, eam, p);
  site_fp[sid] = spline_deriv(eam.frho + 7 * m, p);
}

// site positions with fused multiply-adds (the exact mode uses k_sites in
// k_neigh.cu, built without contraction); also writes the float copy
__global__ void k_sites_fma(const double *__restrict__ nodex, const int *__restrict__ etype,
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
    double a, b, c;
    ip_position(S, nx, a, b, c);
    site_x[base + nj] = make_double4(a, b, c, 0.0);
    site_h[base + nj] = make_float4((float) a, (float) b, (float) c, 0.f);
  }
}

}  // namespace

void filter_atoms(const float4 *xh, const int *num, const int *list, int stride, int nlocal,
                  float cut_pass, int *snum, int *slist, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_filter_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(xh, num, list, stride, nlocal, cut_pass,
                                                  snum, slist);
  check(cudaGetLastError(), "filter_atoms");
}

void filter_rows(const double *nodex, const int *etype, const int *row_elem, const int *row_jj,
                 int nrows, const int *ipnum, const int *ipent, int rowstride,
                 const float4 *site_h, ElemTables t, float cut_pass, int only_needed, int *snum,
                 int *sent, cudaStream_t s, const int *row_list, const unsigned char *skip) {
  if (nrows <= 0) return;
  k_filter_rows<<<nblk(nrows, 128), 128, 0, s>>>(nodex, etype, row_elem, row_jj, nrows, ipnum,
                                                ipent, rowstride, site_h, t, cut_pass,
                                                only_needed, snum, sent, row_list, skip);
  check(cudaGetLastError(), "filter_rows");
}

void mark_sites(const int *ipnum, const int *ipent, int nrows, int rowstride, int *flag,
                cudaStream_t s) {
  if (nrows <= 0) return;
  k_mark_sites<<<nblk(nrows, 128), 128, 0, s>>>(ipnum, ipent, nrows, rowstride, flag);
  check(cudaGetLastError(), "mark_sites");
}

void need_compact(const int *flag, const int *pos, int nsites, const int *site_base, int nall,
                  int *need, int *need_elem, cudaStream_t s) {
  if (nsites <= 0) return;
  k_need_compact<<<nblk(nsites, 256), 256, 0, s>>>(flag, pos, nsites, site_base, nall, need,
                                                  need_elem);
  check(cudaGetLastError(), "need_compact");
}

void sites_needed(const double *nodex, const int *etype, const int *site_base, const int *need,
                  const int *need_elem, int nneed, ElemTables t, double4 *site_x, float4 *site_h,
                  cudaStream_t s) {
  if (nneed <= 0) return;
  k_sites_needed<<<nblk(nneed, 128), 128, 0, s>>>(nodex, etype, site_base, need, need_elem,
                                                 nneed, t, site_x, site_h);
  check(cudaGetLastError(), "sites_needed");
}

void site_fp_needed(const double *erho, const int *etype, const int *site_base, const int *need,
                    const int *need_elem, int nneed, ElemTables t, EamTables e, double *site_fp,
                    cudaStream_t s) {
  if (nneed <= 0) return;
  k_site_fp_needed<<<nblk(nneed, 128), 128, 0, s>>>(erho, etype, site_base, need, need_elem,
                                                   nneed, t, e, site_fp);
  check(cudaGetLastError(), "site_fp_needed");
}

void sites(const double *nodex, const int *etype, const int *site_base, int nelem, ElemTables t,
           double4 *site_x, float4 *site_h, cudaStream_t s) {
  if (nelem <= 0) return;
  k_sites_fma<<<nelem, 128, 0, s>>>(nodex, etype, site_base, t, site_x, site_h);
  check(cudaGetLastError(), "sites_fma");
}

void lj_atoms(const double4 *x, const float4 *xh, const int *type, const int *num,
              const int *list, int stride, int nlocal, const void *tab, float cut_pass,
              double *f, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_lj_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(x, xh, type, num, list, stride, nlocal,
                                              (const LJTab *) tab, cut_pass, f);
  check(cudaGetLastError(), "lj_atoms_fma");
}

void eam_rho_atoms(const double4 *x, const float4 *xh, const int *num, const int *list,
                   int stride, int nlocal, EamTables e, float cut_pass, double *rho,
                   double *fp, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_eam_rho_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(x, xh, num, list, stride, nlocal, e,
                                                   cut_pass, rho, fp);
  check(cudaGetLastError(), "eam_rho_atoms_fma");
}

void eam_force_atoms(const double4 *x, const float4 *xh, const int *num, const int *list,
                     int stride, int nlocal, EamTables e, float cut_pass, const double *fp,
                     double *f, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_eam_force_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(x, xh, num, list, stride, nlocal, e,
                                                     cut_pass, fp, f);
  check(cudaGetLastError(), "eam_force_atoms_fma");
}

void lj_ip(const double *nodex, const int *etype, const int *row_elem, const int *row_jj,
           int nrows, const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,
           const float4 *site_h, ElemTables t, double lj1, double lj2, double cutsq,
           float cut_pass, const int *rows, double *fip, cudaStream_t s) {
  if (nrows <= 0) return;
  k_lj_ip<<<nblk(nrows, 128), 128, 0, s>>>(nodex, etype, row_elem, row_jj, nrows, ipnum, ipent,
                                          rowstride, site_x, site_h, t, lj1, lj2, cutsq,
                                          cut_pass, rows, fip);
  check(cudaGetLastError(), "lj_ip_fma");
}

void eam_erho(const double *nodex, const int *etype, const int *row_first, int nlocal_e,
              const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,
              const float4 *site_h, ElemTables t, EamTables e, float cut_pass, double *erho,
              cudaStream_t s) {
  if (nlocal_e <= 0) return;
  k_eam_erho<<<nblk((long long) nlocal_e * NPE, 128), 128, 0, s>>>(
      nodex, etype, row_first, nlocal_e, ipnum, ipent, rowstride, site_x, site_h, t, e,
      cut_pass, erho);
  check(cudaGetLastError(), "eam_erho_fma");
}

void eam_site_fp(const double *erho, const int *etype, const int *site_base, int nelem,
                 ElemTables t, EamTables e, double *site_fp, cudaStream_t s) {
  if (nelem <= 0) return;
  k_eam_site_fp<<<nelem, 128, 0, s>>>(erho, etype, site_base, t, e, site_fp);
  check(cudaGetLastError(), "eam_site_fp_fma");
}

void eam_ip(const double *nodex, const double *erho, const int *etype, const int *row_elem,
            const int *row_jj, int nrows, const int *ipnum, const int *ipent, int rowstride,
            const double4 *site_x, const float4 *site_h, const double *site_fp, ElemTables t,
            EamTables e, float cut_pass, const int *rows, double *fip, cudaStream_t s) {
  if (nrows <= 0) return;
  k_eam_ip<<<nblk(nrows, 128), 128, 0, s>>>(nodex, erho, etype, row_elem, row_jj, nrows, ipnum,
                                           ipent, rowstride, site_x, site_h, site_fp, t, e,
                                           cut_pass, rows, fip);
  check(cudaGetLastError(), "eam_ip_fma");
}

void gather_nodef(const double *fip, const int *etype, const int *row_first, int nlocal_e,
                  ElemTables t, double *nodef, cudaStream_t s) {
  if (nlocal_e <= 0) return;
  k_gather_nodef<<<nblk((long long) nlocal_e * 24, 128), 128, 0, s>>>(fip, etype, row_first,
                                                                     nlocal_e, t, nodef);
  check(cudaGetLastError(), "gather_nodef_fma");
}

}  // namespace fp64_fma
}  // namespace cacg
