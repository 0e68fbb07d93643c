// Mixed-precision pair kernels (sm_103a): FP32 pair terms, FP64 accumulation.
//
// Same formulas as the FP64 kernels (PairLJCut::compute/ecompute,
// pair_lj_cut.cpp:227-442; PairEAM::compute/ecompute, pair_eam.cpp:584-1141),
// evaluated in FP32 where the spec allows it:
//  * atom coordinates are double-single pairs (hi = float(x), lo = float(x-hi)),
//    so a pair vector (hi_i-hi_j)+(lo_i-lo_j) is good to ~1e-6 A at any box size;
//  * element sites are interpolated in FP32 from node offsets to the element
//    centre, the centre-to-centre offset taken in FP64 once per neighbor element;
//  * r, 1/r and the rho(r), r*phi(r) splines are FP32, the spline coefficients
//    FP32 in shared memory, loaded once by each resident block (persistent grid);
//  * the cutoff test is made in FP32 and re-made in FP64 inside a thin guard
//    band, so the set of interacting pairs is exactly the FP64 set;
//  * per-site densities and forces are summed in FP32 over chunks of 8 pairs and
//    the chunks in FP64; F'(rho) is evaluated from the FP64 table in FP64.
#include "internal.h"

namespace cacg {
namespace mixed {

namespace {

constexpr int CHUNK = 8;

struct RhoVal {  // rho(r) spline value coefficients c3..c6 per knot
  float4 c;
};

__device__ __forceinline__ int findex(float r, float rdr, int nr, float &p) {
  p = r * rdr + 1.0f;
  int m = (int) p;
  m = m < nr - 1 ? m : nr - 1;
  p -= (float) m;
  p = fminf(p, 1.0f);
  return m;
}

__device__ __forceinline__ double fprime64(double rho, const double *__restrict__ frho,
                                           int nrho, double rdrho) {
  double p = rho * rdrho + 1.0;
  int m = (int) p;
  m = m < nrho - 1 ? m : nrho - 1;
  m = 1 > m ? 1 : m;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  const double *c = frho + 7 * m;
  return (c[0] * p + c[1]) * p + c[2];
}

// exact FP64 cutoff decision for pairs whose FP32 rsq falls in the guard band
__device__ __forceinline__ bool inside64(const double4 &a, const double4 &b, double cutsq) {
  double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return dx * dx + dy * dy + dz * dz < cutsq;
}

__global__ void k_split_hilo(const double4 *__restrict__ x, float4 *__restrict__ xh,
                             float4 *__restrict__ xl, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = x[i];
  float hx = (float) p.x, hy = (float) p.y, hz = (float) p.z;
  xh[i] = make_float4(hx, hy, hz, 0.f);
  xl[i] = make_float4((float) (p.x - hx), (float) (p.y - hy), (float) (p.z - hz), 0.f);
}

// node offsets from the element centre, FP32 (element-relative coordinates)
__global__ void k_elem_rel(const double *__restrict__ nodex, const double *__restrict__ ex,
                           int n, float *__restrict__ u) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 24) return;
  int e = t / 24, c = t % 3;
  u[t] = (float) (nodex[t] - ex[3 * e + c]);
}

__device__ __forceinline__ void pair_vec(const float4 &hi, const float4 &li, const float4 &hj,
                                         const float4 &lj, float &dx, float &dy, float &dz) {
  dx = (hi.x - hj.x) + (li.x - lj.x);
  dy = (hi.y - hj.y) + (li.y - lj.y);
  dz = (hi.z - hj.z) + (li.z - lj.z);
}

struct AtomArgs {
  const double4 *x;
  const float4 *xh, *xl;
  const int *num, *list;
  int stride, nlocal;
  float cutsq_f, band_lo, band_hi;  // [band_lo, band_hi]: decide in FP64
  double cutsq;
};

__global__ void __launch_bounds__(256)
k_eam_rho_atoms(AtomArgs a, const float4 *__restrict__ rhor_val, int nr, float rdr,
                const double *__restrict__ frho, int nrho, double rdrho,
                double *__restrict__ rho, double *__restrict__ fp) {
  extern __shared__ float4 s_val[];
  for (int m = threadIdx.x; m <= nr; m += blockDim.x) s_val[m] = rhor_val[m];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nlocal; i += gridDim.x * blockDim.x) {
    const float4 hi = a.xh[i], li = a.xl[i];
    const int n = a.num[i];
    double acc = 0.0;
    float part = 0.f;
    for (int k = 0; k < n; k++) {
      int j = __ldg(a.list + (size_t) k * a.stride + i);
      float dx, dy, dz;
      pair_vec(hi, li, __ldg(a.xh + j), __ldg(a.xl + j), dx, dy, dz);
      float rsq = dx * dx + dy * dy + dz * dz;
      bool in = rsq < a.cutsq_f;
      if (rsq >= a.band_lo && rsq <= a.band_hi) in = inside64(a.x[i], a.x[j], a.cutsq);
      if (in) {
        float p;
        int m = findex(sqrtf(rsq), rdr, nr, p);
        float4 c = s_val[m];
        part += ((c.x * p + c.y) * p + c.z) * p + c.w;
      }
      if ((k & (CHUNK - 1)) == CHUNK - 1) {
        acc += (double) part;
        part = 0.f;
      }
    }
    acc += (double) part;
    rho[i] = acc;
    fp[i] = fprime64(acc, frho, nrho, rdrho);
  }
}

// force table per knot: rho'(r) c0..c2 (x,y,z of f0), r*phi c0..c6 (w of f0, f1, f2.xy)
__global__ void __launch_bounds__(256)
k_eam_force_atoms(AtomArgs a, const float4 *__restrict__ ftab, int nr, float rdr,
                  const double *__restrict__ fp, double *__restrict__ f) {
  extern __shared__ float4 s_tab[];  // 3 float4 per knot
  for (int m = threadIdx.x; m < 3 * (nr + 1); m += blockDim.x) s_tab[m] = ftab[m];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nlocal; i += gridDim.x * blockDim.x) {
    const float4 hi = a.xh[i], li = a.xl[i];
    const float fpi = (float) fp[i];
    const int n = a.num[i];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    float px = 0.f, py = 0.f, pz = 0.f;
    for (int k = 0; k < n; k++) {
      int j = __ldg(a.list + (size_t) k * a.stride + i);
      float dx, dy, dz;
      pair_vec(hi, li, __ldg(a.xh + j), __ldg(a.xl + j), dx, dy, dz);
      float rsq = dx * dx + dy * dy + dz * dz;
      bool in = rsq < a.cutsq_f;
      if (rsq >= a.band_lo && rsq <= a.band_hi) in = inside64(a.x[i], a.x[j], a.cutsq);
      if (in) {
        float recip = rsqrtf(rsq);
        float r = rsq * recip;
        float p;
        int m = findex(r, rdr, nr, p);
        float4 t0 = s_tab[3 * m], t1 = s_tab[3 * m + 1], t2 = s_tab[3 * m + 2];
        float rhoip = (t0.x * p + t0.y) * p + t0.z;
        float z2p = (t0.w * p + t1.x) * p + t1.y;
        float z2 = ((t1.z * p + t1.w) * p + t2.x) * p + t2.y;
        float phi = z2 * recip;
        float phip = z2p * recip - phi * recip;
        float psip = (fpi + (float) __ldg(fp + j)) * rhoip + phip;
        float fpair = -psip * recip;
        px += dx * fpair;
        py += dy * fpair;
        pz += dz * fpair;
      }
      if ((k & (CHUNK - 1)) == CHUNK - 1) {
        fx += (double) px;
        fy += (double) py;
        fz += (double) pz;
        px = py = pz = 0.f;
      }
    }
    f[3 * i] = fx + (double) px;
    f[3 * i + 1] = fy + (double) py;
    f[3 * i + 2] = fz + (double) pz;
  }
}

// band_lo/band_hi are relative factors here: a pair with rsq in
// [band_lo, band_hi] * cutsq(type pair) is decided in FP64
__global__ void __launch_bounds__(256)
k_lj_atoms(AtomArgs a, const int *__restrict__ type, const float *__restrict__ lj1,
           const float *__restrict__ lj2, const float *__restrict__ cutsq_t,
           const double *__restrict__ cutsq64, double *__restrict__ f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nlocal; i += gridDim.x * blockDim.x) {
    const float4 hi = a.xh[i], li = a.xl[i];
    const int it = type[i];
    const int n = a.num[i];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    float px = 0.f, py = 0.f, pz = 0.f;
    for (int k = 0; k < n; k++) {
      int j = __ldg(a.list + (size_t) k * a.stride + i);
      float dx, dy, dz;
      pair_vec(hi, li, __ldg(a.xh + j), __ldg(a.xl + j), dx, dy, dz);
      float rsq = dx * dx + dy * dy + dz * dz;
      int ij = it * (MAXT + 1) + type[j];
      float cs = cutsq_t[ij];
      bool in = rsq < cs;
      if (rsq >= a.band_lo * cs && rsq <= a.band_hi * cs) in = inside64(a.x[i], a.x[j], cutsq64[ij]);
      if (in) {
        float r2inv = __frcp_rn(rsq);
        float r6inv = r2inv * r2inv * r2inv;
        float fpair = r6inv * (lj1[ij] * r6inv - lj2[ij]) * r2inv;
        px += dx * fpair;
        py += dy * fpair;
        pz += dz * fpair;
      }
      if ((k & (CHUNK - 1)) == CHUNK - 1) {
        fx += (double) px;
        fy += (double) py;
        fz += (double) pz;
        px = py = pz = 0.f;
      }
    }
    f[3 * i] = fx + (double) px;
    f[3 * i + 1] = fy + (double) py;
    f[3 * i + 2] = fz + (double) pz;
  }
}

// ---------------------------------------------------------------- elements

struct ElemArgs {
  const double *nodex, *ex, *erho;
  const float *u;           // [nall][24] node offsets from the centre
  const int *etype, *row_elem, *row_jj, *row_first, *ipnum, *ipent, *site_base;
  int nrows, rowstride, nall, nlocal_e;
  const double *spa_int, *weight;
  const int *int_off, *node_list;
  const float *shape;       // [ninter][8] FP32 site shape functions (type 1)
  int ninter;
  float cutsq_f, band_lo, band_hi;
  double cutsq;
};

// locate the element owning site id `sid` (site_base ascending), starting from
// the current range; entries of a row come grouped by element
__device__ __forceinline__ int site_elem(const int *__restrict__ sb, int nall, int sid) {
  int lo = 0, hi = nall;  // sb[lo] <= sid < sb[hi]
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (__ldg(sb + mid) <= sid) lo = mid;
    else hi = mid;
  }
  return lo;
}

__device__ __forceinline__ void site_rel(const float *__restrict__ S, const float *__restrict__ u,
                                         float &x, float &y, float &z) {
  x = 0.f;
  y = 0.f;
  z = 0.f;
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    x += S[k] * u[3 * k];
    y += S[k] * u[3 * k + 1];
    z += S[k] * u[3 * k + 2];
  }
}

// FP64 position of a site, for the guard-band re-test
__device__ __forceinline__ void site64(const double *__restrict__ S, const double *__restrict__ nx,
                                       double &x, double &y, double &z) {
  x = 0;
  y = 0;
  z = 0;
  for (int k = 0; k < NPE; k++) {
    x += S[k] * nx[3 * k];
    y += S[k] * nx[3 * k + 1];
    z += S[k] * nx[3 * k + 2];
  }
}

// One thread per integration point (row); node rows of weight 0 are skipped
// unless `node_rows` (EAM nodal density pass), which visits only node rows.
template <bool EAM, bool DENSITY>
__global__ void __launch_bounds__(256)
k_ip(ElemArgs a, const double *__restrict__ spa_inter64, const float4 *__restrict__ tab,
     int nr, float rdr, const double *__restrict__ frho, int nrho, double rdrho,
     float lj1, float lj2, double *__restrict__ out) {
  extern __shared__ float4 smem[];
  float *s_shape = (float *) smem;                       // ninter*8 floats
  float4 *s_tab = smem + 2 * a.ninter;                   // EAM table after the shapes
  for (int k = threadIdx.x; k < a.ninter * NPE; k += blockDim.x) s_shape[k] = a.shape[k];
  const int ntab = EAM ? (DENSITY ? (nr + 1) : 3 * (nr + 1)) : 0;
  for (int m = threadIdx.x; m < ntab; m += blockDim.x) s_tab[m] = tab[m];
  __syncthreads();
  const int nitems = DENSITY ? a.nlocal_e * NPE : a.nrows;
  for (int it = blockIdx.x * blockDim.x + threadIdx.x; it < nitems; it += gridDim.x * blockDim.x) {
    int r, e, ty;
    const double *N64;
    if (DENSITY) {
      e = it / NPE;
      int q = it % NPE;
      ty = a.etype[e];
      int jj = a.node_list[ty * NPE + q];
      r = a.row_first[e] + jj;
      N64 = a.spa_int + ((size_t) a.int_off[ty] + jj) * NPE;
    } else {
      r = it;
      e = a.row_elem[r];
      ty = a.etype[e];
      int jj = a.row_jj[r];
      if (a.weight[a.int_off[ty] + jj] == 0.0) {
        out[3 * r] = out[3 * r + 1] = out[3 * r + 2] = 0.0;
        continue;
      }
      N64 = a.spa_int + ((size_t) a.int_off[ty] + jj) * NPE;
    }
    const float *ue = a.u + 24 * (size_t) e;
    float ipx = 0.f, ipy = 0.f, ipz = 0.f;
    double fpi = 0.0;
    double rhoi = 0.0;
#pragma unroll
    for (int k = 0; k < NPE; k++) {
      float nk = (float) N64[k];
      ipx += nk * ue[3 * k];
      ipy += nk * ue[3 * k + 1];
      ipz += nk * ue[3 * k + 2];
      if (EAM && !DENSITY) rhoi += N64[k] * a.erho[NPE * (size_t) e + k];
    }
    if (EAM && !DENSITY) fpi = fprime64(rhoi, frho, nrho, rdrho);
    const double cex = a.ex[3 * e], cey = a.ex[3 * e + 1], cez = a.ex[3 * e + 2];
    int j = -1, sb0 = 0, sb1 = 0;
    float ox = 0.f, oy = 0.f, oz = 0.f;
    float uj[24];
    float erj[NPE];
    double acc = 0.0, fx = 0.0, fy = 0.0, fz = 0.f;
    float part = 0.f, px = 0.f, py = 0.f, pz = 0.f;
    const int n = a.ipnum[r];
    for (int k = 0; k < n; k++) {
      int sid = __ldg(a.ipent + (size_t) k * a.rowstride + r);
      if (sid < sb0 || sid >= sb1) {
        j = site_elem(a.site_base, a.nall, sid);
        sb0 = __ldg(a.site_base + j);
        sb1 = __ldg(a.site_base + j + 1);
        ox = (float) (cex - a.ex[3 * j]);
        oy = (float) (cey - a.ex[3 * j + 1]);
        oz = (float) (cez - a.ex[3 * j + 2]);
        for (int q = 0; q < 24; q++) uj[q] = a.u[24 * (size_t) j + q];
        if (EAM && !DENSITY)
          for (int q = 0; q < NPE; q++) erj[q] = (float) a.erho[NPE * (size_t) j + q];
      }
      const int nj = sid - sb0;
      const float *S = s_shape + nj * NPE;
      float sx, sy, sz;
      site_rel(S, uj, sx, sy, sz);
      float dx = ox + (ipx - sx), dy = oy + (ipy - sy), dz = oz + (ipz - sz);
      float rsq = dx * dx + dy * dy + dz * dz;
      bool in = rsq < a.cutsq_f;
      if (rsq >= a.band_lo && rsq <= a.band_hi) {
        // FP64 re-test from the nodes, exactly as the FP64 path positions them
        double ix, iy, iz, jx, jy, jz;
        site64(N64, a.nodex + 24 * (size_t) e, ix, iy, iz);
        site64(spa_inter64 + (size_t) nj * NPE, a.nodex + 24 * (size_t) j, jx, jy, jz);
        double ddx = ix - jx, ddy = iy - jy, ddz = iz - jz;
        if (DENSITY) {
          const double *nxq = a.nodex + 24 * (size_t) e;
          int q = it % NPE;
          ddx = nxq[3 * q] - jx;
          ddy = nxq[3 * q + 1] - jy;
          ddz = nxq[3 * q + 2] - jz;
        }
        in = ddx * ddx + ddy * ddy + ddz * ddz < a.cutsq;
      }
      if (in) {
        if (EAM) {
          float recip = rsqrtf(rsq);
          float rr = rsq * recip;
          float p;
          int m = findex(rr, rdr, nr, p);
          if (DENSITY) {
            float4 c = s_tab[m];
            part += ((c.x * p + c.y) * p + c.z) * p + c.w;
          } else {
            double rhoj = 0.0;
            float rj = 0.f;
#pragma unroll
            for (int q = 0; q < NPE; q++) rj += S[q] * erj[q];
            rhoj = (double) rj;
            float fpj = (float) fprime64(rhoj, frho, nrho, rdrho);
            float4 t0 = s_tab[3 * m], t1 = s_tab[3 * m + 1], t2 = s_tab[3 * m + 2];
            float rhoip = (t0.x * p + t0.y) * p + t0.z;
            float z2p = (t0.w * p + t1.x) * p + t1.y;
            float z2 = ((t1.z * p + t1.w) * p + t2.x) * p + t2.y;
            float phi = z2 * recip;
            float phip = z2p * recip - phi * recip;
            float psip = ((float) fpi + fpj) * rhoip + phip;
            float fpair = -psip * recip;
            px += dx * fpair;
            py += dy * fpair;
            pz += dz * fpair;
          }
        } else {
          float r2inv = __frcp_rn(rsq);
          float r6inv = r2inv * r2inv * r2inv;
          float fpair = r6inv * (lj1 * r6inv - lj2) * r2inv;
          px += dx * fpair;
          py += dy * fpair;
          pz += dz * fpair;
        }
      }
      if ((k & (CHUNK - 1)) == CHUNK - 1) {
        acc += (double) part;
        fx += (double) px;
        fy += (double) py;
        fz += (double) pz;
        part = px = py = pz = 0.f;
      }
    }
    if (DENSITY) {
      out[it] = acc + (double) part;
    } else {
      out[3 * r] = fx + (double) px;
      out[3 * r + 1] = fy + (double) py;
      out[3 * r + 2] = fz + (double) pz;
    }
  }
}

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

int persistent_grid(const void *kernel, int threads, size_t smem, long long work) {
  int dev = 0, nsm = 0, occ = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem);
  if (occ < 1) occ = 1;
  long long need = (work + threads - 1) / threads;
  long long g = (long long) nsm * occ;
  return (int) (need < g ? (need > 0 ? need : 1) : g);
}

}  // namespace

void split_hilo(const double4 *x, float4 *xh, float4 *xl, int n, cudaStream_t s) {
  if (n <= 0) return;
  k_split_hilo<<<nblk(n, 256), 256, 0, s>>>(x, xh, xl, n);
  check(cudaGetLastError(), "split_hilo");
}

void elem_rel(const double *nodex, const double *ex, int n, float *u, cudaStream_t s) {
  if (n <= 0) return;
  k_elem_rel<<<nblk((long long) n * 24, 256), 256, 0, s>>>(nodex, ex, n, u);
  check(cudaGetLastError(), "elem_rel");
}

void eam_rho_atoms(const MixedAtoms &m, const float4 *rhor_val, const EamTables &e,
                   double *rho, double *fp, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xh, m.xl, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq};
  size_t smem = sizeof(float4) * (e.nr + 1);
  int g = persistent_grid((const void *) k_eam_rho_atoms, 256, smem, m.nlocal);
  k_eam_rho_atoms<<<g, 256, smem, s>>>(a, rhor_val, e.nr, (float) e.rdr, e.frho, e.nrho,
                                       e.rdrho, rho, fp);
  check(cudaGetLastError(), "eam_rho_atoms_mixed");
}

void eam_force_atoms(const MixedAtoms &m, const float4 *ftab, const EamTables &e,
                     const double *fp, double *f, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xh, m.xl, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq};
  size_t smem = sizeof(float4) * 3 * (e.nr + 1);
  int g = persistent_grid((const void *) k_eam_force_atoms, 256, smem, m.nlocal);
  k_eam_force_atoms<<<g, 256, smem, s>>>(a, ftab, e.nr, (float) e.rdr, fp, f);
  check(cudaGetLastError(), "eam_force_atoms_mixed");
}

void lj_atoms(const MixedAtoms &m, const int *type, const float *lj1, const float *lj2,
              const float *cutsq_t, const double *cutsq64, double *f, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xh, m.xl, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq};
  int g = persistent_grid((const void *) k_lj_atoms, 256, 0, m.nlocal);
  k_lj_atoms<<<g, 256, 0, s>>>(a, type, lj1, lj2, cutsq_t, cutsq64, f);
  check(cudaGetLastError(), "lj_atoms_mixed");
}

void ip_pass(const MixedElems &m, int pass, const double *spa_inter64, const float4 *tab,
             const EamTables &e, float lj1, float lj2, double *out, cudaStream_t s) {
  ElemArgs a{m.nodex, m.ex, m.erho, m.u, m.etype, m.row_elem, m.row_jj, m.row_first,
             m.ipnum, m.ipent, m.site_base, m.nrows, m.rowstride, m.nall, m.nlocal_e,
             m.spa_int, m.weight, m.int_off, m.node_list, m.shape, m.ninter, m.cutsq_f,
             m.band_lo, m.band_hi, m.cutsq};
  size_t smem_shape = sizeof(float4) * 2 * (size_t) m.ninter;
  long long work;
  if (pass == 0) {  // LJ forces
    work = m.nrows;
    size_t smem = smem_shape;
    int g = persistent_grid((const void *) k_ip<false, false>, 256, smem, work);
    k_ip<false, false><<<g, 256, smem, s>>>(a, spa_inter64, tab, 0, 0.f, nullptr, 0, 0.0,
                                           lj1, lj2, out);
  } else if (pass == 1) {  // EAM nodal densities
    work = (long long) m.nlocal_e * NPE;
    size_t smem = smem_shape + sizeof(float4) * (e.nr + 1);
    int g = persistent_grid((const void *) k_ip<true, true>, 256, smem, work);
    k_ip<true, true><<<g, 256, smem, s>>>(a, spa_inter64, tab, e.nr, (float) e.rdr, e.frho,
                                         e.nrho, e.rdrho, 0.f, 0.f, out);
  } else {  // EAM forces
    work = m.nrows;
    size_t smem = smem_shape + sizeof(float4) * 3 * (e.nr + 1);
    int g = persistent_grid((const void *) k_ip<true, false>, 256, smem, work);
    k_ip<true, false><<<g, 256, smem, s>>>(a, spa_inter64, tab, e.nr, (float) e.rdr, e.frho,
                                          e.nrho, e.rdrho, 0.f, 0.f, out);
  }
  check(cudaGetLastError(), "ip_pass_mixed");
}

}  // namespace mixed
}  // namespace cacg
