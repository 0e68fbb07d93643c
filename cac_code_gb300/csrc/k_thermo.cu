// Energy, virial and kinetic energy (sm_103a, FP64).
//
// The reference computes none of these (Pair::compute ignores eflag/vflag,
// pair_lj_cut.cpp:227-288 and pair_eam.cpp:584-746; compute pe/temp/pressure
// are stubs, compute_pe.cpp:16-49).  The formulas are the standard ones of the
// same pair styles, written against the reference's own tables:
//   LJ   e_ij = r^-6 (lj3 r^-6 - lj4),  lj3 = 4 eps sigma^12, lj4 = 4 eps sigma^6
//   EAM  e_i  = F(rho_i) + 1/2 sum_j phi(r_ij),  phi = z2r(r)/r,  F from the frho
//        spline value ((c3 p + c4) p + c5) p + c6 (pair_eam.cpp:552-580 layout)
// With full lists every pair is visited from both ends, so pair energies and
// the pair virial r_a f_b carry a factor 1/2.  Element integration points
// contribute weight * (their site energy and virial).  Each block writes its
// partial sums; the host adds the partials in block order (deterministic).
#include "internal.h"

namespace cacg {
namespace thermo {

namespace {

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }
constexpr int TB = 256;
constexpr int NQ = 7;  // energy, vxx, vyy, vzz, vxy, vxz, vyz

__device__ __forceinline__ void block_reduce_store(double (&q)[NQ], double *__restrict__ part) {
  __shared__ double sh[NQ][TB / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NQ; k++) {
    double v = q[k];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) sh[k][wid] = v;
  }
  __syncthreads();
  if (threadIdx.x < NQ) {
    double v = 0.0;
    for (int w = 0; w < TB / 32; w++) v += sh[threadIdx.x][w];
    part[(size_t) blockIdx.x * NQ + threadIdx.x] = v;
  }
}

__device__ __forceinline__ void rsplines(const EamTables &e, double r, double &phi, double &phip,
                                         double &rhop) {
  double p = r * e.rdr + 1.0;
  int m = (int) p;
  m = m < e.nr - 1 ? m : e.nr - 1;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  const double *z = e.z2r + 7 * m;
  const double *c = e.rhor + 7 * m;
  double z2 = ((z[3] * p + z[4]) * p + z[5]) * p + z[6];
  double z2p = (z[0] * p + z[1]) * p + z[2];
  rhop = (c[0] * p + c[1]) * p + c[2];
  double recip = 1.0 / r;
  phi = z2 * recip;
  phip = z2p * recip - phi * recip;
}

__device__ __forceinline__ double embed(const EamTables &e, double rho, double &fprime) {
  double p = rho * e.rdrho + 1.0;
  int m = (int) p;
  m = m < e.nrho - 1 ? m : e.nrho - 1;
  m = 1 > m ? 1 : m;
  p -= m;
  p = p < 1.0 ? p : 1.0;
  const double *c = e.frho + 7 * m;
  fprime = (c[0] * p + c[1]) * p + c[2];
  return ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
}

__device__ __forceinline__ void add_virial(double (&q)[NQ], double w, double dx, double dy,
                                           double dz, double fpair) {
  q[1] += w * dx * dx * fpair;
  q[2] += w * dy * dy * fpair;
  q[3] += w * dz * dz * fpair;
  q[4] += w * dx * dy * fpair;
  q[5] += w * dx * dz * fpair;
  q[6] += w * dy * dz * fpair;
}

struct LJ {
  const double *lj1, *lj2, *lj3, *lj4, *cutsq;  // [(MAXT+1)^2]
};

__global__ void __launch_bounds__(TB)
k_atoms_lj(const double4 *__restrict__ x, const int *__restrict__ type,
           const int *__restrict__ num, const int *__restrict__ list, int stride, int n, LJ t,
           double *__restrict__ part) {
  double q[NQ] = {0, 0, 0, 0, 0, 0, 0};
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double4 xi = x[i];
    const int it = type[i];
    for (int k = 0; k < num[i]; k++) {
      int j = list[(size_t) k * stride + i];
      double4 xj = x[j];
      double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      int ij = it * (MAXT + 1) + type[j];
      if (rsq < t.cutsq[ij]) {
        double r2inv = 1.0 / rsq;
        double r6inv = r2inv * r2inv * r2inv;
        double fpair = r6inv * (t.lj1[ij] * r6inv - t.lj2[ij]) * r2inv;
        q[0] += 0.5 * r6inv * (t.lj3[ij] * r6inv - t.lj4[ij]);
        add_virial(q, 0.5, dx, dy, dz, fpair);
      }
    }
  }
  block_reduce_store(q, part);
}

__global__ void __launch_bounds__(TB)
k_atoms_eam(const double4 *__restrict__ x, const int *__restrict__ num,
            const int *__restrict__ list, int stride, int n, EamTables e,
            const double *__restrict__ rho, const double *__restrict__ fp,
            double *__restrict__ part) {
  double q[NQ] = {0, 0, 0, 0, 0, 0, 0};
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double4 xi = x[i];
    double fpi;
    q[0] = embed(e, rho[i], fpi);
    for (int k = 0; k < num[i]; k++) {
      int j = list[(size_t) k * stride + i];
      double4 xj = x[j];
      double dx = xi.x - xj.x, dy = xi.y - xj.y, dz = xi.z - xj.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < e.cutforcesq) {
        double r = sqrt(rsq), phi, phip, rhop;
        rsplines(e, r, phi, phip, rhop);
        q[0] += 0.5 * phi;
        double fpair = -(fpi * rhop + fp[j] * rhop + phip) / r;
        add_virial(q, 0.5, dx, dy, dz, fpair);
      }
    }
  }
  block_reduce_store(q, part);
}

// integration points of nonzero weight; EAM uses erho and per-site F'(rho)
__global__ void __launch_bounds__(TB)
k_ip(const double *__restrict__ nodex, const double *__restrict__ erho,
     const int *__restrict__ etype, const int *__restrict__ row_elem,
     const int *__restrict__ row_jj, const int *__restrict__ rows, int nforce,
     const int *__restrict__ ipnum, const int *__restrict__ ipent, int rowstride,
     const double4 *__restrict__ site_x, const double *__restrict__ site_fp, ElemTables t,
     EamTables e, int eam, double lj1, double lj2, double lj3, double lj4, double ljcutsq,
     double *__restrict__ part) {
  double q[NQ] = {0, 0, 0, 0, 0, 0, 0};
  int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it < nforce) {
    const int r = rows[it];
    const int el = row_elem[r], jj = row_jj[r], ty = etype[el];
    const double w = t.weight[t.int_off[ty] + jj];
    const double *N = t.spa_int + ((size_t) t.int_off[ty] + jj) * NPE;
    const double *nx = nodex + 24 * (size_t) el;
    double ix = 0, iy = 0, iz = 0, rhoi = 0;
    for (int k = 0; k < NPE; k++) {
      ix = __dadd_rn(ix, __dmul_rn(N[k], nx[3 * k]));
      iy = __dadd_rn(iy, __dmul_rn(N[k], nx[3 * k + 1]));
      iz = __dadd_rn(iz, __dmul_rn(N[k], nx[3 * k + 2]));
      if (eam) rhoi += N[k] * erho[NPE * (size_t) el + k];
    }
    double fpi = 0.0, ei = 0.0;
    if (eam) ei = embed(e, rhoi, fpi);
    for (int k = 0; k < ipnum[r]; k++) {
      int sid = ipent[(size_t) k * rowstride + r];
      double4 s = site_x[sid];
      double dx = ix - s.x, dy = iy - s.y, dz = iz - s.z;
      double rsq = dx * dx + dy * dy + dz * dz;
      if (eam) {
        if (rsq < e.cutforcesq) {
          double rr = sqrt(rsq), phi, phip, rhop;
          rsplines(e, rr, phi, phip, rhop);
          ei += 0.5 * phi;
          double fpair = -((fpi + site_fp[sid]) * rhop + phip) / rr;
          add_virial(q, 0.5 * w, dx, dy, dz, fpair);
        }
      } else if (rsq < ljcutsq) {
        double r2inv = 1.0 / rsq;
        double r6inv = r2inv * r2inv * r2inv;
        double fpair = r6inv * (lj1 * r6inv - lj2) * r2inv;
        ei += 0.5 * r6inv * (lj3 * r6inv - lj4);
        add_virial(q, 0.5 * w, dx, dy, dz, fpair);
      }
    }
    q[0] = w * ei;
  }
  block_reduce_store(q, part);
}

// 1/2 m v^2 per atom (mass by type) or per node (M_e / 8 by element type)
__global__ void __launch_bounds__(TB)
k_kinetic(const double *__restrict__ v, const int *__restrict__ type,
          const double *__restrict__ mass, int n, int per_item, double scale,
          double *__restrict__ part) {
  double q[NQ] = {0, 0, 0, 0, 0, 0, 0};
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    double m = mass[type[i / per_item]] * scale;
    double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
    q[0] = 0.5 * m * (vx * vx + vy * vy + vz * vz);
    q[1] = m * vx * vx;
    q[2] = m * vy * vy;
    q[3] = m * vz * vz;
    q[4] = m * vx * vy;
    q[5] = m * vx * vz;
    q[6] = m * vy * vz;
  }
  block_reduce_store(q, part);
}

}  // namespace

int partial_blocks(long long n) { return nblk(n > 0 ? n : 1, TB); }

void atoms_lj(const double4 *x, const int *type, const int *num, const int *list, int stride,
              int n, const double *lj /*[5][(MAXT+1)^2]*/, double *part, cudaStream_t s) {
  const int T = (MAXT + 1) * (MAXT + 1);
  LJ t{lj, lj + T, lj + 2 * T, lj + 3 * T, lj + 4 * T};
  k_atoms_lj<<<partial_blocks(n), TB, 0, s>>>(x, type, num, list, stride, n, t, part);
  check(cudaGetLastError(), "thermo_atoms_lj");
}

void atoms_eam(const double4 *x, const int *num, const int *list, int stride, int n,
               EamTables e, const double *rho, const double *fp, double *part, cudaStream_t s) {
  k_atoms_eam<<<partial_blocks(n), TB, 0, s>>>(x, num, list, stride, n, e, rho, fp, part);
  check(cudaGetLastError(), "thermo_atoms_eam");
}

void ip(const double *nodex, const double *erho, const int *etype, const int *row_elem,
        const int *row_jj, const int *rows, int nforce, const int *ipnum, const int *ipent,
        int rowstride, const double4 *site_x, const double *site_fp, ElemTables t, EamTables e,
        int eam, double lj1, double lj2, double lj3, double lj4, double ljcutsq, double *part,
        cudaStream_t s) {
  k_ip<<<partial_blocks(nforce), TB, 0, s>>>(nodex, erho, etype, row_elem, row_jj, rows, nforce,
                                             ipnum, ipent, rowstride, site_x, site_fp, t, e,
                                             eam, lj1, lj2, lj3, lj4, ljcutsq, part);
  check(cudaGetLastError(), "thermo_ip");
}

void kinetic(const double *v, const int *type, const double *mass, int n, int per_item,
             double scale, double *part, cudaStream_t s) {
  k_kinetic<<<partial_blocks(n), TB, 0, s>>>(v, type, mass, n, per_item, scale, part);
  check(cudaGetLastError(), "thermo_kinetic");
}

}  // namespace thermo
}  // namespace cacg
