// Mixed-precision pair kernels (sm_103a): FP32 pair terms, no FP64 instruction in
// any pair loop.
//
// Same formulas as the FP64 kernels (PairLJCut::compute/ecompute,
// pair_lj_cut.cpp:227-442; PairEAM::compute/ecompute, pair_eam.cpp:584-1141),
// evaluated in FP32 within a 1e-4 relative force tolerance:
//  * positions are packed cell-relative: xyz = the offset from a cell of
//    power-of-two size g in FP32, w = the cell; a pair vector
//    (q_i - q_j) + g (cell_i - cell_j) is exact up to one FP32 rounding at any
//    box size.  Atoms are packed from their FP64 positions, element sites and
//    integration points from double-single interpolation of the nodes;
//  * r, 1/r and the rho(r), r*phi(r) splines are FP32, the spline coefficients
//    FP32 in shared memory, loaded once by each resident block (persistent grid);
//  * the cutoff test is made in FP32 and re-made in FP64 inside a thin guard
//    band, so the set of interacting pairs is the FP64 set;
//  * densities and forces are summed in FP32 over chunks of 8 pairs and the
//    chunks as FP32 double-single pairs; F'(rho) of atoms and sites is FP32.
#include <algorithm>
#include <vector>

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

// The force spline per knot, 2 float4 (FTAB_W): rho'(r) c0..c2 | r*phi c3,
// then r*phi c4..c6.  The derivative of r*phi comes from its value
// coefficients, as array2spline forms it (c0 = 3 c3 / dr, c1 = 2 c4 / dr,
// c2 = c5 / dr, pair_eam.cpp:565-571): one 16-byte shared load less per pair.
__device__ __forceinline__ void force_spline(const float4 *__restrict__ tab, int m, float p,
                                             float rdr, float &rhoip, float &z2, float &z2p) {
  const float4 t0 = tab[FTAB_W * m], t1 = tab[FTAB_W * m + 1];
  rhoip = (t0.x * p + t0.y) * p + t0.z;
  z2 = ((t0.w * p + t1.x) * p + t1.y) * p + t1.z;
  z2p = ((3.0f * t0.w * p + 2.0f * t1.x) * p + t1.y) * rdr;
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

__device__ __forceinline__ float fprime32(float rho, const float4 *__restrict__ fp4, int nrho,
                                          float rdrho) {
  float p = rho * rdrho + 1.0f;
  int m = (int) p;
  m = m < nrho - 1 ? m : nrho - 1;
  m = 1 > m ? 1 : m;
  p -= (float) m;
  p = fminf(p, 1.0f);
  const float4 c = __ldg(fp4 + m);
  return (c.x * p + c.y) * p + c.z;
}

// FP32 double-single accumulator: the FP32 chunk sums are added by Knuth's
// TwoSum, without FP64 instructions (the FP64 pipe issues a warp instruction
// at a small fraction of the FP32 rate on this GPU, and it was the limit of
// the atom force pass when the chunks were added in FP64)
struct dsacc {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void add(float v) {
    const float s = __fadd_rn(h, v);
    const float b = __fsub_rn(s, h);
    l = __fadd_rn(l, __fadd_rn(__fsub_rn(h, __fsub_rn(s, b)), __fsub_rn(v, b)));
    h = s;
  }
  __device__ __forceinline__ double value() const { return (double) h + (double) l; }
};

// Double-single FP32 arithmetic: a value is an unevaluated sum hi + lo of two
// floats; products and sums use error-free transformations (TwoProduct via
// fma, Knuth's TwoSum), about 44 bits without an FP64 instruction.
struct ds {
  float h, l;
};

// fast TwoSum (|s| >= |e|)
__device__ __forceinline__ ds ds_renorm(float s, float e) {
  const float h = __fadd_rn(s, e);
  return ds{h, __fsub_rn(e, __fsub_rn(h, s))};
}

__device__ __forceinline__ ds ds_add(ds a, ds b) {
  const float s = __fadd_rn(a.h, b.h);
  const float v = __fsub_rn(s, a.h);
  float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, v)), __fsub_rn(b.h, v));
  e = __fadd_rn(e, __fadd_rn(a.l, b.l));
  return ds_renorm(s, e);
}

__device__ __forceinline__ ds ds_sub(ds a, ds b) { return ds_add(a, ds{-b.h, -b.l}); }

// x + a * d, dropping a.l * d.l
__device__ __forceinline__ ds ds_madd(ds a, ds d, ds x) {
  const float p = __fmul_rn(a.h, d.h);
  float pe = __fmaf_rn(a.h, d.h, -p);
  pe = __fmaf_rn(a.h, d.l, pe);
  pe = __fmaf_rn(a.l, d.h, pe);
  return ds_add(x, ds{p, pe});
}

// A double as a double-single by integer operations on its bits, without an
// FP64 instruction: hi keeps the sign, the exponent and the top 23 stored
// mantissa bits (a truncation, exact in FP32), lo the remaining 29 bits
// scaled by 2^(e-1075) (rounded once).  Zero and values below 2^-74 give 0.
__device__ __forceinline__ ds ds_of_double(double x) {
  const unsigned bh = (unsigned) __double2hiint(x), bl = (unsigned) __double2loint(x);
  const int ex = (int) ((bh >> 20) & 0x7FF);
  if (ex < 949) return ds{0.f, 0.f};
  const unsigned sign = bh & 0x80000000u;
  const float h = __uint_as_float(sign | ((unsigned) (ex - 896) << 23) | ((bh & 0xFFFFFu) << 3) |
                                  (bl >> 29));
  const float scale = __uint_as_float((unsigned) (ex - 948) << 23);  // 2^(ex - 1075)
  const float l = __fmul_rn(__uint2float_rn(bl & 0x1FFFFFFFu), scale);
  return ds{h, sign ? -l : l};
}

// F'(rho) as fprime64 forms it (pair_eam.cpp:1090-1100: knot index, clamps,
// cubic) from the FP64 spline's coefficients as double-single pairs, in
// double-single arithmetic: the FP32 rounding of the FP64 result, without an
// FP64 instruction
__device__ __forceinline__ float fprime_ds(ds rho, const float2 *__restrict__ c3, int nrho,
                                           float2 rdrho) {
  ds p = ds_madd(rho, ds{rdrho.x, rdrho.y}, ds{1.f, 0.f});
  int m = (int) p.h;  // floor of p.h + p.l (p >= 1)
  if ((float) m == p.h && p.l < 0.f) m -= 1;
  m = m < nrho - 1 ? m : nrho - 1;
  m = 1 > m ? 1 : m;
  p = ds_add(ds{p.h - (float) m, 0.f}, ds{p.l, 0.f});
  if (p.h + p.l > 1.f) p = ds{1.f, 0.f};
  const float2 a = c3[3 * m], b = c3[3 * m + 1], c = c3[3 * m + 2];
  ds q = ds_madd(p, ds{a.x, a.y}, ds{b.x, b.y});
  q = ds_madd(p, q, ds{c.x, c.y});
  return q.h + q.l;
}

// sum of a double-single over each aligned group of G lanes (xor shuffles)
template <int G>
__device__ __forceinline__ void group_sum(dsacc &a) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) {
    const float h = __shfl_xor_sync(0xffffffffu, a.h, o);
    const float l = __shfl_xor_sync(0xffffffffu, a.l, o);
    a.add(h);
    a.l = __fadd_rn(a.l, l);
  }
}

// exact FP64 cutoff decision for pairs whose FP32 rsq falls in the guard band
__device__ __forceinline__ bool inside64(const double4 &a, const double4 &b, double cutsq) {
  double dx = a.x - b.x, dy = a.y - b.y, dz = a.z - b.z;
  return dx * dx + dy * dy + dz * dz < cutsq;
}

// The cell fields as floats without a conversion instruction: a field k below
// 2^23 OR-ed into the bits of 2^23 reads as the float 2^23 + k, so the
// difference of two such floats is the exact integer difference of the
// fields.  The y field is left in place (bits 12-21), its difference scaled
// by 2^-12; the z field (bits 22-31) is shifted down.
constexpr int MAGIC = 0x4B000000;  // the bits of 2^23

__device__ __forceinline__ void cell_of(const float4 &q, float &cx, float &cy, float &cz) {
  const int w = __float_as_int(q.w);
  cx = __int_as_float((w & 0xFFF) | MAGIC);
  cy = __int_as_float((w & 0x3FF000) | MAGIC);
  cz = __int_as_float((int) ((unsigned) w >> 22) | MAGIC);
}

// pair vector from cell-relative coordinates: (q_i - q_j) + g * (cell_i - cell_j)
__device__ __forceinline__ void rel_vec(const float4 &qi, float cx, float cy, float cz,
                                        const float4 &qj, float g, float &dx, float &dy,
                                        float &dz) {
  float jx, jy, jz;
  cell_of(qj, jx, jy, jz);
  dx = (qi.x - qj.x) + g * (cx - jx);
  dy = (qi.y - qj.y) + (g * (1.0f / 4096.0f)) * (cy - jy);
  dz = (qi.z - qj.z) + g * (cz - jz);
}

struct AtomArgs {
  const double4 *x;
  const float4 *xq;
  float qg;
  const int *num, *list;
  int stride, nlocal;
  float cutsq_f, band_lo, band_hi;  // [band_lo, band_hi]: decide in FP64
  double cutsq;
  int *snum, *slist;  // short list written by the density pass, read by the force pass
  // displacement culling of the density pass (null: every entry is scanned):
  // nnear[i].x/.y/.z leading entries of the reordered list lay within
  // r_c + CULL_D1/D2/DELTA at the reorder; the entries beyond the level that
  // twice the largest displacement since then (dmax2: its square, float bits)
  // plus CULL_MARGIN reaches are skipped
  const int4 *nnear;
  const unsigned *dmax2;  // [0]: squared displacement bits; [1]: reordered in this step
  // F'(rho) of the density pass: from the FP64 spline at the double-single
  // density (fprime_ds: the FP32 rounding of the FP64 result), else from the
  // FP32 spline at the FP32 density (fprime32)
  const float2 *frho_ds = nullptr;
  float2 rdrho_ds = {0.f, 0.f};
};

__device__ __forceinline__ bool moved_little(const unsigned *dmax2) {
  return 2.0f * sqrtf(__uint_as_float(dmax2[0])) + CULL_MARGIN <= CULL_DELTA;
}

__device__ __forceinline__ bool cull_ok(const unsigned *dmax2) {
  return dmax2[1] != 0u || moved_little(dmax2);
}

// the culling level of this step: 1..3 (nnear .x/.y/.z), 4 = no culling
__device__ __forceinline__ int cull_level(const unsigned *dmax2) {
  if (dmax2[1] != 0u) return 1;  // reordered from this step's positions
  const float d = 2.0f * sqrtf(__uint_as_float(dmax2[0])) + CULL_MARGIN;
  return d <= CULL_D1 ? 1 : d <= CULL_D2 ? 2 : d <= CULL_DELTA ? 3 : 4;
}

__device__ __forceinline__ int culled_count(int level, const int4 &nn, int nfull) {
  return level == 1 ? nn.x : level == 2 ? nn.y : level == 3 ? nn.z : nfull;
}

// the part of an entry at squared distance rsq: 0 within the cutoff, 1..3
// within r_c + CULL_D1/D2/DELTA, 4 beyond
__device__ __forceinline__ int cull_part(float rsq, const float4 &lim) {
  return rsq <= lim.x ? 0 : rsq <= lim.y ? 1 : rsq <= lim.z ? 2 : rsq <= lim.w ? 3 : 4;
}

// Reorder of one list in two sweeps, each part in list order: the first sweep
// classifies every entry (index(k) -> entry, rsq(entry) -> squared distance)
// and counts the parts, keeping the 4-bit part codes in thread-local memory;
// the second re-reads the entries and places each at its part's cursor.  Lists
// longer than REORDER_CAP classify again in the second sweep.
constexpr int REORDER_CAP = 256;

// The first sweep keeps the list index two entries ahead and the fetched
// data of the next entry in flight (fetch(entry) -> what rsq needs), so
// that no gather waits on a list load issued in the same iteration.
template <class Index, class Fetch, class Rsq, class Put>
__device__ __forceinline__ int4 reorder_parts(int n, const float4 &lim, Index index, Fetch fetch,
                                              Rsq rsq, Put put) {
  unsigned codes[REORDER_CAP / 8];
  const bool keep = n <= REORDER_CAP;
  int c[4] = {0, 0, 0, 0};
  unsigned word = 0u;
  int en = n > 0 ? index(0) : 0, enn = n > 1 ? index(1) : 0;
  auto fn = fetch(en);
  for (int k = 0; k < n; k++) {
    const auto fk = fn;
    en = enn;
    if (k + 2 < n) enn = index(k + 2);
    if (k + 1 < n) fn = fetch(en);
    const int p = cull_part(rsq(fk), lim);
    if (p < 4) c[p]++;
    if (keep) {
      word |= (unsigned) p << (4 * (k & 7));
      if ((k & 7) == 7 || k == n - 1) {
        codes[k >> 3] = word;
        word = 0u;
      }
    }
  }
  int m[5] = {0, c[0], c[0] + c[1], c[0] + c[1] + c[2], c[0] + c[1] + c[2] + c[3]};
  const int4 nn = make_int4(m[2], m[3], m[4], n);
  for (int k = 0; k < n; k++) {
    const int e = index(k);
    int p;
    if (keep) {
      if ((k & 7) == 0) word = codes[k >> 3];
      p = (int) ((word >> (4 * (k & 7))) & 15u);
    } else {
      p = cull_part(rsq(fetch(e)), lim);
    }
    put(m[p]++, e);
  }
  return nn;
}

// 40 registers at three 512-thread blocks per SM (48 warps): more gathers in flight
__global__ void __launch_bounds__(512, 3)
k_eam_rho_atoms(AtomArgs a, const float4 *__restrict__ rhor_val, int nr, float rdr,
                const float4 *__restrict__ fp4, int nrho, float rdrho,
                double *__restrict__ rho, float *__restrict__ fp) {
  extern __shared__ float4 s_val[];
  for (int m = threadIdx.x; m <= nr; m += blockDim.x) s_val[m] = rhor_val[m];
  __syncthreads();
  const int level = a.nnear ? cull_level(a.dmax2) : 4;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nlocal; i += gridDim.x * blockDim.x) {
    const float4 qi = a.xq[i];
    float cx, cy, cz;
    cell_of(qi, cx, cy, cz);
    const int n = level < 4 ? culled_count(level, a.nnear[i], 0) : a.num[i];
    dsacc acc;
    float part = 0.f;
    int ns = 0, cnt = 0;
    // software pipeline: the list index two entries ahead and the coordinates
    // one entry ahead are in flight while this entry is evaluated, so the
    // gather never waits on a list load issued in the same iteration
    int jn = 0, jnn = 0;
    float4 qn = qi;
    if (n > 0) {
      jn = __ldg(a.list + i);
      qn = __ldg(a.xq + jn);
    }
    if (n > 1) jnn = __ldg(a.list + (size_t) a.stride + i);
    for (int k = 0; k < n; k++) {
      const int j = jn;
      const float4 qj = qn;
      jn = jnn;
      if (k + 2 < n) jnn = __ldg(a.list + (size_t) (k + 2) * a.stride + i);
      if (k + 1 < n) qn = __ldg(a.xq + jn);
      float dx, dy, dz;
      rel_vec(qi, cx, cy, cz, qj, a.qg, dx, dy, dz);
      float rsq = dx * dx + dy * dy + dz * dz;
      if (rsq > a.band_hi) continue;
      a.slist[(size_t) ns++ * a.stride + i] = j;
      bool in = rsq < a.cutsq_f;
      if (rsq >= a.band_lo) in = inside64(a.x[i], a.x[j], a.cutsq);
      if (in) {
        float p;
        int m = findex(sqrtf(rsq), rdr, nr, p);
        float4 c = s_val[m];
        part += ((c.x * p + c.y) * p + c.z) * p + c.w;
        if ((++cnt & (CHUNK - 1)) == 0) {
          acc.add(part);
          part = 0.f;
        }
      }
    }
    a.snum[i] = ns;
    acc.add(part);
    rho[i] = acc.value();
    fp[i] = a.frho_ds ? fprime_ds(ds_renorm(acc.h, acc.l), a.frho_ds, nrho, a.rdrho_ds)
                       : fprime32(__fadd_rn(acc.h, acc.l), fp4, nrho, rdrho);
  }
}

// The list of each atom reordered in five parts, each in list order: the
// entries within the cutoff (at the positions of the reorder), within
// r_c + CULL_D1, r_c + CULL_D2, r_c + CULL_DELTA, and the rest; nnear[i]
// counts the entries through the second, third and fourth parts.  Atoms move
// little, so in the density pass the lanes of a warp meet the in-range entries
// together and the out-of-range ones together, and the farther parts are
// skipped while no atom has moved far enough to reach them.  Launched every
// step: it returns at once while no atom has moved (CULL_DELTA - CULL_MARGIN)
// / 2 since the last reorder, else it reorders from the current positions,
// keeps them as the new reference and flags the step (dmax2[1]).
__global__ void k_list_partition(const float4 *__restrict__ xq, float g, const int *__restrict__ num,
                                 const int *__restrict__ list, int stride, int nlocal, float4 lim,
                                 int *__restrict__ out, int4 *__restrict__ nnear,
                                 float4 *__restrict__ ref, unsigned *__restrict__ dmax2,
                                 unsigned *__restrict__ reorders) {
  // (the gate reads only dmax2[0], which no block of this kernel writes)
  if (moved_little(dmax2)) return;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    dmax2[1] = 1u;
    if (reorders) *reorders += 1u;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nlocal; i += gridDim.x * blockDim.x) {
    const float4 qi = xq[i];
    ref[i] = qi;
    float cx, cy, cz;
    cell_of(qi, cx, cy, cz);
    auto index = [&](int k) { return __ldg(list + (size_t) k * stride + i); };
    auto fetch = [&](int j) { return __ldg(xq + j); };
    auto rsq = [&](const float4 &qj) {
      float dx, dy, dz;
      rel_vec(qi, cx, cy, cz, qj, g, dx, dy, dz);
      return dx * dx + dy * dy + dz * dz;
    };
    auto put = [&](int at, int j) { out[(size_t) at * stride + i] = j; };
    nnear[i] = reorder_parts(num[i], lim, index, fetch, rsq, put);
  }
}

// ---- neighbor unions staged in shared memory (EAM atom passes) ----
//
// The 32 atoms a warp owns (consecutive local indices) share most of their
// neighbors.  At each list build the union of their list entries is
// collected (at most UMAX distinct atoms; a larger union marks the group for
// the direct path) and every list entry is re-expressed as a 16-bit slot
// into it.  Each step a warp loads the union's packed coordinates (and, in
// the force pass, F') once into shared memory and then walks its lists
// exactly as the direct kernels do, reading neighbors from shared memory: the
// arithmetic and its order are unchanged, the L2 gathers drop by the
// neighbor overlap (about 7x for lattice-ordered atoms).
constexpr int UGROUP = 32, UMAX = 640, UHASH = 2048, UWARPS = 8;

// one block per group: hash the group's entries, number the distinct atoms,
// write each entry's slot
__global__ void __launch_bounds__(256)
k_union_build(const int *__restrict__ num, const int *__restrict__ list, int stride, int nlocal,
              int *__restrict__ union_j, int *__restrict__ union_n,
              unsigned short *__restrict__ slot) {
  __shared__ int keys[UHASH], vals[UHASH];
  __shared__ int count, overflow;
  const int g = blockIdx.x, i0 = g * UGROUP;
  for (int h = threadIdx.x; h < UHASH; h += blockDim.x) keys[h] = -1;
  if (threadIdx.x == 0) {
    count = 0;
    overflow = 0;
  }
  __syncthreads();
  // insert: thread t takes entries t, t + 256, ... of the group (atom-major)
  int maxn = 0;
  for (int a = 0; a < UGROUP && i0 + a < nlocal; a++) maxn = max(maxn, num[i0 + a]);
  const int total = UGROUP * maxn;
  for (int e = threadIdx.x; e < total && !*((volatile int *) &overflow); e += blockDim.x) {
    const int a = e % UGROUP, k = e / UGROUP, i = i0 + a;
    if (i >= nlocal || k >= num[i]) continue;
    const int j = list[(size_t) k * stride + i];
    unsigned h = ((unsigned) j * 2654435761u) & (UHASH - 1);
    for (int probe = 0; probe < UHASH; probe++) {
      const int old = atomicCAS(&keys[h], -1, j);
      if (old == -1) {
        if (atomicAdd(&count, 1) >= UMAX) overflow = 1;
        break;
      }
      if (old == j) break;
      h = (h + 1) & (UHASH - 1);
    }
  }
  __syncthreads();
  if (overflow || count > UMAX) {
    if (threadIdx.x == 0) union_n[g] = -1;
    return;
  }
  if (threadIdx.x == 0) count = 0;
  __syncthreads();
  for (int h = threadIdx.x; h < UHASH; h += blockDim.x)
    if (keys[h] != -1) {
      const int sl = atomicAdd(&count, 1);
      vals[h] = sl;
      union_j[(size_t) g * UMAX + sl] = keys[h];
    }
  __syncthreads();
  if (threadIdx.x == 0) union_n[g] = count;
  for (int e = threadIdx.x; e < total; e += blockDim.x) {
    const int a = e % UGROUP, k = e / UGROUP, i = i0 + a;
    if (i >= nlocal || k >= num[i]) continue;
    const int j = list[(size_t) k * stride + i];
    unsigned h = ((unsigned) j * 2654435761u) & (UHASH - 1);
    for (int probe = 0; probe < UHASH && keys[h] != j; probe++) h = (h + 1) & (UHASH - 1);
    slot[(size_t) k * stride + i] = (unsigned short) vals[h];
  }
}

struct UnionArgs {
  const int *union_j, *union_n;
  const unsigned short *slot;  // list entries as union slots
  unsigned short *sslot;       // short list as union slots (staged groups)
};

__global__ void __launch_bounds__(UGROUP * UWARPS, 1)
k_eam_rho_union(AtomArgs a, UnionArgs u, const float4 *__restrict__ rhor_val, int nr, float rdr,
                const float4 *__restrict__ fp4, int nrho, float rdrho,
                double *__restrict__ rho, float *__restrict__ fp) {
  extern __shared__ float4 sm[];
  float4 *s_val = sm;                                  // nr + 1 knots
  float4 *sx = sm + (nr + 1) + (threadIdx.x >> 5) * UMAX;  // this warp's union
  for (int m = threadIdx.x; m <= nr; m += blockDim.x) s_val[m] = rhor_val[m];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int ngroups = (a.nlocal + UGROUP - 1) / UGROUP;
  for (int g = blockIdx.x * UWARPS + (threadIdx.x >> 5); g < ngroups; g += gridDim.x * UWARPS) {
    const int nu = u.union_n[g];
    const int i = g * UGROUP + lane;
    if (nu >= 0)
      for (int s = lane; s < nu; s += 32) sx[s] = __ldg(a.xq + u.union_j[(size_t) g * UMAX + s]);
    __syncwarp();
    if (i < a.nlocal) {
      const float4 qi = a.xq[i];
      float cx, cy, cz;
      cell_of(qi, cx, cy, cz);
      const int n = a.num[i];
      dsacc acc;
      float part = 0.f;
      int ns = 0, cnt = 0;
      for (int k = 0; k < n; k++) {
        int j, sl = 0;
        float4 qj;
        if (nu >= 0) {
          sl = u.slot[(size_t) k * a.stride + i];
          qj = sx[sl];
          j = -1;
        } else {
          j = __ldg(a.list + (size_t) k * a.stride + i);
          qj = __ldg(a.xq + j);
        }
        float dx, dy, dz;
        rel_vec(qi, cx, cy, cz, qj, a.qg, dx, dy, dz);
        float rsq = dx * dx + dy * dy + dz * dz;
        if (rsq > a.band_hi) continue;
        if (nu >= 0) u.sslot[(size_t) ns++ * a.stride + i] = (unsigned short) sl;
        else a.slist[(size_t) ns++ * a.stride + i] = j;
        bool in = rsq < a.cutsq_f;
        if (rsq >= a.band_lo) {
          if (j < 0) j = u.union_j[(size_t) g * UMAX + sl];
          in = inside64(a.x[i], a.x[j], a.cutsq);
        }
        if (in) {
          float p;
          int m = findex(sqrtf(rsq), rdr, nr, p);
          float4 c = s_val[m];
          part += ((c.x * p + c.y) * p + c.z) * p + c.w;
          if ((++cnt & (CHUNK - 1)) == 0) {
            acc.add(part);
            part = 0.f;
          }
        }
      }
      a.snum[i] = ns;
      acc.add(part);
      rho[i] = acc.value();
      fp[i] = a.frho_ds ? fprime_ds(ds_renorm(acc.h, acc.l), a.frho_ds, nrho, a.rdrho_ds)
                        : fprime32(__fadd_rn(acc.h, acc.l), fp4, nrho, rdrho);
    }
    __syncwarp();  // the union is overwritten by the warp's next group
  }
}

__global__ void __launch_bounds__(UGROUP * UWARPS, 1)
k_eam_force_union(AtomArgs a, UnionArgs u, const float4 *__restrict__ ftab, int nr, float rdr,
                  const float *__restrict__ fp, double *__restrict__ f) {
  extern __shared__ float4 sm[];
  float4 *s_tab = sm;  // 3 float4 per knot
  float4 *sx = sm + FTAB_W * (nr + 1) + (threadIdx.x >> 5) * UMAX;
  float *sfp = reinterpret_cast<float *>(sm + FTAB_W * (nr + 1) + UWARPS * UMAX) + (threadIdx.x >> 5) * UMAX;
  for (int m = threadIdx.x; m < FTAB_W * (nr + 1); m += blockDim.x) s_tab[m] = ftab[m];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int ngroups = (a.nlocal + UGROUP - 1) / UGROUP;
  for (int g = blockIdx.x * UWARPS + (threadIdx.x >> 5); g < ngroups; g += gridDim.x * UWARPS) {
    const int nu = u.union_n[g];
    const int i = g * UGROUP + lane;
    if (nu >= 0)
      for (int s = lane; s < nu; s += 32) {
        const int j = u.union_j[(size_t) g * UMAX + s];
        sx[s] = __ldg(a.xq + j);
        sfp[s] = __ldg(fp + j);
      }
    __syncwarp();
    if (i < a.nlocal) {
      const float4 qi = a.xq[i];
      float cx, cy, cz;
      cell_of(qi, cx, cy, cz);
      const float fpi = fp[i];
      const int n = a.snum[i];
      dsacc fx, fy, fz;
      float px = 0.f, py = 0.f, pz = 0.f;
      int cnt = 0;
      for (int k = 0; k < n; k++) {
        int j = -1, sl = 0;
        float4 qj;
        float fpj;
        if (nu >= 0) {
          sl = u.sslot[(size_t) k * a.stride + i];
          qj = sx[sl];
          fpj = sfp[sl];
        } else {
          j = __ldg(a.slist + (size_t) k * a.stride + i);
          qj = __ldg(a.xq + j);
          fpj = __ldg(fp + j);
        }
        float dx, dy, dz;
        rel_vec(qi, cx, cy, cz, qj, a.qg, dx, dy, dz);
        float rsq = dx * dx + dy * dy + dz * dz;
        bool in = rsq < a.cutsq_f;
        if (rsq >= a.band_lo && rsq <= a.band_hi) {
          if (j < 0) j = u.union_j[(size_t) g * UMAX + sl];
          in = inside64(a.x[i], a.x[j], a.cutsq);
        }
        if (in) {
          float recip = rsqrtf(rsq);
          float r = rsq * recip;
          float p;
          int m = findex(r, rdr, nr, p);
          float rhoip, z2, z2p;
          force_spline(s_tab, m, p, rdr, rhoip, z2, z2p);
          float phi = z2 * recip;
          float phip = z2p * recip - phi * recip;
          float psip = (fpi + fpj) * rhoip + phip;
          float fpair = -psip * recip;
          px += dx * fpair;
          py += dy * fpair;
          pz += dz * fpair;
          if ((++cnt & (CHUNK - 1)) == 0) {
            fx.add(px);
            fy.add(py);
            fz.add(pz);
            px = py = pz = 0.f;
          }
        }
      }
      fx.add(px);
      f[3 * i] = fx.value();
      fy.add(py);
      f[3 * i + 1] = fy.value();
      fz.add(pz);
      f[3 * i + 2] = fz.value();
    }
    __syncwarp();
  }
}

// force table per knot: FTAB_W float4 (force_spline).  For large systems one
// 1024-thread block per SM: the 64 KB table is held once per SM, which leaves
// the unified L1/shared memory's rest to the neighbor gathers (smaller systems
// keep the tuned block size, for more blocks than SMs).
constexpr int FORCE_BLOCK = 1024;
__global__ void __launch_bounds__(FORCE_BLOCK, 1)
k_eam_force_atoms(AtomArgs a, const float4 *__restrict__ ftab, int nr, float rdr,
                  const float *__restrict__ fp, double *__restrict__ f) {
  extern __shared__ float4 s_tab[];  // 3 float4 per knot
  for (int m = threadIdx.x; m < FTAB_W * (nr + 1); m += blockDim.x) s_tab[m] = ftab[m];
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nlocal; i += gridDim.x * blockDim.x) {
    const float4 qi = a.xq[i];
    float cx, cy, cz;
    cell_of(qi, cx, cy, cz);
    const float fpi = fp[i];
    const int n = a.snum[i];
    dsacc fx, fy, fz;
    float px = 0.f, py = 0.f, pz = 0.f;
    int cnt = 0;
    // software pipeline: the list index two entries ahead and the next
    // entry's coordinates and F' in flight while this entry is evaluated, so
    // that no gather waits on a list load issued in the same iteration
    int jn = 0, jnn = 0;
    float4 qn = qi;
    float fpn = 0.f;
    if (n > 0) {
      jn = __ldg(a.slist + i);
      qn = __ldg(a.xq + jn);
      fpn = __ldg(fp + jn);
    }
    if (n > 1) jnn = __ldg(a.slist + (size_t) a.stride + i);
    for (int k = 0; k < n; k++) {
      const int j = jn;
      const float4 qj = qn;
      const float fpj = fpn;
      jn = jnn;
      if (k + 2 < n) jnn = __ldg(a.slist + (size_t) (k + 2) * a.stride + i);
      if (k + 1 < n) {
        qn = __ldg(a.xq + jn);
        fpn = __ldg(fp + jn);
      }
      float dx, dy, dz;
      rel_vec(qi, cx, cy, cz, qj, a.qg, dx, dy, dz);
      float rsq = dx * dx + dy * dy + dz * dz;
      bool in = rsq < a.cutsq_f;
      if (rsq >= a.band_lo && rsq <= a.band_hi) in = inside64(a.x[i], a.x[j], a.cutsq);
      if (in) {
        float recip = rsqrtf(rsq);
        float r = rsq * recip;
        float p;
        int m = findex(r, rdr, nr, p);
        float rhoip, z2, z2p;
        force_spline(s_tab, m, p, rdr, rhoip, z2, z2p);
        float phi = z2 * recip;
        float phip = z2p * recip - phi * recip;
        float psip = (fpi + fpj) * rhoip + phip;
        float fpair = -psip * recip;
        px += dx * fpair;
        py += dy * fpair;
        pz += dz * fpair;
        if ((++cnt & (CHUNK - 1)) == 0) {
          fx.add(px);
          fy.add(py);
          fz.add(pz);
          px = py = pz = 0.f;
        }
      }
    }
    fx.add(px);
    f[3 * i] = fx.value();
    fy.add(py);
    f[3 * i + 1] = fy.value();
    fz.add(pz);
    f[3 * i + 2] = fz.value();
  }
}

// band_lo/band_hi are relative factors here: a pair with rsq in
// [band_lo, band_hi] * cutsq(type pair) is decided in FP64
__global__ void __launch_bounds__(512, 2)
k_lj_atoms(AtomArgs a, const int *__restrict__ type, const float *__restrict__ lj1,
           const float *__restrict__ lj2, const float *__restrict__ cutsq_t,
           const double *__restrict__ cutsq64, double *__restrict__ f) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < a.nlocal; i += gridDim.x * blockDim.x) {
    const float4 qi = a.xq[i];
    float cx, cy, cz;
    cell_of(qi, cx, cy, cz);
    const int it = type[i];
    const int n = a.num[i];
    dsacc fx, fy, fz;
    float px = 0.f, py = 0.f, pz = 0.f;
    // the list index two entries ahead, the next coordinates one ahead
    int jn = 0, jnn = 0;
    float4 qn = qi;
    if (n > 0) {
      jn = __ldg(a.list + i);
      qn = __ldg(a.xq + jn);
    }
    if (n > 1) jnn = __ldg(a.list + (size_t) a.stride + i);
    for (int k = 0; k < n; k++) {
      const int j = jn;
      const float4 qj = qn;
      jn = jnn;
      if (k + 2 < n) jnn = __ldg(a.list + (size_t) (k + 2) * a.stride + i);
      if (k + 1 < n) qn = __ldg(a.xq + jn);
      float dx, dy, dz;
      rel_vec(qi, cx, cy, cz, qj, a.qg, dx, dy, dz);
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
        fx.add(px);
        fy.add(py);
        fz.add(pz);
        px = py = pz = 0.f;
      }
    }
    fx.add(px);
    f[3 * i] = fx.value();
    fy.add(py);
    f[3 * i + 1] = fy.value();
    fz.add(pz);
    f[3 * i + 2] = fz.value();
  }
}

// ---------------------------------------------------------------- elements
//
// Element sites are computed once per step in double-single FP32 arithmetic (a
// value is an unevaluated sum hi + lo of two floats; products and sums use
// error-free transformations: TwoProduct via fma and Knuth's TwoSum), so a site
// carries ~44 bits from the FP64 nodes without a single FP64 instruction per
// site, and is stored in the same cell-relative packed form as the atoms
// (16 bytes a site).  The trilinear map of an element is evaluated as lerps:
// along x per lattice column, along y per lattice line, and along z per site
// (x(i,j,k) = U(i,j) + c_k D(i,j)), so a site costs three double-single
// multiply-adds.

__device__ __forceinline__ ds ds_lerp(ds x, ds y, ds a) { return ds_madd(a, ds_sub(y, x), x); }

// the lattice fraction k / (n - 1) along an axis of a type, as a double-single
__device__ __forceinline__ ds frac_of(const Lattice &lat, int ty, int axis, int k) {
  const float2 v = __ldg(lat.frac + (size_t) (ty * 3 + axis) * lat.fstride + k);
  return ds{v.x, v.y};
}

// node coordinates as double-single pairs, once per element and step
// with a reference (the split nodes of the last integration-point list
// reorder) the largest squared node displacement since then is folded into
// *dmax2 (float bits, one atomic max per block): every site and integration
// point is a convex combination of its element's nodes, so none moved more
constexpr int SPLIT_BLOCK = 256;

__global__ void __launch_bounds__(SPLIT_BLOCK)
k_node_split(const double *__restrict__ nodex, int n, float2 *__restrict__ hl,
             const float2 *__restrict__ ref, unsigned *__restrict__ dmax2) {
  __shared__ unsigned s_max[SPLIT_BLOCK / 32];
  const int t = blockIdx.x * blockDim.x + threadIdx.x;  // one node (3 coordinates)
  float d2 = 0.f;
  if (t < n * NPE) {
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const ds v = ds_of_double(nodex[3 * (size_t) t + d]);
      hl[3 * (size_t) t + d] = make_float2(v.h, v.l);
      if (ref) {
        const float2 r = ref[3 * (size_t) t + d];
        const float dd = __fsub_rn(v.h, r.x) + __fsub_rn(v.l, r.y);
        d2 += dd * dd;
      }
    }
  }
  if (ref) {  // the same for every thread of the grid
    unsigned m = __reduce_max_sync(0xffffffffu, __float_as_uint(d2));
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
      m = threadIdx.x < SPLIT_BLOCK / 32 ? s_max[threadIdx.x] : 0u;
      m = __reduce_max_sync(0xffffffffu, m);
      if (threadIdx.x == 0 && m) atomicMax(dmax2, m);
    }
  }
}

__device__ __forceinline__ ds node_ds(const float2 *nx, int k, int d) {
  const float2 v = nx[3 * k + d];
  return ds{v.x, v.y};
}

// Packing of a double-single offset u = x - l0 into (cell, rel): the cell
// index floor(u.h / g) is exact (g a power of two), u.h - k g is exact
// (Sterbenz), so rel = (u.h - k g) + u.l is rounded once.
__device__ __forceinline__ float rel_of(ds u, float g, float ig, int lim, int &k, bool &bad) {
  k = (int) floorf(__fmul_rn(u.h, ig));
  if (k < 0 || k > lim) {
    bad = true;
    k = k < 0 ? 0 : lim;
  }
  return __fadd_rn(__fsub_rn(u.h, __fmul_rn((float) k, g)), u.l);
}

__device__ __forceinline__ float4 pack_u(ds ux, ds uy, ds uz, const PackGrid &pg) {
  int cx, cy, cz;
  bool bad = false;
  const float rx = rel_of(ux, pg.g, pg.ig, 4095, cx, bad);
  const float ry = rel_of(uy, pg.g, pg.ig, 1023, cy, bad);
  const float rz = rel_of(uz, pg.g, pg.ig, 1023, cz, bad);
  if (bad && pg.oob) atomicAdd(pg.oob, 1);
  return make_float4(rx, ry, rz, __int_as_float(cx | (cy << 12) | (cz << 22)));
}

// packed coordinates; with a reference (the packed coordinates of the list
// reorder, same grid) the largest squared displacement of the first nref
// atoms is folded into *dmax2 (float bits, one atomic max per block)
constexpr int PACK_BLOCK = 256;

__global__ void __launch_bounds__(PACK_BLOCK)
k_pack_rel(const double4 *__restrict__ x, int n, PackGrid pg, float4 *__restrict__ xq,
           const float4 *__restrict__ ref, int nref, unsigned *__restrict__ dmax2) {
  __shared__ unsigned s_max[PACK_BLOCK / 32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned m = 0u;
  if (i < n) {
    const double4 p = x[i];
    const float4 q = pack_u(ds_sub(ds_of_double(p.x), ds{pg.l0h[0], pg.l0l[0]}),
                            ds_sub(ds_of_double(p.y), ds{pg.l0h[1], pg.l0l[1]}),
                            ds_sub(ds_of_double(p.z), ds{pg.l0h[2], pg.l0l[2]}), pg);
    xq[i] = q;
    if (ref && i < nref) {
      float cx, cy, cz, dx, dy, dz;
      cell_of(q, cx, cy, cz);
      rel_vec(q, cx, cy, cz, ref[i], pg.g, dx, dy, dz);
      m = __float_as_uint(dx * dx + dy * dy + dz * dz);
    }
  }
  if (ref) {  // the same for every thread of the grid
    m = __reduce_max_sync(0xffffffffu, m);
    if ((threadIdx.x & 31) == 0) s_max[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
      m = threadIdx.x < PACK_BLOCK / 32 ? s_max[threadIdx.x] : 0u;
      m = __reduce_max_sync(0xffffffffu, m);
      if (threadIdx.x == 0 && m) atomicMax(dmax2, m);
    }
  }
}

// the x-lerps of one lattice column ii: E0..E3 of the y/z edges (-,-), (+,-), (-,+), (+,+)
__device__ __forceinline__ void column_ds(const float2 *nx, ds a, int d, ds (&E)[4]) {
  E[0] = ds_lerp(node_ds(nx, 0, d), node_ds(nx, 1, d), a);
  E[1] = ds_lerp(node_ds(nx, 3, d), node_ds(nx, 2, d), a);
  E[2] = ds_lerp(node_ds(nx, 4, d), node_ds(nx, 5, d), a);
  E[3] = ds_lerp(node_ds(nx, 7, d), node_ds(nx, 6, d), a);
}

// Lattice lines of this step: per element, per lattice column ii the x-lerps
// give P = E0 - l0, Q = E1 - E0, R = E2 - E0 and S = (E3 - E2) - (E1 - E0),
// so that a line (ii, jj) starts at U = P + b Q and steps D = R + b S
// (b = jj / (ny - 1)); its site kk is U + c D (c = kk / (nz - 1)), all in
// double-single.  One warp per element writes U and D of every line that a
// scanned list entry references (48 bytes a line); the integration-point
// passes evaluate the sites from them.
constexpr int LCH = 128;

// line data: U.x, U.y | U.z, D.x | D.y, D.z as double-single pairs
// list entries are line codes: line << lat.kb | kk
__device__ __forceinline__ int code_line(const Lattice &lat, int code) { return code >> lat.kb; }
__device__ __forceinline__ int code_kk(const Lattice &lat, int code) {
  return code & ((1 << lat.kb) - 1);
}

__device__ __forceinline__ void line_site(const float4 *__restrict__ lp, int line, ds c,
                                          ds (&x)[3]) {
  const float4 a = __ldg(lp + 3 * (size_t) line);
  const float4 b = __ldg(lp + 3 * (size_t) line + 1);
  const float4 d = __ldg(lp + 3 * (size_t) line + 2);
  x[0] = ds_madd(c, ds{b.z, b.w}, ds{a.x, a.y});
  x[1] = ds_madd(c, ds{d.x, d.y}, ds{a.z, a.w});
  x[2] = ds_madd(c, ds{d.z, d.w}, ds{b.x, b.y});
}

__global__ void __launch_bounds__(LCH)
k_lines(const float2 *__restrict__ node_hl, const int *__restrict__ etype, Lattice lat,
        const unsigned long long *__restrict__ line_mask,
        const unsigned long long *__restrict__ line_mask_near, const unsigned *__restrict__ eflags,
        int maxlines, PackGrid pg, int nelem, int max_nax, float4 *__restrict__ line_pos,
        const unsigned *__restrict__ gate) {
  // one warp per element: [nax][3][4] P, Q, R, S of the warp's element
  extern __shared__ ds s_cols[];
  __shared__ float2 s_nodes[LCH / 32][24];
  if (gate && moved_little(gate)) return;  // no list reorder in this step
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  ds *s_col = s_cols + (size_t) w * 12 * max_nax;
  float2 *s_nx = s_nodes[w];
  // a persistent grid (a gated step then costs one short launch)
  for (int e = blockIdx.x * (LCH / 32) + w; e < nelem; e += gridDim.x * (LCH / 32)) {
  const int ty = etype[e];
  const int *nae = lat.nae;
  const int nax = nae[3 * ty], nay = nae[3 * ty + 1];
  if (lane < 24) s_nx[lane] = node_hl[24 * (size_t) e + lane];
  __syncwarp();
  const ds l0[3] = {{pg.l0h[0], pg.l0l[0]}, {pg.l0h[1], pg.l0l[1]}, {pg.l0h[2], pg.l0l[2]}};
  for (int q = lane; q < 3 * nax; q += 32) {
    const int ii = q / 3, d = q % 3;
    ds E[4];
    column_ds(s_nx, frac_of(lat, ty, 0, ii), d, E);
    ds *o = s_col + (ii * 3 + d) * 4;
    const ds q1 = ds_sub(E[1], E[0]);
    o[0] = ds_sub(E[0], l0[d]);
    o[1] = q1;
    o[2] = ds_sub(E[2], E[0]);
    o[3] = ds_sub(ds_sub(E[3], E[2]), q1);
  }
  __syncwarp();
  // while culling holds only the lines of the rows' near entries are needed
  const unsigned long long *lm =
      (line_mask_near && cull_ok(eflags) ? line_mask_near : line_mask) + (size_t) e * maxlines;
  float4 *out = line_pos + 3 * (size_t) e * maxlines;
  for (int L = lane; L < nax * nay; L += 32) {
    if (lm[L] == 0ull) continue;
    const int ii = L / nay, jj = L - ii * nay;
    const ds b = frac_of(lat, ty, 1, jj);
    ds U[3], D[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const ds *c = s_col + (ii * 3 + d) * 4;
      U[d] = ds_madd(b, c[1], c[0]);
      D[d] = ds_madd(b, c[3], c[2]);
    }
    out[3 * L] = make_float4(U[0].h, U[0].l, U[1].h, U[1].l);
    out[3 * L + 1] = make_float4(U[2].h, U[2].l, D[0].h, D[0].l);
    out[3 * L + 2] = make_float4(D[1].h, D[1].l, D[2].h, D[2].l);
  }
  __syncwarp();  // the warp's shared columns are rewritten for its next element
  }
}

// Nodal-density lines, FP32: rho at site kk of line (ii, jj) is B + c (T - B)
// with B, T the bilinear values of the nodal densities on the z = -1 and z = +1
// faces (pair_eam.cpp:1060-1065: rho_s = sum_k N_k erho_k).  One warp per
// element, the lines that a scanned force-row entry references.
__global__ void __launch_bounds__(LCH)
k_line_rho(const double *__restrict__ erho, const int *__restrict__ etype, Lattice lat,
           const unsigned long long *__restrict__ line_mask,
           const unsigned long long *__restrict__ line_mask_near,
           const unsigned *__restrict__ eflags, int maxlines, int nelem,
           float2 *__restrict__ line_rho) {
  // one warp per element
  __shared__ float s_erho[LCH / 32][NPE];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int e = blockIdx.x * (LCH / 32) + w;
  if (e >= nelem) return;
  float *s_er = s_erho[w];
  const int ty = etype[e];
  const int nax = lat.nae[3 * ty], nay = lat.nae[3 * ty + 1];
  if (lane < NPE) s_er[lane] = (float) erho[NPE * (size_t) e + lane];
  __syncwarp();
  const unsigned long long *lm =
      (line_mask_near && cull_ok(eflags) ? line_mask_near : line_mask) + (size_t) e * maxlines;
  float2 *out = line_rho + (size_t) e * maxlines;
  for (int L = lane; L < nax * nay; L += 32) {
    if (lm[L] == 0ull) continue;
    const int ii = L / nay, jj = L - ii * nay;
    const float a = frac_of(lat, ty, 0, ii).h, b = frac_of(lat, ty, 1, jj).h;
    const float e0 = s_er[0] + a * (s_er[1] - s_er[0]), e1 = s_er[3] + a * (s_er[2] - s_er[3]);
    const float e2 = s_er[4] + a * (s_er[5] - s_er[4]), e3 = s_er[7] + a * (s_er[6] - s_er[7]);
    const float B = e0 + b * (e1 - e0), T = e2 + b * (e3 - e2);
    out[L] = make_float2(B, T - B);
  }
}

// Line masks from the entry codes: bit kk of mask[line] for every entry of
// every row (mask) and of the rows of nonzero weight (mask_f); with `gate`,
// only after a reorder in this step, from the rows' culled parts.
__global__ void k_masks_clear(unsigned long long *__restrict__ mask,
                              unsigned long long *__restrict__ mask_f, long long n,
                              const unsigned *__restrict__ gate) {
  if (gate && gate[1] == 0u) return;
  for (long long t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    mask[t] = 0ull;
    mask_f[t] = 0ull;
  }
}

// lattice lines with at least one referenced site, in mask and mask_f
__global__ void k_count_lines(const unsigned long long *__restrict__ mask,
                              const unsigned long long *__restrict__ mask_f, long long n,
                              unsigned long long *__restrict__ count) {
  unsigned long long a = 0, b = 0;
  for (long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x; t < n;
       t += (long long) gridDim.x * blockDim.x) {
    a += mask[t] != 0ull;
    b += mask_f[t] != 0ull;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(count, a);
    atomicAdd(count + 1, b);
  }
}

__global__ void k_masks_or(const int *__restrict__ row_start, const int *__restrict__ ent,
                           const int4 *__restrict__ nnear_row, int nrows, Lattice lat,
                           const unsigned char *__restrict__ isforce,
                           unsigned long long *__restrict__ mask,
                           unsigned long long *__restrict__ mask_f,
                           const unsigned *__restrict__ gate) {
  if (gate && gate[1] == 0u) return;
  const int stride = gridDim.x * blockDim.x;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    const int s0 = row_start[r];
    const int n = nnear_row ? nnear_row[r].z : row_start[r + 1] - s0;  // every culled part
    const bool f = isforce[r] != 0;
    for (int k = 0; k < n; k++) {
      const int code = __ldg(ent + s0 + k);
      const unsigned long long bit = 1ull << code_kk(lat, code);
      atomicOr(mask + code_line(lat, code), bit);
      if (f) atomicOr(mask_f + code_line(lat, code), bit);
    }
  }
}

// the integration-point lists' site ids turned into line codes
// (element * maxlines + line) << 6 | kk
__global__ void k_ent_codes(int *__restrict__ ent, long long n, const int *__restrict__ site_base,
                            int nall_e, const int *__restrict__ etype, const int *__restrict__ nae,
                            int maxlines, int kb) {
  for (long long t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const int sid = ent[t];
    int lo = 0, hi = nall_e;  // site_base[lo] <= sid < site_base[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (site_base[mid] <= sid) lo = mid;
      else hi = mid;
    }
    const int naz = nae[3 * etype[lo] + 2], nj = sid - site_base[lo];
    const int L = nj / naz, kk = nj - L * naz;
    ent[t] = (int) ((((long long) lo * maxlines + L) << kb) | kk);
  }
}

struct ElemArgs {
  const float4 *line_pos;  // lattice lines of this step (k_lines)
  const float2 *line_rho;  // nodal-density lines (EAM force pass)
  const float4 *fp4;       // FP32 F' spline, c0..c2 per knot
  int nrho;
  float rdrho;
  const float4 *ip_q;    // packed integration-point positions of this step
  const float4 *ip_h, *ip_l;  // their double-single positions (guard band)
  const float *row_fp;        // F'(rho) at the rows of nonzero weight (EAM force pass)
  const int *etype, *row_elem, *row_first, *node_list;
  const int *row_start, *ent;  // integration-point lists, row-major line codes (near first)
  const int4 *nnear_row;       // culled entry counts per row (null: no culling)
  const unsigned *eflags;      // [0] node displacement^2 since the reorder, [1] reordered now
  int nlocal_e;
  const int *rows;
  int nforce;
  float cutsq_f, band_lo, band_hi;
  double cutsq;
  const unsigned char *skip;
  Lattice lat;
  PackGrid pg;
};

// integration-point position in double-single from the split nodes and the
// split integration-point shape functions
__device__ __forceinline__ void ip_ds(const float2 *__restrict__ N, const float2 *__restrict__ nx,
                                      ds (&x)[3]) {
#pragma unroll
  for (int d = 0; d < 3; d++) {
    float h = 0.f, l = 0.f;
#pragma unroll
    for (int k = 0; k < NPE; k++) {
      const float2 w = N[k], c = nx[3 * k + d];
      // (h, l) += (w.x + w.y) * (c.x + c.y), dropping w.y * c.y
      const float p = __fmul_rn(w.x, c.x);
      float e = __fmaf_rn(w.x, c.x, -p);
      e = __fmaf_rn(w.x, c.y, e);
      e = __fmaf_rn(w.y, c.x, e);
      const float s = __fadd_rn(h, p);
      const float v = __fsub_rn(s, h);
      const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, v)), __fsub_rn(p, v));
      l = __fadd_rn(l, __fadd_rn(e, err));
      h = s;
    }
    x[d] = ds_renorm(h, l);
  }
}

// Every row's integration point, once per step: packed, and in double-single
// for the guard-band tests
__global__ void k_row_q(const int *__restrict__ row_elem, const int *__restrict__ row_jj,
                        const int *__restrict__ etype, const int *__restrict__ int_off,
                        const float2 *__restrict__ spa_int_hl, const float2 *__restrict__ node_hl,
                        int nrows, PackGrid pg, float4 *__restrict__ ip_q,
                        float4 *__restrict__ ip_h, float4 *__restrict__ ip_l,
                        const unsigned *__restrict__ gate) {
  if (gate && moved_little(gate)) return;  // no list reorder in this step
  const ds l0[3] = {{pg.l0h[0], pg.l0l[0]}, {pg.l0h[1], pg.l0l[1]}, {pg.l0h[2], pg.l0l[2]}};
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    const int e = row_elem[r], ty = etype[e];
    ds x[3];
    ip_ds(spa_int_hl + ((size_t) int_off[ty] + row_jj[r]) * NPE, node_hl + 24 * (size_t) e, x);
    ip_q[r] = pack_u(ds_sub(x[0], l0[0]), ds_sub(x[1], l0[1]), ds_sub(x[2], l0[2]), pg);
    ip_h[r] = make_float4(x[0].h, x[1].h, x[2].h, 0.f);
    ip_l[r] = make_float4(x[0].l, x[1].l, x[2].l, 0.f);
  }
}

// F'(rho_i) at the rows of nonzero weight, rho_i = sum_k N_k erho_k in FP64
// (pair_eam.cpp:1090-1100)
__global__ void k_row_fp(const int *__restrict__ rows, int nforce, const int *__restrict__ row_elem,
                         const int *__restrict__ row_jj, const int *__restrict__ etype,
                         const int *__restrict__ int_off, const double *__restrict__ spa_int,
                         const double *__restrict__ erho, const double *__restrict__ frho, int nrho,
                         double rdrho, float *__restrict__ row_fp) {
  const int it = blockIdx.x * blockDim.x + threadIdx.x;
  if (it >= nforce) return;
  const int r = rows[it], e = row_elem[r], ty = etype[e];
  const double *N = spa_int + ((size_t) int_off[ty] + row_jj[r]) * NPE;
  double rho = 0.0;
#pragma unroll
  for (int k = 0; k < NPE; k++) rho += N[k] * erho[NPE * (size_t) e + k];
  row_fp[r] = (float) fprime64(rho, frho, nrho, rdrho);
}

// row-major copy of the column-major integration-point lists
__global__ void k_ip_csr(const int *__restrict__ ipnum, const int *__restrict__ ipent, int nrows,
                         int rowstride, const int *__restrict__ row_start, int *__restrict__ ent) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows) return;
  const int n = ipnum[r], s0 = row_start[r];
  for (int k = 0; k < n; k++) ent[s0 + k] = __ldg(ipent + (size_t) k * rowstride + r);
}

// Displacement culling of the integration-point lists (as for the atoms): each
// row's entries reordered, those within r_c + CULL_DELTA at the reorder first
// (nnear_row), the rest after; the node positions of the reorder kept as the
// reference.  Launched every step, it returns at once while no node has moved
// (CULL_DELTA - CULL_MARGIN) / 2 since the last reorder; else it reorders from
// this step's packed positions (all referenced sites are computed in such a
// step) and flags the step (eflags[1]).
__global__ void k_ip_reorder(const int *__restrict__ row_start, const int *__restrict__ ent,
                             int nrows, const float4 *__restrict__ ip_q,
                             const float4 *__restrict__ line_pos, Lattice lat, PackGrid pg,
                             float4 lim, int *__restrict__ ent_near, int4 *__restrict__ nnear_row,
                             const float2 *__restrict__ node_hl, long long nvals,
                             float2 *__restrict__ node_ref, unsigned *__restrict__ eflags) {
  if (moved_little(eflags)) return;  // reads eflags[0] only, which no block writes
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    eflags[1] = 1u;
    eflags[2] += 1u;  // reorders so far
  }
  const int stride = gridDim.x * blockDim.x;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += stride) {
    const float4 qi = ip_q[r];
    float cx, cy, cz;
    cell_of(qi, cx, cy, cz);
    const int s0 = row_start[r];
    auto index = [&](int k) { return __ldg(ent + s0 + k); };
    auto rsq = [&](int code) {
      ds x[3];
      line_site(line_pos, code_line(lat, code), frac_of(lat, 1, 2, code_kk(lat, code)), x);
      float dx, dy, dz;
      rel_vec(qi, cx, cy, cz, pack_u(x[0], x[1], x[2], pg), pg.g, dx, dy, dz);
      return dx * dx + dy * dy + dz * dz;
    };
    auto put = [&](int at, int code) { ent_near[s0 + at] = code; };
    auto fetch = [&](int code) { return code; };
    nnear_row[r] = reorder_parts(row_start[r + 1] - s0, lim, index, fetch, rsq, put);
  }
  for (long long t = blockIdx.x * blockDim.x + threadIdx.x; t < nvals; t += stride)
    node_ref[t] = node_hl[t];
}

// FP64 cutoff test of a guard-band pair from the double-single positions: the
// integration point's (ip_h + ip_l) and the site's (line data, relative to l0)
// (arguments by value: a reference to the kernel's arrays would put them in
// local memory on every iteration of the caller's loop)
__device__ __noinline__ bool inside_band_pt(float4 h, float4 l, PackGrid pg, double cutsq,
                                            float x0h, float x0l, float x1h, float x1l,
                                            float x2h, float x2l) {
  const double lx = (double) pg.l0h[0] + pg.l0l[0];
  const double ly = (double) pg.l0h[1] + pg.l0l[1];
  const double lz = (double) pg.l0h[2] + pg.l0l[2];
  const double dx = (((double) h.x + l.x) - lx) - ((double) x0h + x0l);
  const double dy = (((double) h.y + l.y) - ly) - ((double) x1h + x1l);
  const double dz = (((double) h.z + l.z) - lz) - ((double) x2h + x2l);
  return dx * dx + dy * dy + dz * dz < cutsq;
}

__device__ __forceinline__ bool inside_band(const float4 *__restrict__ ip_h,
                                            const float4 *__restrict__ ip_l, PackGrid pg,
                                            double cutsq, int r, float x0h, float x0l, float x1h,
                                            float x1l, float x2h, float x2l) {
  return inside_band_pt(__ldg(ip_h + r), __ldg(ip_l + r), pg, cutsq, x0h, x0l, x1h, x1l, x2h,
                        x2l);
}

// G lanes per integration point, each taking every G-th entry of the row's
// list; the lanes' sums meet by shuffles.  DENSITY: node rows -> erho (EAM);
// otherwise rows of nonzero weight -> forces (LJ or EAM).  Every scanned entry
// is a line code: the site is formed from its lattice line (double-single,
// then packed), tested in FP32, and in the guard band in FP64 on the
// double-single positions.
template <bool EAM, bool DENSITY, int G>
__global__ void __launch_bounds__(512, 2)
k_ipg(ElemArgs a, const float4 *__restrict__ tab, int nr, float rdr, float lj1, float lj2,
      double *__restrict__ out, float2 *__restrict__ outf) {
  extern __shared__ float4 s_tab[];
  const int ntab = EAM ? (DENSITY ? (nr + 1) : FTAB_W * (nr + 1)) : 0;
  for (int m = threadIdx.x; m < ntab; m += blockDim.x) s_tab[m] = tab[m];
  __syncthreads();
  const float g = a.pg.g;
  constexpr int GPW = 32 / G;  // groups per warp
  const int lane = threadIdx.x & (G - 1), gsub = (threadIdx.x & 31) / G;
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  const int nitems = DENSITY ? a.nlocal_e * NPE : a.nforce;
  const int level = a.nnear_row ? cull_level(a.eflags) : 4;
  // warp-uniform trip count: every lane reaches the shuffles
  for (int wb = warp * GPW; wb < nitems; wb += nwarps * GPW) {
    const int it = wb + gsub;
    int r = 0, e = 0, n = 0;
    bool live = it < nitems;
    if (live) {
      if (DENSITY) {
        e = it / NPE;
        r = a.row_first[e] + a.node_list[a.etype[e] * NPE + it % NPE];
      } else {
        r = a.rows[it];  // rows of nonzero weight only; the others stay zero
        e = a.row_elem[r];
        if (a.skip && a.skip[e]) live = false;  // nodal forces from the surrogate
      }
    }
    int s0 = 0;
    float4 qi = make_float4(0.f, 0.f, 0.f, 0.f);
    float fpi = 0.f;
    if (live) {
      s0 = a.row_start[r];
      n = level < 4 ? culled_count(level, a.nnear_row[r], 0) : a.row_start[r + 1] - s0;
      qi = __ldg(a.ip_q + r);
      if (EAM && !DENSITY) fpi = __ldg(a.row_fp + r);
    }
    float cx, cy, cz;
    cell_of(qi, cx, cy, cz);
    dsacc acc, fx, fy, fz;
    float part = 0.f, px = 0.f, py = 0.f, pz = 0.f;
    int cn = 0, cnt = 0;
    if (lane < n) cn = __ldg(a.ent + s0 + lane);
    for (int k = lane; k < n; k += G) {
      const int code = cn;
      if (k + G < n) cn = __ldg(a.ent + s0 + k + G);  // the next entry's code in flight
      // the site from its lattice line: (line data, kk) -> double-single -> packed
      const ds c = frac_of(a.lat, 1, 2, code_kk(a.lat, code));
      ds x[3];
      line_site(a.line_pos, code_line(a.lat, code), c, x);
      const float4 qj = pack_u(x[0], x[1], x[2], a.pg);
      float dx, dy, dz;
      rel_vec(qi, cx, cy, cz, qj, g, dx, dy, dz);
      const float rsq = dx * dx + dy * dy + dz * dz;
      bool in = rsq < a.cutsq_f;
      if (rsq >= a.band_lo && rsq <= a.band_hi)
        in = inside_band(a.ip_h, a.ip_l, a.pg, a.cutsq, r, x[0].h, x[0].l, x[1].h, x[1].l,
                         x[2].h, x[2].l);
      if (in) {
        if (EAM) {
          const float recip = rsqrtf(rsq);
          const float rr = rsq * recip;
          float p;
          const int m = findex(rr, rdr, nr, p);
          if (DENSITY) {
            const float4 c = s_tab[m];
            part += ((c.x * p + c.y) * p + c.z) * p + c.w;
          } else {
            // the site's density from its nodal-density line, then F'
            const float2 lr = __ldg(a.line_rho + code_line(a.lat, code));
            const float fpj = fprime32(lr.x + c.h * lr.y, a.fp4, a.nrho, a.rdrho);
            float rhoip, z2, z2p;
            force_spline(s_tab, m, p, rdr, rhoip, z2, z2p);
            const float phi = z2 * recip;
            const float phip = z2p * recip - phi * recip;
            const float psip = (fpi + fpj) * rhoip + phip;
            const float fpair = -psip * recip;
            px += dx * fpair;
            py += dy * fpair;
            pz += dz * fpair;
          }
        } else {
          const float r2inv = __frcp_rn(rsq);
          const float r6inv = r2inv * r2inv * r2inv;
          const float fpair = r6inv * (lj1 * r6inv - lj2) * r2inv;
          px += dx * fpair;
          py += dy * fpair;
          pz += dz * fpair;
        }
        if ((++cnt & (CHUNK - 1)) == 0) {
          acc.add(part);
          fx.add(px);
          fy.add(py);
          fz.add(pz);
          part = px = py = pz = 0.f;
        }
      }
    }
    if (DENSITY) {
      acc.add(part);
      group_sum<G>(acc);
      if (live && lane == 0) out[NPE * (size_t) e + it % NPE] = acc.value();
    } else {
      fx.add(px);
      fy.add(py);
      fz.add(pz);
      group_sum<G>(fx);
      group_sum<G>(fy);
      group_sum<G>(fz);
      if (live && lane == 0) {  // double-single: the nodal gather reads it without FP64
        outf[3 * r] = make_float2(fx.h, fx.l);
        outf[3 * r + 1] = make_float2(fy.h, fy.l);
        outf[3 * r + 2] = make_float2(fz.h, fz.l);
      }
    }
  }
}

// Nodal forces f_q = sum_r w_r N_q(r) f_r (the FP64 gather's formula) from the
// double-single row forces, with the products w_r N_q(r) as FP32 and the sum
// as a double-single: no FP64 instruction but the final conversion
__global__ void k_gather_nodef_ds(const float2 *__restrict__ fipf, const int *__restrict__ etype,
                                  const int *__restrict__ row_first, const int *__restrict__ numint,
                                  const int *__restrict__ int_off, const float *__restrict__ wn,
                                  int nlocal_e, double *__restrict__ nodef) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  if (tid >= nlocal_e * 24) return;
  const int e = tid / 24, rem = tid % 24, q = rem / 3, c = rem % 3;
  const int ty = etype[e], nint = numint[ty], r0 = row_first[e];
  const float *w = wn + (size_t) int_off[ty] * NPE;
  dsacc acc;
  for (int jj = 0; jj < nint; jj++) {
    const float wq = __ldg(w + jj * NPE + q);
    if (wq == 0.f) continue;  // rows of zero weight carry no force
    const float2 f = fipf[3 * (r0 + jj) + c];
    acc.add(__fmul_rn(wq, f.x));
    acc.add(__fmul_rn(wq, f.y));
  }
  nodef[tid] = acc.value();
}

// ---- fused element passes (self-contained elements) ----
//
// When every list entry of an element's rows references a site of that same
// element (the reference's element lists are then empty: no element centre
// lies within another's neighbor stencil, element_neighbor.cpp:11-75), every
// pair of the element's rows lies inside the element, and one warp evaluates
// the element whole, without forming a site position.  The element's
// trilinear map in its lattice fractions (a, b, c) = (i, j, k) / (n - 1) is
//   x(a, b, c) = x0 + Ka a + Kb b + Kc c + Kab ab + Kac ac + Kbc bc + Kabc abc
// (Ka = x1 - x0, Kb = x3 - x0, Kc = x4 - x0, Kab = x0 - x1 + x2 - x3, ...,
// shape functions of element.cpp:1340-1347); the warp keeps the seven
// coefficient vectors as FP32, from the double-single nodes.  The pair vector
// of a row's point p and a site s is sum_m Km (m(p) - m(s)), the monomial
// differences formed from the integer lattice-index differences: FP32
// roundings of a few 1e-7 A per pair (the coefficients' own roundings deform
// the element smoothly, by about 1e-6 A over its length).  The nodal
// densities enter the same way (rho(a, b, c) with scalar coefficients).
// Pairs whose FP32 squared distance falls in the 1e-4 guard band around the
// cutoff are decided in FP64 from the FP64 nodes and shape functions
// (Spa_inter_ele, Spa_int), so the set of interacting pairs is the FP64 set.
// Sums: FP32 over chunks of 8 pairs, double-single across chunks and lanes;
// F'(rho) of the rows in FP64 (k_row_fp), of the sites in FP32.
constexpr int FG = 4;           // lanes per row: 8 rows per warp
constexpr int FUSED_MAXF = 32;  // rows of nonzero weight per type, at most
constexpr int FUSED_BLOCK = 512;

struct FusedArgs {
  const float2 *node_hl;       // split nodes of this step
  const double *nodex;         // FP64 nodes (guard-band decisions)
  const int *etype, *row_first, *node_list, *int_off, *inter_off;
  const int4 *intp;            // lattice indices (i, j, k) of every type's rows
  const float2 *spa_int_hl;    // the rows' shape functions as double-single pairs
  const float2 *frho_ds;       // F' spline c0..c2 per knot as double-single pairs
  float2 rdrho_ds;             // 1 / drho as a double-single pair
  const double *spa_int;       // FP64 shape functions of the rows
  const double *spa_inter;     // FP64 shape functions of the sites
  const int *fjj, *fjj_off;    // per type: the rows of nonzero weight, ascending
  const float *wn;             // weight x shape function per row and node
  const float *wnf;            // the same for the rows of nonzero weight, per type in order
  const int *row_start, *ent;  // row-major line codes, culling parts in order
  const int4 *nnear_row;
  const unsigned *eflags;
  int nlocal_e, maxlines;
  float cutsq_f, band_lo, band_hi;
  double cutsq;
  const unsigned char *skip;   // elements the surrogate evaluates
  int *band;                   // the guard-band list (band_list)
  int e_begin, e_end;          // the elements of this launch (the exact pass: the list)
  const float4 *lat_rec;       // per type 1/(n_a-1), 1/(n_b-1), 1/(n_c-1), 1/n_b
  Lattice lat;
  const float4 *fp4;           // FP32 F' spline (sites)
  int nrho;
  float rdrho;
  const double *frho;          // FP64 F spline (rows)
  double rdrho64;
};

// The trilinear coefficient vectors of the element, m = a, b, c, ab, ac, bc,
// abc (lanes 0..20: m = lane / 3, axis d = lane % 3), K_a = x1 - x0,
// K_b = x3 - x0, K_c = x4 - x0, K_ab = x0 - x1 + x2 - x3, K_ac = x0 - x1 + x5 -
// x4, K_bc = x0 - x3 + x7 - x4, K_abc = x1 - x0 + x3 - x2 + x4 - x5 + x6 - x7,
// and the nodal-density coefficients likewise (rho_0, then the same seven
// monomials), as signed sums over the 8 nodes in node order: bit k of byte m
// of POS / NEG marks node k added / subtracted.  Every lane runs the same
// eight double-single additions (no divergent cases).
constexpr unsigned long long COEF_POS = 0x5A81210510080200ull;  // bytes: a b c ab ac bc abc
constexpr unsigned long long COEF_NEG = 0xA518120A01010100ull;
constexpr unsigned long long RHO_POS = 0x5A81210510080201ull;   // bytes: 0 a b c ab ac bc abc
constexpr unsigned long long RHO_NEG = 0xA518120A01010100ull;

__device__ __forceinline__ ds signed_node_sum(const float2 *v, int stride, unsigned pos,
                                              unsigned neg) {
  ds s = ds{0.f, 0.f};
#pragma unroll
  for (int k = 0; k < NPE; k++) {
    const float sg = (float) ((int) ((pos >> k) & 1u) - (int) ((neg >> k) & 1u));
    const float2 x = v[stride * k];
    s = ds_add(s, ds{sg * x.x, sg * x.y});
  }
  return s;
}

// K from the double-single nodes staged in the warp's shared memory
// (s_nx[3 k + d]): s_k[3 m + d] (kept in registers), or with by_axis
// s_k[8 d + m] (read from shared memory as two float4 per axis)
__device__ __forceinline__ void fused_coeffs(const float2 *s_nx, int lane, float *s_k,
                                             bool by_axis) {
  if (lane < 21) {
    const int m = lane / 3, d = lane % 3;
    const ds v = signed_node_sum(s_nx + d, 3, (unsigned) (COEF_POS >> (8 * (m + 1))) & 0xFFu,
                                 (unsigned) (COEF_NEG >> (8 * (m + 1))) & 0xFFu);
    s_k[by_axis ? 8 * d + m : lane] = v.h + v.l;
  }
}

// a 16-byte shared-memory load that the compiler keeps inside the loop
__device__ __forceinline__ float4 lds_v4(const float4 *p) {
  float4 v;
  asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "r"((unsigned) __cvta_generic_to_shared(p)));
  return v;
}

// F'(rho) at a row, rho = sum_k N_k erho_k, as fprime64 forms it (pair_eam.cpp:
// 1090-1100, knot index, clamps, cubic) in double-single FP32 arithmetic from
// the double-single shape functions, nodal densities (erds) and spline
// coefficients: the FP32 value of the FP64 result, without an FP64
// instruction (also *rho32, rho rounded to FP32)
__device__ __forceinline__ float row_fprime_ds(const float2 *__restrict__ N,
                                               const float2 *__restrict__ erds,
                                               const float2 *__restrict__ c3, int nrho,
                                               float2 rdrho, float &rho32) {
  ds rho = ds{0.f, 0.f};
#pragma unroll
  for (int k = 0; k < NPE; k++)
    rho = ds_madd(ds{N[k].x, N[k].y}, ds{erds[k].x, erds[k].y}, rho);
  rho32 = rho.h + rho.l;
  return fprime_ds(rho, c3, nrho, rdrho);
}

// FP64 cutoff decision of a guard-band pair: the row's point and the site from
// the FP64 nodes and shape functions
__device__ __noinline__ bool fused_band64(const double *N, const double *M, const double *x,
                                          double cutsq) {
  double rsq = 0.0;
#pragma unroll
  for (int d = 0; d < 3; d++) {
    double p = 0.0, q = 0.0;
#pragma unroll
    for (int k = 0; k < NPE; k++) {
      p += N[k] * x[3 * k + d];
      q += M[k] * x[3 * k + d];
    }
    rsq += (p - q) * (p - q);
  }
  return rsq < cutsq;
}

// lattice geometry of a type as the kernels use it
struct FusedLat {
  int nay, naz;
  float ia, ib, ic;     // 1 / (n - 1) per axis
  float inay;           // 1 / nay, for the line's (ii, jj)
};

// one row of the element, FG lanes: the scan of its culled list, pair vectors
// from the coefficient vectors k (registers) and the row's lattice indices
// F'(rho) from the FP32 coefficient table in shared memory (fprime32's arithmetic)
__device__ __forceinline__ float fprime32_s(float rho, const float4 *s_fp, int nrho, float rdrho) {
  float p = rho * rdrho + 1.0f;
  int m = (int) p;
  m = m < nrho - 1 ? m : nrho - 1;
  m = 1 > m ? 1 : m;
  p -= (float) m;
  p = fminf(p, 1.0f);
  const float4 c = s_fp[m];
  return (c.x * p + c.y) * p + c.z;
}

// V = 0: coefficients in registers; V = 1: read from shared memory (sk4:
// two float4 per axis, then the density coefficients) at every entry, fewer
// registers; V = 2: as 1, two entries in flight per lane.
// EXACT: a pair in the guard band is decided in FP64 (fused_band64) in the
// loop; otherwise the loop only reports that it met one (the return value):
// the caller lists the element for the exact pass, and the call with its
// register saves stays out of the common case's loop
template <bool EAM, bool DENSITY, int V, bool EXACT>
__device__ __forceinline__ bool fused_row(const FusedArgs &a, const FusedLat &g, int e, int rfirst,
                                          int ty, int jj, int level, int glane, const float (&k)[21],
                                          const float (&rk)[8], const float4 *sk4,
                                          const float4 *s_tab, const float4 *s_fp, int nr,
                                          float rdr, float fpi, float lj1, float lj2, bool live,
                                          dsacc &acc, dsacc &fx, dsacc &fy, dsacc &fz) {
  int n = 0, s0 = 0;
  int ip = 0, jp = 0, kp = 0;
  if (live) {
    const int r = rfirst + jj;
    s0 = a.row_start[r];
    n = level < 4 ? culled_count(level, a.nnear_row[r], 0) : a.row_start[r + 1] - s0;
    const int4 q = a.intp[a.int_off[ty] + jj];
    ip = q.x;
    jp = q.y;
    kp = q.z;
  }
  const float ap = (float) ip * g.ia, bp = (float) jp * g.ib, cp = (float) kp * g.ic;
  const float abp = ap * bp;
  const int lbase = e * a.maxlines;
  float part = 0.f, px = 0.f, py = 0.f, pz = 0.f;
  int cn = 0, cnt = 0;
  bool band = false;
  if (glane < n) cn = __ldg(a.ent + s0 + glane);
#pragma unroll(V == 2 ? 2 : 1)
  for (int t = glane; t < n; t += FG) {
    const int code = cn;
    if (t + FG < n) cn = __ldg(a.ent + s0 + t + FG);
    const int L = code_line(a.lat, code) - lbase, kk = code_kk(a.lat, code);
    const int ii = (int) (((float) L + 0.5f) * g.inay);
    const int js = L - ii * g.nay;
    // monomial differences m(p) - m(s)
    const float da = (float) (ip - ii) * g.ia, db = (float) (jp - js) * g.ib,
                dc = (float) (kp - kk) * g.ic;
    const float dab = fmaf(ap, db, fmaf(bp, da, -da * db));
    const float dac = fmaf(ap, dc, fmaf(cp, da, -da * dc));
    const float dbc = fmaf(bp, dc, fmaf(cp, db, -db * dc));
    const float dabc = fmaf(abp, dc, fmaf(cp, dab, -dab * dc));
    float v[3];
    if (V == 0) {
#pragma unroll
      for (int d = 0; d < 3; d++) {
        float w = k[d] * da;
        w = fmaf(k[3 + d], db, w);
        w = fmaf(k[6 + d], dc, w);
        w = fmaf(k[9 + d], dab, w);
        w = fmaf(k[12 + d], dac, w);
        w = fmaf(k[15 + d], dbc, w);
        v[d] = fmaf(k[18 + d], dabc, w);
      }
    } else {
#pragma unroll
      for (int d = 0; d < 3; d++) {
        const float4 c0 = lds_v4(sk4 + 2 * d), c1 = lds_v4(sk4 + 2 * d + 1);
        float w = c0.x * da;
        w = fmaf(c0.y, db, w);
        w = fmaf(c0.z, dc, w);
        w = fmaf(c0.w, dab, w);
        w = fmaf(c1.x, dac, w);
        w = fmaf(c1.y, dbc, w);
        v[d] = fmaf(c1.z, dabc, w);
      }
    }
    const float dx = v[0], dy = v[1], dz = v[2];
    const float rsq = dx * dx + dy * dy + dz * dz;
    bool in = rsq < a.cutsq_f;
    if (rsq >= a.band_lo && rsq <= a.band_hi) {
      if (EXACT)
        in = fused_band64(a.spa_int + ((size_t) a.int_off[ty] + jj) * NPE,
                          a.spa_inter + ((size_t) a.inter_off[ty] + L * g.naz + kk) * NPE,
                          a.nodex + 24 * (size_t) e, a.cutsq);
      else
        band = true;
    }
    if (in) {
      if (EAM) {
        const float recip = rsqrtf(rsq);
        const float rr = rsq * recip;
        float p;
        const int m = findex(rr, rdr, nr, p);
        if (DENSITY) {
          const float4 cc = s_tab[m];
          part += ((cc.x * p + cc.y) * p + cc.z) * p + cc.w;
        } else {
          // the site's density from the nodal densities: rho(p) - sum Rm (m(p) - m(s))
          float dr;
          if (V == 0) {
            dr = rk[1] * da;
            dr = fmaf(rk[2], db, dr);
            dr = fmaf(rk[3], dc, dr);
            dr = fmaf(rk[4], dab, dr);
            dr = fmaf(rk[5], dac, dr);
            dr = fmaf(rk[6], dbc, dr);
            dr = fmaf(rk[7], dabc, dr);
          } else {
            const float4 r0 = lds_v4(sk4 + 6), r1 = lds_v4(sk4 + 7);
            dr = r0.y * da;
            dr = fmaf(r0.z, db, dr);
            dr = fmaf(r0.w, dc, dr);
            dr = fmaf(r1.x, dab, dr);
            dr = fmaf(r1.y, dac, dr);
            dr = fmaf(r1.z, dbc, dr);
            dr = fmaf(r1.w, dabc, dr);
          }
          const float fpj = fprime32_s(rk[0] - dr, s_fp, a.nrho, a.rdrho);
          float rhoip, z2, z2p;
          force_spline(s_tab, m, p, rdr, rhoip, z2, z2p);
          const float phi = z2 * recip;
          const float phip = z2p * recip - phi * recip;
          const float psip = (fpi + fpj) * rhoip + phip;
          const float fpair = -psip * recip;
          px += dx * fpair;
          py += dy * fpair;
          pz += dz * fpair;
        }
      } else {
        const float r2inv = __frcp_rn(rsq);
        const float r6inv = r2inv * r2inv * r2inv;
        const float fpair = r6inv * (lj1 * r6inv - lj2) * r2inv;
        px += dx * fpair;
        py += dy * fpair;
        pz += dz * fpair;
      }
      if ((++cnt & (CHUNK - 1)) == 0) {  // the pass's own sums only
        if (DENSITY) {
          acc.add(part);
          part = 0.f;
        } else {
          fx.add(px);
          fy.add(py);
          fz.add(pz);
          px = py = pz = 0.f;
        }
      }
    }
  }
  if (DENSITY) {
    acc.add(part);
    group_sum<FG>(acc);
  } else {
    fx.add(px);
    fy.add(py);
    fz.add(pz);
    group_sum<FG>(fx);
    group_sum<FG>(fy);
    group_sum<FG>(fz);
  }
  return band;
}

// the type's lattice sizes and their reciprocals (from the host's table: no
// division per element)
__device__ __forceinline__ FusedLat fused_lat(const Lattice &lat, const float4 *rec, int ty) {
  FusedLat g;
  g.nay = __ldg(lat.nae + 3 * ty + 1);
  g.naz = __ldg(lat.nae + 3 * ty + 2);
  const float4 r = __ldg(rec + ty);
  g.ia = r.x;
  g.ib = r.y;
  g.ic = r.z;
  g.inay = r.w;
  return g;
}

// per-warp shared memory: coefficient vectors (21), density coefficients (8),
// row forces (3 per row of nonzero weight), then the element's staged nodes
// (24 float2) and nodal densities (8 double-single float2)
constexpr int FUSED_WARP_FLOATS = 32 + 2 * 3 * FUSED_MAXF + 48 + 16;
constexpr int FUSED_NX_AT = 32 + 2 * 3 * FUSED_MAXF, FUSED_ER_AT = FUSED_NX_AT + 48;
static_assert(FUSED_NX_AT % 2 == 0 && FUSED_ER_AT % 2 == 0 && FUSED_WARP_FLOATS % 2 == 0,
              "8-byte alignment of the staged nodes and densities");

// threads per block of each variant (V = 0: coefficients in registers)
__host__ __device__ constexpr int fused_block(int V) { return V == 0 ? FUSED_BLOCK : 768; }

// The guard-band list (a.band: count, blocks done, elements re-run so far,
// then the element indices).  A fused pass lists every element in which some
// pair fell in the guard band; the exact pass (FIX) runs the listed elements
// again with the FP64 decisions, overwriting their outputs, and its last block
// to finish resets the list for the next pass.
constexpr int BAND_LIST = 3;

__device__ __forceinline__ void band_list(int *band, int e, int cap) {
  const int slot = atomicAdd(band, 1);
  if (slot < cap) band[BAND_LIST + slot] = e;
}

__device__ __forceinline__ void band_done(int *band, int ne) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(band + 1, 1) == (int) gridDim.x - 1) {
      band[2] += ne;
      band[0] = 0;
      band[1] = 0;
    }
  }
}

// EAM nodal densities: the element's 8 node rows, one row per FG lanes
// (FIX: the listed elements, guard-band pairs decided in FP64)
template <int V, bool FIX>
__global__ void __launch_bounds__(fused_block(V), 1)
k_elem_rho_fused(FusedArgs a, const float4 *__restrict__ tab, int nr, float rdr,
                 double *__restrict__ erho) {
  const int ne = FIX ? min(a.band[0], a.nlocal_e) : a.e_end - a.e_begin;
  if (FIX && ne == 0) return;  // the whole grid (the count is the same for every block)
  extern __shared__ float4 smem[];
  float4 *s_tab = smem;
  for (int m = threadIdx.x; m <= nr; m += blockDim.x) s_tab[m] = tab[m];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *s_k = reinterpret_cast<float *>(smem + nr + 1) + (size_t) w * FUSED_WARP_FLOATS;
  __syncthreads();
  const int gw = (int) (((long long) blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nw = (int) (((long long) gridDim.x * blockDim.x) >> 5);
  const int level = a.nnear_row ? cull_level(a.eflags) : 4;
  const int gsub = lane / FG, glane = lane % FG;
  const float rk[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  float2 *s_nx = reinterpret_cast<float2 *>(s_k + FUSED_NX_AT);
  // the next element's nodes, type and first row are loaded while this
  // element's rows run
  float2 pn = make_float2(0.f, 0.f);
  int pty = 0, prf = 0, pe = a.e_begin + gw;
  if (gw < ne) {
    if (FIX) pe = a.band[BAND_LIST + gw];
    if (lane < 24) pn = __ldg(a.node_hl + 24 * (size_t) pe + lane);
    pty = __ldg(a.etype + pe);
    prf = __ldg(a.row_first + pe);
  }
  for (int i = gw; i < ne; i += nw) {
    const int e = FIX ? pe : a.e_begin + i, ty = pty, rfirst = prf;
    if (lane < 24) s_nx[lane] = pn;
    const int in = i + nw;
    if (in < ne) {
      const int en = FIX ? a.band[BAND_LIST + in] : a.e_begin + in;
      if (FIX) pe = en;
      if (lane < 24) pn = __ldg(a.node_hl + 24 * (size_t) en + lane);
      pty = __ldg(a.etype + en);
      prf = __ldg(a.row_first + en);
    }
    const FusedLat g = fused_lat(a.lat, a.lat_rec, ty);
    __syncwarp();
    fused_coeffs(s_nx, lane, s_k, V != 0);
    __syncwarp();
    float k[21];
    if (V == 0) {
#pragma unroll
      for (int q = 0; q < 21; q++) k[q] = s_k[q];
    }
    bool band = false;
    for (int kb = 0; kb < NPE; kb += 32 / FG) {
      const int q = kb + gsub;
      const bool live = q < NPE;
      const int jj = live ? a.node_list[ty * NPE + q] : 0;
      dsacc acc, fx, fy, fz;
      band |= fused_row<true, true, V, FIX>(a, g, e, rfirst, ty, jj, level, glane, k, rk,
                                            reinterpret_cast<const float4 *>(s_k), s_tab, nullptr,
                                            nr, rdr, 0.f, 0.f, 0.f, live, acc, fx, fy, fz);
      if (live && glane == 0) erho[NPE * (size_t) e + q] = acc.value();
    }
    if (!FIX && __any_sync(0xffffffffu, band) && lane == 0) band_list(a.band, e, a.nlocal_e);
    __syncwarp();
  }
  if (FIX) band_done(a.band, ne);
}

// Forces of the element's rows of nonzero weight and their gather onto the
// nodes (EAM with the nodal densities and row F'(rho), or LJ)
// (FIX: the listed elements, guard-band pairs decided in FP64)
template <bool EAM, int V, bool FIX>
__global__ void __launch_bounds__(fused_block(V), 1)
k_elem_force_fused(FusedArgs a, const float4 *__restrict__ tab, int nr, float rdr, float lj1,
                   float lj2, const double *__restrict__ erho, double *__restrict__ nodef) {
  const int ne = FIX ? min(a.band[0], a.nlocal_e) : a.e_end - a.e_begin;
  if (FIX && ne == 0) return;  // the whole grid (the count is the same for every block)
  extern __shared__ float4 smem[];
  float4 *s_tab = smem;
  const int ntab = EAM ? FTAB_W * (nr + 1) : 0;
  const int nfp = EAM ? a.nrho + 1 : 0;
  float4 *s_fp = smem + ntab;
  for (int m = threadIdx.x; m < ntab; m += blockDim.x) s_tab[m] = tab[m];
  for (int m = threadIdx.x; m < nfp; m += blockDim.x) s_fp[m] = a.fp4[m];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float *s_k = reinterpret_cast<float *>(smem + ntab + nfp) + (size_t) w * FUSED_WARP_FLOATS;
  float *s_r = s_k + 24;
  float2 *s_f = reinterpret_cast<float2 *>(s_k + 32);
  __syncthreads();
  const int gw = (int) (((long long) blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int nw = (int) (((long long) gridDim.x * blockDim.x) >> 5);
  const int level = a.nnear_row ? cull_level(a.eflags) : 4;
  const int gsub = lane / FG, glane = lane % FG;
  float2 *s_nx = reinterpret_cast<float2 *>(s_k + FUSED_NX_AT);
  float2 *s_erds = reinterpret_cast<float2 *>(s_k + FUSED_ER_AT);  // nodal densities, ds
  // the next element's nodes, type and first row are loaded while this
  // element's rows run
  float2 pn = make_float2(0.f, 0.f);
  int pty = 0, prf = 0, pe = a.e_begin + gw;
  if (gw < ne) {
    if (FIX) pe = a.band[BAND_LIST + gw];
    if (lane < 24) pn = __ldg(a.node_hl + 24 * (size_t) pe + lane);
    pty = __ldg(a.etype + pe);
    prf = __ldg(a.row_first + pe);
  }
  for (int i = gw; i < ne; i += nw) {
    const int e = FIX ? pe : a.e_begin + i, ty = pty, rfirst = prf;
    const float2 cn = pn;
    const int in = i + nw;
    if (in < ne) {
      const int en = FIX ? a.band[BAND_LIST + in] : a.e_begin + in;
      if (FIX) pe = en;
      if (lane < 24) pn = __ldg(a.node_hl + 24 * (size_t) en + lane);
      pty = __ldg(a.etype + en);
      prf = __ldg(a.row_first + en);
    }
    if (a.skip && a.skip[e]) continue;  // nodal forces from the surrogate (warp-uniform)
    if (lane < 24) s_nx[lane] = cn;
    else if (EAM) {
      const ds d = ds_of_double(__ldg(erho + NPE * (size_t) e + (lane - 24)));
      s_erds[lane - 24] = make_float2(d.h, d.l);
    }
    const FusedLat g = fused_lat(a.lat, a.lat_rec, ty);
    const int f0 = a.fjj_off[ty], nf = a.fjj_off[ty + 1] - f0;
    __syncwarp();
    if (EAM) {
      // the coefficient vectors (lanes 0-20, as fused_coeffs) and the
      // nodal-density coefficients (lanes 24-31; FP32, formed in double-single
      // from the doubles' bits: no FP64 instruction) in one pass: the same
      // eight double-single additions from different sources
      const bool dens = lane >= 24;
      if (lane < 21 || dens) {
        const int m = dens ? lane - 24 : lane / 3, d = lane % 3;
        const unsigned long long pm = dens ? RHO_POS : COEF_POS, nm = dens ? RHO_NEG : COEF_NEG;
        const int sh = dens ? 8 * m : 8 * (m + 1);
        const ds v = signed_node_sum(dens ? s_erds : s_nx + d, dens ? 1 : 3,
                                     (unsigned) (pm >> sh) & 0xFFu, (unsigned) (nm >> sh) & 0xFFu);
        if (dens) s_r[m] = v.h + v.l;
        else s_k[V != 0 ? 8 * d + m : lane] = v.h + v.l;
      }
    } else {
      fused_coeffs(s_nx, lane, s_k, V != 0);
    }
    __syncwarp();
    float k[21];
    if (V == 0) {
#pragma unroll
      for (int q = 0; q < 21; q++) k[q] = s_k[q];
    }
    float rk[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    bool band = false;
    for (int fb = 0; fb < nf; fb += 32 / FG) {
      const int j = fb + gsub;
      const bool live = j < nf;
      const int jj = live ? a.fjj[f0 + j] : 0;
      float fpi = 0.f;
      if (EAM) {
        // F'(rho) at the row, rho in FP64 from the nodal densities (k_row_fp);
        // the row's density in FP32 for the sites' (rho(p) in rk[0])
        float rho32 = 0.f;
        if (live)  // every lane of the row's group (no shuffle)
          fpi = row_fprime_ds(a.spa_int_hl + ((size_t) a.int_off[ty] + jj) * NPE, s_erds,
                              a.frho_ds, a.nrho, a.rdrho_ds, rho32);
        rk[0] = rho32;
        if (V == 0) {
#pragma unroll
          for (int q = 1; q < 8; q++) rk[q] = s_r[q];
        }
      }
      dsacc acc, fx, fy, fz;
      band |= fused_row<EAM, false, V, FIX>(a, g, e, rfirst, ty, jj, level, glane, k, rk,
                                            reinterpret_cast<const float4 *>(s_k), s_tab, s_fp,
                                            nr, rdr, fpi, lj1, lj2, live, acc, fx, fy, fz);
      if (live && glane == 0) {
        s_f[3 * j] = make_float2(fx.h, fx.l);
        s_f[3 * j + 1] = make_float2(fy.h, fy.l);
        s_f[3 * j + 2] = make_float2(fz.h, fz.l);
      }
    }
    __syncwarp();
    if (lane < 24) {  // the nodal gather (k_gather_nodef_ds), rows in ascending order
      const int q = lane / 3, c = lane % 3;
      const float *wt = a.wnf + (size_t) f0 * NPE + q;
      dsacc acc;
      for (int j = 0; j < nf; j++) {
        const float wq = __ldg(wt + j * NPE);
        if (wq == 0.f) continue;
        const float2 f = s_f[3 * j + c];
        acc.add(__fmul_rn(wq, f.x));
        acc.add(__fmul_rn(wq, f.y));
      }
      nodef[24 * (size_t) e + lane] = acc.value();
    }
    if (!FIX && __any_sync(0xffffffffu, band) && lane == 0) band_list(a.band, e, a.nlocal_e);
    __syncwarp();
  }
  if (FIX) band_done(a.band, ne);
}

// every entry of every row references a site of the row's own element:
// count the entries that do not
__global__ void k_self_check(const int *__restrict__ row_start, const int *__restrict__ ent,
                             const int *__restrict__ row_elem, int nrows, Lattice lat,
                             int maxlines, unsigned long long *__restrict__ foreign) {
  unsigned long long c = 0;
  for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < nrows; r += gridDim.x * blockDim.x) {
    const int e = row_elem[r];
    const long long lo = (long long) e * maxlines, hi = lo + maxlines;
    for (int k = row_start[r]; k < row_start[r + 1]; k++) {
      const long long L = code_line(lat, __ldg(ent + k));
      c += L < lo || L >= hi;
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(foreign, c);
}

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

// SM count x resident blocks, cached per (kernel, block size, shared memory)
int persistent_grid(const void *kernel, int threads, size_t smem, long long work) {
  struct Key {
    const void *k;
    int t;
    size_t m;
    int dev, nsm, occ;
  };
  static thread_local std::vector<Key> cache;
  int dev = 0;
  cudaGetDevice(&dev);
  int nsm = 0, occ = 0;
  bool hit = false;
  for (const Key &c : cache)
    if (c.k == kernel && c.t == threads && c.m == smem && c.dev == dev) {
      nsm = c.nsm;
      occ = c.occ;
      hit = true;
      break;
    }
  if (!hit) {
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    if (smem > 48 * 1024)
      cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kernel, threads, smem);
    cache.push_back(Key{kernel, threads, smem, dev, nsm, occ});
  }
  if (occ < 1) occ = 1;
  long long need = (work + threads - 1) / threads;
  long long g = (long long) nsm * occ;
  return (int) (need < g ? (need > 0 ? need : 1) : g);
}

}  // namespace

PackGrid make_pack_grid(const double l0[3], double g, int *oob) {
  PackGrid pg{};
  for (int d = 0; d < 3; d++) {
    pg.l0h[d] = (float) l0[d];
    pg.l0l[d] = (float) (l0[d] - (double) pg.l0h[d]);
  }
  pg.g = (float) g;
  pg.ig = (float) (1.0 / g);
  pg.oob = oob;
  return pg;
}

void pack_rel(const double4 *x, int n, const PackGrid &pg, float4 *xq, const float4 *ref, int nref,
              unsigned *dmax2, cudaStream_t s) {
  if (n <= 0) return;
  k_pack_rel<<<nblk(n, PACK_BLOCK), PACK_BLOCK, 0, s>>>(x, n, pg, xq, ref, nref, dmax2);
  check(cudaGetLastError(), "pack_rel");
}

void eam_rho_atoms(const MixedAtoms &m, const float4 *rhor_val, const EamTables &e,
                   const float4 *fp4, double *rho, float *fp, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xq, m.qg, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq, m.snum, m.slist, m.nnear, m.dmax2};
  if (m.fprime64) {
    a.frho_ds = m.frho_ds;
    const float h = (float) e.rdrho;
    a.rdrho_ds = make_float2(h, (float) (e.rdrho - (double) h));
  }
  size_t smem = sizeof(float4) * (e.nr + 1);
  int g = persistent_grid((const void *) k_eam_rho_atoms, m.block, smem, m.nlocal);
  k_eam_rho_atoms<<<g, m.block, smem, s>>>(a, rhor_val, e.nr, (float) e.rdr, fp4, e.nrho,
                                           (float) e.rdrho, rho, fp);
  check(cudaGetLastError(), "eam_rho_atoms_mixed");
}

static float4 part_limits(float cut_rsq, float cutoff) {
  const float r1 = cutoff + CULL_D1, r2 = cutoff + CULL_D2, r3 = cutoff + CULL_DELTA;
  return make_float4(cut_rsq, r1 * r1, r2 * r2, r3 * r3);
}

void list_partition(const float4 *xq, float g, const int *num, const int *list, int stride,
                    int nlocal, float cut_rsq, float cutoff, int *out, int4 *nnear, float4 *ref,
                    unsigned *dmax2, unsigned *reorders, cudaStream_t s) {
  if (nlocal <= 0) return;
  const int grid = persistent_grid((const void *) k_list_partition, 256, 0, nlocal);
  k_list_partition<<<grid, 256, 0, s>>>(xq, g, num, list, stride, nlocal,
                                        part_limits(cut_rsq, cutoff), out, nnear, ref, dmax2,
                                        reorders);
  check(cudaGetLastError(), "list_partition");
}

void union_build(const int *num, const int *list, int stride, int nlocal, int *union_j,
                 int *union_n, unsigned short *slot, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_union_build<<<(nlocal + UGROUP - 1) / UGROUP, 256, 0, s>>>(num, list, stride, nlocal, union_j,
                                                             union_n, slot);
  check(cudaGetLastError(), "union_build");
}

int union_max() { return UMAX; }

static int union_grid(const void *k, size_t smem, int nlocal) {
  int ngroups = (nlocal + UGROUP - 1) / UGROUP;
  int need = (ngroups + UWARPS - 1) / UWARPS;
  return std::min(need, persistent_grid(k, UGROUP * UWARPS, smem, (long long) need * UGROUP * UWARPS));
}

void eam_rho_union(const MixedAtoms &m, const int *union_j, const int *union_n,
                   const unsigned short *slot, unsigned short *sslot, const float4 *rhor_val,
                   const EamTables &e, const float4 *fp4, double *rho, float *fp,
                   cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xq, m.qg, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq, m.snum, m.slist, nullptr, nullptr};
  if (m.fprime64) {
    a.frho_ds = m.frho_ds;
    const float h = (float) e.rdrho;
    a.rdrho_ds = make_float2(h, (float) (e.rdrho - (double) h));
  }
  UnionArgs u{union_j, union_n, slot, sslot};
  size_t smem = sizeof(float4) * ((e.nr + 1) + (size_t) UWARPS * UMAX);
  int g = union_grid((const void *) k_eam_rho_union, smem, m.nlocal);
  k_eam_rho_union<<<g, UGROUP * UWARPS, smem, s>>>(a, u, rhor_val, e.nr, (float) e.rdr, fp4,
                                                  e.nrho, (float) e.rdrho, rho, fp);
  check(cudaGetLastError(), "eam_rho_union");
}

void eam_force_union(const MixedAtoms &m, const int *union_j, const int *union_n,
                     const unsigned short *sslot, const float4 *ftab, const EamTables &e,
                     const float *fp, double *f, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xq, m.qg, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq, m.snum, m.slist, nullptr, nullptr};
  UnionArgs u{union_j, union_n, nullptr, const_cast<unsigned short *>(sslot)};
  size_t smem = sizeof(float4) * (FTAB_W * (size_t) (e.nr + 1) + (size_t) UWARPS * UMAX) +
                sizeof(float) * (size_t) UWARPS * UMAX;
  int g = union_grid((const void *) k_eam_force_union, smem, m.nlocal);
  k_eam_force_union<<<g, UGROUP * UWARPS, smem, s>>>(a, u, ftab, e.nr, (float) e.rdr, fp, f);
  check(cudaGetLastError(), "eam_force_union");
}

void eam_force_atoms(const MixedAtoms &m, const float4 *ftab, const EamTables &e,
                     const float *fp, double *f, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xq, m.qg, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq, m.snum, m.slist, nullptr, nullptr};
  size_t smem = sizeof(float4) * FTAB_W * (e.nr + 1);
  int dev = 0, nsm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int block = m.nlocal >= 4LL * nsm * FORCE_BLOCK ? FORCE_BLOCK : m.block;
  int g = persistent_grid((const void *) k_eam_force_atoms, block, smem, m.nlocal);
  k_eam_force_atoms<<<g, block, smem, s>>>(a, ftab, e.nr, (float) e.rdr, fp, f);
  check(cudaGetLastError(), "eam_force_atoms_mixed");
}

void lj_atoms(const MixedAtoms &m, const int *type, const float *lj1, const float *lj2,
              const float *cutsq_t, const double *cutsq64, double *f, cudaStream_t s) {
  if (m.nlocal <= 0) return;
  AtomArgs a{m.x, m.xq, m.qg, m.num, m.list, m.stride, m.nlocal, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq, m.snum, m.slist, nullptr, nullptr};
  int g = persistent_grid((const void *) k_lj_atoms, m.block, 0, m.nlocal);
  k_lj_atoms<<<g, m.block, 0, s>>>(a, type, lj1, lj2, cutsq_t, cutsq64, f);
  check(cudaGetLastError(), "lj_atoms_mixed");
}

void node_split(const double *nodex, int n, float2 *hl, const float2 *ref, unsigned *dmax2,
                cudaStream_t s) {
  if (n <= 0) return;
  k_node_split<<<nblk((long long) n * NPE, SPLIT_BLOCK), SPLIT_BLOCK, 0, s>>>(nodex, n, hl, ref,
                                                                           dmax2);
  check(cudaGetLastError(), "node_split");
}

void lines(const float2 *node_hl, const int *etype, const Lattice &lat, int max_nax,
           const unsigned long long *mask, const unsigned long long *mask_near,
           const unsigned *eflags, int maxlines, const PackGrid &pg, int nelem, float4 *line_pos,
           cudaStream_t s, const unsigned *gate) {
  if (nelem <= 0) return;
  const size_t smem = sizeof(ds) * 12 * (size_t) max_nax * (LCH / 32);
  const int grid = persistent_grid((const void *) k_lines, LCH, smem, (long long) nelem * 32);
  k_lines<<<grid, LCH, smem, s>>>(node_hl, etype, lat, mask, mask_near, eflags, maxlines, pg,
                                  nelem, max_nax, line_pos, gate);
  check(cudaGetLastError(), "lines");
}

void line_rho(const double *erho, const int *etype, const Lattice &lat,
              const unsigned long long *mask, const unsigned long long *mask_near,
              const unsigned *eflags, int maxlines, int nelem, float2 *out, cudaStream_t s) {
  if (nelem <= 0) return;
  const int grid = (nelem + LCH / 32 - 1) / (LCH / 32);
  k_line_rho<<<grid, LCH, 0, s>>>(erho, etype, lat, mask, mask_near, eflags, maxlines, nelem, out);
  check(cudaGetLastError(), "line_rho");
}

void ent_codes(int *ent, long long n, const int *site_base, int nall_e, const int *etype,
               const int *nae, int maxlines, int kb, cudaStream_t s) {
  if (n <= 0) return;
  const int grid = persistent_grid((const void *) k_ent_codes, 256, 0, n);
  k_ent_codes<<<grid, 256, 0, s>>>(ent, n, site_base, nall_e, etype, nae, maxlines, kb);
  check(cudaGetLastError(), "ent_codes");
}

void line_masks(const int *row_start, const int *ent, const int4 *nnear_row, int nrows,
                const Lattice &lat, const unsigned char *isforce, unsigned long long *mask,
                unsigned long long *mask_f, long long nmask, const unsigned *gate,
                cudaStream_t s) {
  if (nrows <= 0 || nmask <= 0) return;
  const int g1 = persistent_grid((const void *) k_masks_clear, 256, 0, nmask);
  k_masks_clear<<<g1, 256, 0, s>>>(mask, mask_f, nmask, gate);
  const int g2 = persistent_grid((const void *) k_masks_or, 256, 0, nrows);
  k_masks_or<<<g2, 256, 0, s>>>(row_start, ent, nnear_row, nrows, lat, isforce, mask, mask_f,
                                gate);
  check(cudaGetLastError(), "line_masks");
}

void count_lines(const unsigned long long *mask, const unsigned long long *mask_f, long long n,
                 unsigned long long *count, cudaStream_t s) {
  check(cudaMemsetAsync(count, 0, 2 * sizeof(unsigned long long), s), "count_lines");
  if (n <= 0) return;
  const int g = persistent_grid((const void *) k_count_lines, 256, 0, n);
  k_count_lines<<<g, 256, 0, s>>>(mask, mask_f, n, count);
  check(cudaGetLastError(), "count_lines");
}

void ip_reorder(const int *row_start, const int *ent, int nrows, const float4 *ip_q,
                const float4 *line_pos, const Lattice &lat, const PackGrid &pg, float cutoff,
                int *ent_near, int4 *nnear_row, const float2 *node_hl, int nall_e,
                float2 *node_ref, unsigned *eflags, cudaStream_t s) {
  if (nrows <= 0) return;
  const int grid = persistent_grid((const void *) k_ip_reorder, 256, 0, nrows);
  k_ip_reorder<<<grid, 256, 0, s>>>(row_start, ent, nrows, ip_q, line_pos, lat, pg,
                                    part_limits(cutoff * cutoff, cutoff), ent_near, nnear_row,
                                    node_hl, (long long) nall_e * 24, node_ref, eflags);
  check(cudaGetLastError(), "ip_reorder");
}

void row_q(const int *row_elem, const int *row_jj, const int *etype, const int *int_off,
           const float2 *spa_int_hl, const float2 *node_hl, int nrows, const PackGrid &pg,
           float4 *ip_q, float4 *ip_h, float4 *ip_l, cudaStream_t s, const unsigned *gate) {
  if (nrows <= 0) return;
  const int grid = persistent_grid((const void *) k_row_q, 128, 0, nrows);
  k_row_q<<<grid, 128, 0, s>>>(row_elem, row_jj, etype, int_off, spa_int_hl, node_hl, nrows, pg,
                               ip_q, ip_h, ip_l, gate);
  check(cudaGetLastError(), "row_q");
}

void row_fp(const int *rows, int nforce, const int *row_elem, const int *row_jj,
            const int *etype, const int *int_off, const double *spa_int, const double *erho,
            const EamTables &e, float *fp, cudaStream_t s) {
  if (nforce <= 0) return;
  k_row_fp<<<nblk(nforce, 128), 128, 0, s>>>(rows, nforce, row_elem, row_jj, etype, int_off,
                                            spa_int, erho, e.frho, e.nrho, e.rdrho, fp);
  check(cudaGetLastError(), "row_fp");
}

void ip_csr(const int *ipnum, const int *ipent, int nrows, int rowstride, const int *row_start,
            int *ent, cudaStream_t s) {
  if (nrows <= 0) return;
  k_ip_csr<<<nblk(nrows, 128), 128, 0, s>>>(ipnum, ipent, nrows, rowstride, row_start, ent);
  check(cudaGetLastError(), "ip_csr");
}

template <bool EAM, bool DENSITY, int G>
static void launch_ipg(const ElemArgs &a, long long items, int block, const float4 *tab,
                       const EamTables &e, float lj1, float lj2, double *out, float2 *outf,
                       cudaStream_t s) {
  const size_t smem = EAM ? sizeof(float4) * (DENSITY ? 1 : FTAB_W) * (e.nr + 1) : 0;
  const int g = persistent_grid((const void *) k_ipg<EAM, DENSITY, G>, block, smem, items * G);
  k_ipg<EAM, DENSITY, G><<<g, block, smem, s>>>(a, tab, e.nr, (float) e.rdr, lj1, lj2, out, outf);
}

template <bool EAM, bool DENSITY>
static void launch_ip(const ElemArgs &a, long long items, int block, int group,
                      const float4 *tab, const EamTables &e, float lj1, float lj2, double *out,
                      float2 *outf, cudaStream_t s) {
  if (group == 4) launch_ipg<EAM, DENSITY, 4>(a, items, block, tab, e, lj1, lj2, out, outf, s);
  else if (group == 16)
    launch_ipg<EAM, DENSITY, 16>(a, items, block, tab, e, lj1, lj2, out, outf, s);
  else launch_ipg<EAM, DENSITY, 8>(a, items, block, tab, e, lj1, lj2, out, outf, s);
}

void ip_pass(const MixedElems &m, int pass, const float4 *tab, const EamTables &e, float lj1,
             float lj2, double *out, float2 *outf, cudaStream_t s) {
  ElemArgs a{m.line_pos, m.line_rho, m.fp4, m.nrho, m.rdrho, m.ip_q, m.ip_h, m.ip_l,
             m.row_fp, m.etype, m.row_elem, m.row_first, m.node_list, m.row_start, m.ent,
             m.nnear_row, m.eflags, m.nlocal_e, m.rows, m.nforce, m.cutsq_f, m.band_lo,
             m.band_hi, m.cutsq, m.skip, m.lat, m.pg};
  if (pass == 0)  // LJ forces
    launch_ip<false, false>(a, m.nforce, m.block, m.group, tab, e, lj1, lj2, out, outf, s);
  else if (pass == 1)  // EAM nodal densities
    launch_ip<true, true>(a, (long long) m.nlocal_e * NPE, m.block, m.group, tab, e, 0.f, 0.f, out,
                          outf, s);
  else  // EAM forces
    launch_ip<true, false>(a, m.nforce, m.block, m.group, tab, e, 0.f, 0.f, out, outf, s);
  check(cudaGetLastError(), "ip_pass_mixed");
}

template <int V>
static void launch_fused(const FusedArgs &a, int pass, const float4 *tab, const EamTables &e,
                         size_t table, float lj1, float lj2, const double *erho_in,
                         double *erho_out, double *nodef, cudaStream_t s) {
  constexpr int B = fused_block(V);
  const size_t smem = table + sizeof(float) * FUSED_WARP_FLOATS * (B / 32);
  const long long items = (long long) (a.e_end - a.e_begin) * 32;
  // the pass, then the exact pass over the elements it listed (a grid of the
  // same shape; it returns at once when the list is empty)
  if (pass == 1) {
    const int g = persistent_grid((const void *) k_elem_rho_fused<V, false>, B, smem, items);
    k_elem_rho_fused<V, false><<<g, B, smem, s>>>(a, tab, e.nr, (float) e.rdr, erho_out);
    persistent_grid((const void *) k_elem_rho_fused<V, true>, B, smem, items);
    k_elem_rho_fused<V, true><<<g, B, smem, s>>>(a, tab, e.nr, (float) e.rdr, erho_out);
  } else if (pass == 2) {
    const int g =
        persistent_grid((const void *) k_elem_force_fused<true, V, false>, B, smem, items);
    k_elem_force_fused<true, V, false><<<g, B, smem, s>>>(a, tab, e.nr, (float) e.rdr, 0.f, 0.f,
                                                          erho_in, nodef);
    persistent_grid((const void *) k_elem_force_fused<true, V, true>, B, smem, items);
    k_elem_force_fused<true, V, true><<<g, B, smem, s>>>(a, tab, e.nr, (float) e.rdr, 0.f, 0.f,
                                                         erho_in, nodef);
  } else {
    const int g =
        persistent_grid((const void *) k_elem_force_fused<false, V, false>, B, smem, items);
    k_elem_force_fused<false, V, false><<<g, B, smem, s>>>(a, nullptr, 0, 0.f, lj1, lj2, nullptr,
                                                           nodef);
    persistent_grid((const void *) k_elem_force_fused<false, V, true>, B, smem, items);
    k_elem_force_fused<false, V, true><<<g, B, smem, s>>>(a, nullptr, 0, 0.f, lj1, lj2, nullptr,
                                                          nodef);
  }
}

bool fused_fits(int nr, int nrho) {
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t need = sizeof(float4) * (FTAB_W * (size_t) (nr + 1) + (size_t) (nrho + 1)) +
                      sizeof(float) * FUSED_WARP_FLOATS * (fused_block(2) / 32);
  return need <= (size_t) optin;
}

void elem_fused(const MixedElems &m, const FusedTables &t, int pass, const float4 *tab,
                const EamTables &e, float lj1, float lj2, const double *erho_in, double *erho_out,
                double *nodef, cudaStream_t s, int e_begin, int e_end) {
  if (e_end < 0) e_end = m.nlocal_e;
  if (m.nlocal_e <= 0 || e_begin >= e_end) return;
  FusedArgs a{};
  a.e_begin = e_begin;
  a.e_end = e_end;
  a.lat_rec = t.lat_rec;
  a.node_hl = t.node_hl;
  a.nodex = t.nodex;
  a.etype = m.etype;
  a.row_first = m.row_first;
  a.node_list = m.node_list;
  a.int_off = t.int_off;
  a.inter_off = t.inter_off;
  a.intp = t.intp;
  a.spa_int_hl = t.spa_int_hl;
  a.frho_ds = t.frho_ds;
  {
    const float h = (float) e.rdrho;
    a.rdrho_ds = make_float2(h, (float) (e.rdrho - (double) h));
  }
  a.spa_int = t.spa_int;
  a.spa_inter = t.spa_inter;
  a.fjj = t.fjj;
  a.fjj_off = t.fjj_off;
  a.wn = t.wn;
  a.wnf = t.wnf;
  a.row_start = m.row_start;
  a.ent = m.ent;
  a.nnear_row = m.nnear_row;
  a.eflags = m.eflags;
  a.nlocal_e = m.nlocal_e;
  a.maxlines = t.maxlines;
  a.cutsq_f = m.cutsq_f;
  a.band_lo = m.band_lo;
  a.band_hi = m.band_hi;
  a.cutsq = m.cutsq;
  a.skip = m.skip;
  a.band = t.band;
  a.lat = m.lat;
  a.fp4 = m.fp4;
  a.nrho = m.nrho;
  a.rdrho = m.rdrho;
  a.frho = e.frho;
  a.rdrho64 = e.rdrho;
  const bool force = pass != 1;
  const bool eam = pass != 0;
  const size_t table =
      eam ? sizeof(float4) * ((force ? FTAB_W : 1) * (size_t) (e.nr + 1) + (force ? e.nrho + 1 : 0))
          : 0;
  if (t.variant == 1) launch_fused<1>(a, pass, tab, e, table, lj1, lj2, erho_in, erho_out, nodef, s);
  else if (t.variant == 2)
    launch_fused<2>(a, pass, tab, e, table, lj1, lj2, erho_in, erho_out, nodef, s);
  else launch_fused<0>(a, pass, tab, e, table, lj1, lj2, erho_in, erho_out, nodef, s);
  check(cudaGetLastError(), "elem_fused");
}

long long self_check(const int *row_start, const int *ent, const int *row_elem, int nrows,
                     const Lattice &lat, int maxlines, unsigned long long *scratch,
                     cudaStream_t s) {
  if (nrows <= 0) return 0;
  check(cudaMemsetAsync(scratch, 0, sizeof(unsigned long long), s), "self_check");
  const int g = persistent_grid((const void *) k_self_check, 256, 0, nrows);
  k_self_check<<<g, 256, 0, s>>>(row_start, ent, row_elem, nrows, lat, maxlines, scratch);
  check(cudaGetLastError(), "self_check");
  unsigned long long c = 0;
  check(cudaMemcpyAsync(&c, scratch, sizeof(c), cudaMemcpyDeviceToHost, s), "self_check");
  check(cudaStreamSynchronize(s), "self_check");
  return (long long) c;
}

void gather_nodef(const float2 *fipf, const int *etype, const int *row_first, const int *numint,
                  const int *int_off, const float *wn, int nlocal_e, double *nodef,
                  cudaStream_t s) {
  if (nlocal_e <= 0) return;
  k_gather_nodef_ds<<<nblk((long long) nlocal_e * 24, 128), 128, 0, s>>>(
      fipf, etype, row_first, numint, int_off, wn, nlocal_e, nodef);
  check(cudaGetLastError(), "gather_nodef_ds");
}

}  // namespace mixed
}  // namespace cacg
