// BF16 x BF16 -> FP32 GEMM on the 5th-generation tensor cores (sm_103a).
//
//   C[M x N] = A[M x K] * B[N x K]^T        (both operands K-major, row-major)
//
// One CTA computes a 128 x BN tile.  Thread 0 streams 128x64 tiles of A and
// BNx64 tiles of B into shared memory with TMA (128-byte swizzle), issues
// tcgen05.mma (M = 128, N = BN, K = 16 per instruction) into a TMEM
// accumulator, and releases each stage with tcgen05.commit on the stage's
// "empty" mbarrier.  After the last commit the four warps read the
// accumulator back with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, i.e.
// rows 32w..32w+31 of the tile) and apply one of the epilogues below.
//
// Every mbarrier wait is bounded; a wait that runs out sets *err, the CTA
// waits (bounded) for the copies it issued, frees its TMEM and returns.
//
// Epilogues (the surrogate MLP's forward and backward passes):
//   STORE_F32    C = acc                          (fp32, ldc)
//   BIAS_F32     C = acc + bias[n]                (fp32, ldc)
//   BIAS_SILU    Z = acc + bias[n] (fp32, ldc);  H = silu(Z) (bf16, ldh)
//   DSILU        H = acc * silu'(Z[m, n])         (bf16, ldh; Z read, ldc)
//   SILU_ONLY    H = silu(acc + bias[n])          (bf16, ldh; inference)
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "internal.h"

namespace cacg {
namespace gemm {

namespace {

constexpr int BM = 128, BK = 64, NT = 128;
constexpr unsigned WAIT_LIMIT = 1u << 26;

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(unsigned bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}

// bounded wait: false when the limit ran out
__device__ __forceinline__ bool mbar_wait(unsigned bar, unsigned parity) {
  for (unsigned it = 0; it < WAIT_LIMIT; it++)
    if (mbar_try(bar, parity)) return true;
  return false;
}

__device__ __forceinline__ void tma_load_2d(unsigned dst, const CUtensorMap *map, int x, int y,
                                            unsigned bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(dst),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(bar)
      : "memory");
}

// K-major operand, 128-byte swizzle: 8-row atoms of 128 B, 1024 B apart
__device__ __forceinline__ unsigned long long sw128_desc(unsigned addr) {
  unsigned long long d = 0;
  d |= (unsigned long long) ((addr >> 4) & 0x3FFF);
  d |= (unsigned long long) 1 << 16;                  // leading byte offset (unused)
  d |= (unsigned long long) (1024 >> 4) << 32;        // stride byte offset
  d |= (unsigned long long) 1 << 46;                  // descriptor version
  d |= (unsigned long long) 2 << 61;                  // 128-byte swizzle
  return d;
}

// kind::f16 instruction descriptor: D f32, A/B bf16, both K-major, M = 128
__host__ __device__ constexpr unsigned idesc_bf16(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned) (n >> 3) << 17) |
         ((unsigned) (BM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(unsigned tmem, unsigned long long a, unsigned long long b,
                                         unsigned idesc, unsigned acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem),
      "l"(a), "l"(b), "r"(idesc), "r"(acc)
      : "memory");
}

__device__ __forceinline__ void mma_commit(unsigned bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
      : "memory");
}

__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
      "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// sigma(z) = (1 + tanh(z / 2)) / 2 and silu(z) = z sigma(z) = h + h tanh(h), h = z / 2, on
// the hardware tanh (tanh.approx.f32: one special-function instruction against two for
// exp and reciprocal; its error, about 2^-11, is below the bf16 rounding of the
// activations, 2^-9)
__device__ __forceinline__ float tanh_approx(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float sigmoidf_(float z) { return fmaf(0.5f, tanh_approx(0.5f * z), 0.5f); }
__device__ __forceinline__ float siluf_(float z) {
  const float h = 0.5f * z;
  return fmaf(h, tanh_approx(h), h);
}

struct Epi {
  int kind;
  const float *bias;
  float *c;  // fp32 out (STORE_F32, BIAS_F32, BIAS_SILU: Z) or Z in (DSILU)
  int ldc;
  __nv_bfloat16 *h;  // bf16 out (BIAS_SILU, DSILU)
  int ldh;
};

template <int BN, int STAGES>
__global__ void __launch_bounds__(NT, 1)
k_gemm_tn(const __grid_constant__ CUtensorMap tma_a, const __grid_constant__ CUtensorMap tma_b,
          int M, int N, int K, Epi ep, int *err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  // stage buffers on a 1024-byte boundary (swizzle atoms)
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  constexpr int A_BYTES = BM * BK * 2, B_BYTES = BN * BK * 2;
  constexpr int TMEM_COLS = BN < 32 ? 32 : BN;
  unsigned char *sa = base;
  unsigned char *sb = base + STAGES * A_BYTES;
  unsigned long long *bars =
      reinterpret_cast<unsigned long long *>(sb + STAGES * B_BYTES);  // full, empty, done
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + 2 * STAGES + 1);
  __shared__ int s_fail;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int m0 = blockIdx.x * BM, n0 = blockIdx.y * BN;
  const int nk = K / BK;

  if (threadIdx.x == 0) {
    s_fail = 0;
    for (int i = 0; i < 2 * STAGES + 1; i++) mbar_init(smem_u32(bars + i), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;

  if (threadIdx.x == 0) {
    const unsigned idesc = idesc_bf16(BN);
    int issued = 0, consumed = 0;
    bool ok = true;
    for (int s = 0; s < STAGES && s < nk; s++) {
      unsigned fb = smem_u32(bars + s);
      mbar_expect_tx(fb, A_BYTES + B_BYTES);
      tma_load_2d(smem_u32(sa + s * A_BYTES), &tma_a, s * BK, m0, fb);
      tma_load_2d(smem_u32(sb + s * B_BYTES), &tma_b, s * BK, n0, fb);
      issued++;
    }
    for (int kt = 0; kt < nk && ok; kt++) {
      const int s = kt % STAGES;
      const unsigned par = (kt / STAGES) & 1;
      if (!mbar_wait(smem_u32(bars + s), par)) {
        ok = false;
        break;
      }
      consumed++;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned a_addr = smem_u32(sa + s * A_BYTES), b_addr = smem_u32(sb + s * B_BYTES);
#pragma unroll
      for (int kk = 0; kk < BK / 16; kk++)
        mma_bf16(tmem, sw128_desc(a_addr + kk * 32), sw128_desc(b_addr + kk * 32), idesc,
                 (kt | kk) != 0);
      mma_commit(smem_u32(bars + STAGES + s));
      // refill the stage the previous k-tile used, once its MMAs are done
      if (kt >= 1) {
        const int pk = kt - 1, ps = pk % STAGES, nxt = pk + STAGES;
        if (nxt < nk) {
          if (!mbar_wait(smem_u32(bars + STAGES + ps), (pk / STAGES) & 1)) {
            ok = false;
            break;
          }
          unsigned fb = smem_u32(bars + ps);
          mbar_expect_tx(fb, A_BYTES + B_BYTES);
          tma_load_2d(smem_u32(sa + ps * A_BYTES), &tma_a, nxt * BK, m0, fb);
          tma_load_2d(smem_u32(sb + ps * B_BYTES), &tma_b, nxt * BK, n0, fb);
          issued++;
        }
      }
    }
    if (ok) {
      mma_commit(smem_u32(bars + 2 * STAGES));
    } else {
      atomicExch(err, 1);
      // let the copies and MMAs already issued finish before the CTA's
      // shared memory and TMEM go away
      for (int k = consumed; k < issued; k++) mbar_wait(smem_u32(bars + k % STAGES), (k / STAGES) & 1);
      mma_commit(smem_u32(bars + 2 * STAGES));
      mbar_wait(smem_u32(bars + 2 * STAGES), 0);
      s_fail = 1;
    }
  }
  __syncwarp();
  // all threads: wait for the accumulator (or the failure flag)
  bool ready = false;
  for (unsigned it = 0; it < WAIT_LIMIT; it++) {
    if (mbar_try(smem_u32(bars + 2 * STAGES), 0)) {
      ready = true;
      break;
    }
    if (*((volatile int *) &s_fail)) break;
  }
  if (!ready && threadIdx.x == 0) atomicExch(err, 2);
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");

  if (__all_sync(0xffffffffu, ready ? 1 : 0)) {
    const int row = m0 + warp * 32 + lane;
    const unsigned tl = tmem + ((unsigned) (warp * 32) << 16);
#pragma unroll 1
    for (int c = 0; c < BN; c += 16) {
      float v[16];
      tmem_ld16(tl + c, v);
      if (row >= M) continue;
      const int col = n0 + c;
      const bool full = col + 16 <= N;
      if (ep.kind == 0 || ep.kind == 1) {
        float *dst = ep.c + (size_t) row * ep.ldc + col;
        if (ep.kind == 1)
#pragma unroll
          for (int i = 0; i < 16; i++) v[i] += col + i < N ? ep.bias[col + i] : 0.f;
        if (full && (ep.ldc & 3) == 0 && (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
#pragma unroll
          for (int i = 0; i < 4; i++)
            reinterpret_cast<float4 *>(dst)[i] = make_float4(v[4 * i], v[4 * i + 1], v[4 * i + 2], v[4 * i + 3]);
        } else {
#pragma unroll
          for (int i = 0; i < 16; i++)
            if (col + i < N) dst[i] = v[i];
        }
        continue;
      }
      // bf16 outputs: 16 values as two 16-byte stores where the row allows it
      float hv[16];
      if (ep.kind == 2 || ep.kind == 4) {
        float *z = ep.c ? ep.c + (size_t) row * ep.ldc + col : nullptr;
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const float zz = v[i] + (col + i < N ? ep.bias[col + i] : 0.f);
          if (ep.kind == 2 && col + i < N) z[i] = zz;
          hv[i] = zz * sigmoidf_(zz);
        }
      } else {
        const float *z = ep.c + (size_t) row * ep.ldc + col;
#pragma unroll
        for (int i = 0; i < 16; i++) {
          const float zz = col + i < N ? z[i] : 0.f, sg = sigmoidf_(zz);
          hv[i] = v[i] * sg * (1.f + zz * (1.f - sg));
        }
      }
      __nv_bfloat16 *h = ep.h + (size_t) row * ep.ldh + col;
      if (full && (ep.ldh & 7) == 0 && (reinterpret_cast<uintptr_t>(h) & 15) == 0) {
        unsigned w[8];
#pragma unroll
        for (int i = 0; i < 8; i++) {
          __nv_bfloat162 p2 = __floats2bfloat162_rn(hv[2 * i], hv[2 * i + 1]);
          w[i] = *reinterpret_cast<unsigned *>(&p2);
        }
        reinterpret_cast<uint4 *>(h)[0] = make_uint4(w[0], w[1], w[2], w[3]);
        reinterpret_cast<uint4 *>(h)[1] = make_uint4(w[4], w[5], w[6], w[7]);
      } else {
#pragma unroll
        for (int i = 0; i < 16; i++)
          if (col + i < N) h[i] = __float2bfloat16(hv[i]);
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem),
                 "r"(TMEM_COLS)
                 : "memory");
  }
}

// ---------------------------------------------------------------- fused ensemble
//
// The whole surrogate ensemble for 128 elements per CTA in one launch:
// for each member k and layer l the CTA runs D = A_l W_l^T on the tensor cores
// (A_1 = the features tile sX, A_l = the previous layer's activations in sA),
// reads D back from TMEM, applies bias + SiLU and writes the BF16 activations
// into sA in the same 128-byte-swizzled K-major layout TMA would produce, so
// the next layer's MMAs read them directly.  The 13 weight k-tiles of each
// member (W1: 1, W2: 4, W3: 4, W4: 4) stream through four shared-memory
// stages, loaded by TMA up to four tiles ahead of the MMAs.  Sixteen warps
// share the epilogue: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows)
// and columns 64 (w / 4) .. + 63.  The last layer's
// outputs are summed over the members in registers; the kernel writes the
// denormalised ensemble mean and the spread (largest per-output standard
// deviation across members).
constexpr int ENS_NT = 512, ENS_STAGES = 4, ENS_H = 256, ENS_OUT = 24, ENS_BSTRIDE = 3 * 256 + 24;
constexpr int ENS_MAX_MEMBERS = 4;  // shared memory: 16 + 64 + 4 x 32 KB + biases
constexpr int ENS_X_BYTES = BM * BK * 2, ENS_A_BYTES = BM * ENS_H * 2, ENS_W_BYTES = ENS_H * BK * 2;

struct EnsArgs {
  const float *bias;  // [members][b1 256, b2 256, b3 256, b4 24]
  const float *norm;  // out_mean at [64, 88), out_std at [88, 112)
  float *mean, *spread;
  int n, members;
  int *err;
  const int *count;  // rows to evaluate (device; null: n); CTAs past it return at once
};

__device__ __forceinline__ void ens_issue(int g, const CUtensorMap *w1, const CUtensorMap *w2,
                                          const CUtensorMap *w3, const CUtensorMap *w4,
                                          unsigned char *sw, unsigned long long *full) {
  const int k = g / 13, r = g % 13;
  const int st = g % ENS_STAGES;
  const unsigned fb = smem_u32(full + st), dst = smem_u32(sw + st * ENS_W_BYTES);
  if (r == 0) {
    mbar_expect_tx(fb, ENS_W_BYTES);
    tma_load_2d(dst, w1, 0, k * ENS_H, fb);
  } else if (r < 5) {
    mbar_expect_tx(fb, ENS_W_BYTES);
    tma_load_2d(dst, w2, (r - 1) * BK, k * ENS_H, fb);
  } else if (r < 9) {
    mbar_expect_tx(fb, ENS_W_BYTES);
    tma_load_2d(dst, w3, (r - 5) * BK, k * ENS_H, fb);
  } else {
    mbar_expect_tx(fb, 32 * BK * 2);
    tma_load_2d(dst, w4, (r - 9) * BK, k * ENS_OUT, fb);
  }
}

// byte offset of (row, 16-byte chunk) in a 128-row, 64-column bf16 SW128 atom column
__device__ __forceinline__ unsigned sw128_off(int row, int chunk) {
  return (unsigned) ((row >> 3) * 1024 + (row & 7) * 128 + ((chunk ^ (row & 7)) << 4));
}

__global__ void __launch_bounds__(ENS_NT, 1)
k_mlp_ensemble(const __grid_constant__ CUtensorMap tma_x, const __grid_constant__ CUtensorMap tma_w1,
               const __grid_constant__ CUtensorMap tma_w2, const __grid_constant__ CUtensorMap tma_w3,
               const __grid_constant__ CUtensorMap tma_w4, EnsArgs a) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  const int nrows = a.count ? *a.count : a.n;
  if ((int) blockIdx.x * BM >= nrows) return;  // before any barrier or allocation
  unsigned char *base = reinterpret_cast<unsigned char *>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~static_cast<uintptr_t>(1023));
  unsigned char *sx = base;
  unsigned char *sa = sx + ENS_X_BYTES;
  unsigned char *sw = sa + ENS_A_BYTES;
  float *sbias = reinterpret_cast<float *>(sw + ENS_STAGES * ENS_W_BYTES);
  unsigned long long *bars =
      reinterpret_cast<unsigned long long *>(sbias + a.members * ENS_BSTRIDE);  // full[3] empty[3] x done
  unsigned *tmem_slot = reinterpret_cast<unsigned *>(bars + 2 * ENS_STAGES + 2);
  unsigned long long *full = bars, *empty = bars + ENS_STAGES, *xbar = bars + 2 * ENS_STAGES,
                     *done = bars + 2 * ENS_STAGES + 1;
  __shared__ int s_fail;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wg = warp >> 2, q = warp & 3, row = q * 32 + lane;
  const int m0 = blockIdx.x * BM;
  const int T = 13 * a.members;

  for (int i = tid; i < a.members * ENS_BSTRIDE; i += ENS_NT) sbias[i] = a.bias[i];
  if (tid == 0) {
    s_fail = 0;
    for (int i = 0; i < 2 * ENS_STAGES + 2; i++) mbar_init(smem_u32(bars + i), 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(tmem_slot)),
                 "r"(ENS_H)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
  const unsigned tmem = *tmem_slot;

  int issued = 0;
  if (tid == 0) {
    mbar_expect_tx(smem_u32(xbar), ENS_X_BYTES);
    tma_load_2d(smem_u32(sx), &tma_x, 0, m0, smem_u32(xbar));
    for (; issued < ENS_STAGES && issued < T; issued++)
      ens_issue(issued, &tma_w1, &tma_w2, &tma_w3, &tma_w4, sw, full);
  }
  float s1[ENS_OUT], s2[ENS_OUT];
#pragma unroll
  for (int c = 0; c < ENS_OUT; c++) s1[c] = s2[c] = 0.f;

  int g = 0;        // next weight tile to consume
  int nlayer = 0;   // layers completed (parity of `done`)
  bool ok = true;
  for (int k = 0; k < a.members && ok; k++) {
    const float *bk = sbias + k * ENS_BSTRIDE;
    for (int l = 1; l <= 4 && ok; l++) {
      if (tid == 0) {
        bool good = true;
        if (g == 0) good = mbar_wait(smem_u32(xbar), 0);
        const int nk = l == 1 ? 1 : 4;
        const unsigned idesc = idesc_bf16(l == 4 ? 32 : ENS_H);
        for (int kt = 0; kt < nk && good; kt++, g++) {
          const int st = g % ENS_STAGES;
          if (!mbar_wait(smem_u32(full + st), (g / ENS_STAGES) & 1)) {
            good = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
          const unsigned a_addr = l == 1 ? smem_u32(sx) : smem_u32(sa + kt * (BM * BK * 2));
          const unsigned b_addr = smem_u32(sw + st * ENS_W_BYTES);
#pragma unroll
          for (int kk = 0; kk < BK / 16; kk++)
            mma_bf16(tmem, sw128_desc(a_addr + kk * 32), sw128_desc(b_addr + kk * 32), idesc,
                     (kt | kk) != 0);
          mma_commit(smem_u32(empty + st));
          if (g >= 1 && issued < T) {  // refill the stage the previous tile used
            const int pg = g - 1;
            if (!mbar_wait(smem_u32(empty + pg % ENS_STAGES), (pg / ENS_STAGES) & 1)) {
              good = false;
              break;
            }
            ens_issue(issued++, &tma_w1, &tma_w2, &tma_w3, &tma_w4, sw, full);
          }
        }
        mma_commit(smem_u32(done));
        if (!good) {
          atomicExch(a.err, 1);
          s_fail = 1;
        }
      }
      __syncwarp();
      bool ready = false;
      for (unsigned it = 0; it < WAIT_LIMIT; it++) {
        if (mbar_try(smem_u32(done), nlayer & 1)) {
          ready = true;
          break;
        }
      }
      nlayer++;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      const unsigned tl = tmem + ((unsigned) (q * 32) << 16);
      if (l < 4) {
        const float *b = bk + (l - 1) * ENS_H;
#pragma unroll 1
        for (int c = wg * 64; c < wg * 64 + 64; c += 16) {
          float v[16];
          tmem_ld16(tl + c, v);
          unsigned w[8];
#pragma unroll
          for (int i = 0; i < 8; i++) {
            float z0 = v[2 * i] + b[c + 2 * i], z1 = v[2 * i + 1] + b[c + 2 * i + 1];
            __nv_bfloat162 h2 = __floats2bfloat162_rn(siluf_(z0), siluf_(z1));
            w[i] = *reinterpret_cast<unsigned *>(&h2);
          }
          const int ac = c >> 6, ch = (c & 63) >> 3;
          unsigned char *dst = sa + ac * (BM * BK * 2);
          *reinterpret_cast<uint4 *>(dst + sw128_off(row, ch)) = make_uint4(w[0], w[1], w[2], w[3]);
          *reinterpret_cast<uint4 *>(dst + sw128_off(row, ch + 1)) = make_uint4(w[4], w[5], w[6], w[7]);
        }
      } else if (wg == 0) {
        const float *b = bk + 3 * ENS_H;
        float v0[16], v1[16];
        tmem_ld16(tl, v0);
        tmem_ld16(tl + 16, v1);
#pragma unroll
        for (int c = 0; c < ENS_OUT; c++) {
          float y = (c < 16 ? v0[c] : v1[c - 16]) + b[c];
          s1[c] += y;
          s2[c] += y * y;
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (__syncthreads_or(!ready || *((volatile int *) &s_fail))) ok = false;
    }
  }
  if (!ok && tid == 0) {
    atomicExch(a.err, 2);
    // let the weight copies already issued land before the CTA exits
    for (int t = g; t < issued; t++) mbar_wait(smem_u32(full + t % ENS_STAGES), (t / ENS_STAGES) & 1);
  }
  if (ok && wg == 0 && m0 + row < nrows) {
    const float inv = 1.f / a.members;
    float smax = 0.f;
    float *mo = a.mean + (size_t) (m0 + row) * ENS_OUT;
#pragma unroll
    for (int c = 0; c < ENS_OUT; c++) {
      const float mu = s1[c] * inv, var = fmaxf(s2[c] * inv - mu * mu, 0.f);
      const float sd = a.norm[88 + c];
      mo[c] = mu * sd + a.norm[64 + c];
      smax = fmaxf(smax, sqrtf(var) * sd);
    }
    a.spread[m0 + row] = smax;
  }
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ENS_H)
                 : "memory");
  }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    check(cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q),
          "cuTensorMapEncodeTiled entry point");
    if (!p || q != cudaDriverEntryPointSuccess)
      throw CudaError{cudaErrorNotSupported, "cuTensorMapEncodeTiled unavailable"};
    fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

// 2-D bf16 map over rows x cols (cols contiguous, ld elements per row), box 64 x box_rows
CUtensorMap make_map(const void *ptr, int rows, int cols, int ld, int box_rows) {
  CUtensorMap m;
  cuuint64_t dims[2] = {(cuuint64_t) cols, (cuuint64_t) rows};
  cuuint64_t strides[1] = {(cuuint64_t) ld * 2};
  cuuint32_t box[2] = {(cuuint32_t) BK, (cuuint32_t) box_rows};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void *>(ptr), dims,
                           strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                           CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw CudaError{cudaErrorInvalidValue, "cuTensorMapEncodeTiled"};
  return m;
}

template <int BN, int STAGES>
size_t smem_bytes() {
  return 1024 + (size_t) STAGES * (BM * BK * 2 + BN * BK * 2) + (2 * STAGES + 1) * 8 + 16;
}

template <int BN, int STAGES>
void launch(const CUtensorMap &ta, const CUtensorMap &tb, int M, int N, int K, const Epi &ep,
            int *err, cudaStream_t s) {
  static bool attr = false;
  size_t smem = smem_bytes<BN, STAGES>();
  if (!attr) {
    check(cudaFuncSetAttribute(k_gemm_tn<BN, STAGES>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int) smem),
          "gemm smem attribute");
    attr = true;
  }
  dim3 grid((M + BM - 1) / BM, (N + BN - 1) / BN);
  k_gemm_tn<BN, STAGES><<<grid, NT, smem, s>>>(ta, tb, M, N, K, ep, err);
  check(cudaGetLastError(), "k_gemm_tn");
}

}  // namespace

// C = A * B^T with A [M x K] (lda), B [N x K] (ldb), bf16, K % 64 == 0,
// lda, ldb multiples of 8, 16-byte aligned bases.  BN = 32, 64, 128 or 256
// by N (N > 256 is split over grid.y).
void gemm_tn(const void *A, int lda, const void *B, int ldb, int M, int N, int K, int kind,
             const float *bias, float *c, int ldc, void *h, int ldh, int *err, cudaStream_t s) {
  if (M <= 0 || N <= 0) return;
  if (K <= 0 || K % BK || lda % 8 || ldb % 8 || (reinterpret_cast<uintptr_t>(A) & 15) ||
      (reinterpret_cast<uintptr_t>(B) & 15))
    throw CudaError{cudaErrorInvalidValue,
                    "gemm_tn: K must be a multiple of 64, leading dimensions multiples of 8"};
  Epi ep{kind, bias, c, ldc, static_cast<__nv_bfloat16 *>(h), ldh};
  const int bn = N <= 32 ? 32 : N <= 64 ? 64 : N <= 128 ? 128 : 256;
  CUtensorMap ta = make_map(A, M, K, lda, BM);
  CUtensorMap tb = make_map(B, N, K, ldb, bn);
  switch (bn) {
    case 32: launch<32, 4>(ta, tb, M, N, K, ep, err, s); break;
    case 64: launch<64, 4>(ta, tb, M, N, K, ep, err, s); break;
    case 128: launch<128, 4>(ta, tb, M, N, K, ep, err, s); break;
    default: launch<256, 3>(ta, tb, M, N, K, ep, err, s); break;
  }
}

// The fused ensemble on normalised bf16 features xf[n][64]; weights stacked
// over the members: w1s[m*256][64], w2s/w3s[m*256][256], w4s[m*24][256];
// bias[m][792] (b1, b2, b3, b4).
void mlp_ensemble(const void *xf, int n, const void *w1s, const void *w2s, const void *w3s,
                  const void *w4s, const float *bias, int members, const float *norm, float *mean,
                  float *spread, int *err, cudaStream_t s, const int *count) {
  if (n <= 0) return;
  if (members < 1 || members > ENS_MAX_MEMBERS)
    throw CudaError{cudaErrorInvalidValue, "mlp_ensemble: 1..4 members"};
  CUtensorMap tx = make_map(xf, n, 64, 64, BM);
  CUtensorMap t1 = make_map(w1s, members * ENS_H, 64, 64, ENS_H);
  CUtensorMap t2 = make_map(w2s, members * ENS_H, ENS_H, ENS_H, ENS_H);
  CUtensorMap t3 = make_map(w3s, members * ENS_H, ENS_H, ENS_H, ENS_H);
  CUtensorMap t4 = make_map(w4s, members * ENS_OUT, ENS_H, ENS_H, 32);
  const size_t smem = 1024 + ENS_X_BYTES + ENS_A_BYTES + (size_t) ENS_STAGES * ENS_W_BYTES +
                      sizeof(float) * members * ENS_BSTRIDE + (2 * ENS_STAGES + 2) * 8 + 16;
  static size_t attr = 0;
  if (smem > attr) {
    check(cudaFuncSetAttribute(k_mlp_ensemble, cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem),
          "ensemble smem attribute");
    attr = smem;
  }
  EnsArgs a{bias, norm, mean, spread, n, members, err, count};
  k_mlp_ensemble<<<(n + BM - 1) / BM, ENS_NT, smem, s>>>(tx, t1, t2, t3, t4, a);
  check(cudaGetLastError(), "k_mlp_ensemble");
}

}  // namespace gemm
}  // namespace cacg
