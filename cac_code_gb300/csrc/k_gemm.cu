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

__device__ __forceinline__ float sigmoidf_(float z) { return 1.f / (1.f + __expf(-z)); }

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
      if (ep.kind == 0 || ep.kind == 1) {
        float *dst = ep.c + (size_t) row * ep.ldc + col;
#pragma unroll
        for (int i = 0; i < 16; i++)
          if (col + i < N) dst[i] = v[i] + (ep.kind == 1 ? ep.bias[col + i] : 0.f);
      } else if (ep.kind == 2) {
        float *z = ep.c + (size_t) row * ep.ldc + col;
        __nv_bfloat16 *h = ep.h + (size_t) row * ep.ldh + col;
#pragma unroll
        for (int i = 0; i < 16; i++)
          if (col + i < N) {
            float zz = v[i] + ep.bias[col + i];
            z[i] = zz;
            h[i] = __float2bfloat16(zz * sigmoidf_(zz));
          }
      } else if (ep.kind == 4) {
        __nv_bfloat16 *h = ep.h + (size_t) row * ep.ldh + col;
#pragma unroll
        for (int i = 0; i < 16; i++)
          if (col + i < N) {
            float zz = v[i] + ep.bias[col + i];
            h[i] = __float2bfloat16(zz * sigmoidf_(zz));
          }
      } else {
        const float *z = ep.c + (size_t) row * ep.ldc + col;
        __nv_bfloat16 *h = ep.h + (size_t) row * ep.ldh + col;
#pragma unroll
        for (int i = 0; i < 16; i++)
          if (col + i < N) {
            float zz = z[i], sg = sigmoidf_(zz);
            h[i] = __float2bfloat16(v[i] * sg * (1.f + zz * (1.f - sg)));
          }
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

}  // namespace gemm
}  // namespace cacg
