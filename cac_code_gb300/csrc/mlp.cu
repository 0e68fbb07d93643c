// The nodal-force surrogate: an ensemble of MLPs 32 -> 256 -> 256 -> 256 -> 24
// (SiLU) that maps an element's 24 nodal displacements (about their mean,
// relative to the ideal lattice) and 8 nodal densities to its 24 nodal forces.
//
// Every matrix product, forward and backward, runs on the tensor cores through
// gemm::gemm_tn (BF16 operands, FP32 accumulation, k_gemm.cu).  Master weights,
// Adam moments and gradients are FP32; activations cross layers as BF16 and
// pre-activations are kept in FP32 for the SiLU derivative.  The reference has
// no counterpart: it evaluates every element by integration-point quadrature.
//
// Layouts (row-major, K-major operands as the GEMM wants them):
//   parameters per member, flattened: W1[256][32] b1[256] W2[256][256] b2
//   W3[256][256] b3 W4[24][256] b4[24]
//   bf16 copies: w1[256][64] (K padded), w2, w3, w4[24][256];
//   for the backward pass w2t = W2^T, w3t = W3^T, w4t[256][64] = W4^T padded.
//   activations x0[B][64] (features, zero padded), z_l (FP32) and h_l (BF16)
//   [B][256], output y[B][24] (FP32), gradients g4[B][64], g_l[B][256] (BF16).
//   dW_l = g_l^T h_{l-1}: both operands transposed first ([rows][B]).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "cacg.h"
#include "internal.h"

namespace cacg {
namespace mlp {

using bf16 = __nv_bfloat16;

namespace {

constexpr int NIN = MLP_IN, NINP = 64, NH = MLP_HIDDEN, NOUT = MLP_OUT, NGP = 64;
static_assert(NH % 64 == 0 && NIN <= NINP && NOUT <= NGP, "layer shapes the GEMM tiles support");
constexpr long oW1 = 0, ob1 = oW1 + (long) NH * NIN, oW2 = ob1 + NH, ob2 = oW2 + (long) NH * NH,
               oW3 = ob2 + NH, ob3 = oW3 + (long) NH * NH, oW4 = ob3 + NH,
               ob4 = oW4 + (long) NOUT * NH, NPARAM = ob4 + NOUT;

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

__global__ void k_cast_pad(const float *__restrict__ src, int rows, int cols, int lds,
                           bf16 *__restrict__ dst, int ldd, int rows_out) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= (long) rows_out * ldd) return;
  int r = (int) (i / ldd), c = (int) (i % ldd);
  dst[i] = __float2bfloat16(r < rows && c < cols ? src[(long) r * lds + c] : 0.f);
}

// dst[c][r] = src[r][c] (rows x cols -> cols x ldd, zero beyond rows)
__global__ void k_cast_transpose(const float *__restrict__ src, int rows, int cols,
                                 bf16 *__restrict__ dst, int ldd) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= (long) cols * ldd) return;
  int c = (int) (i / ldd), r = (int) (i % ldd);
  dst[i] = __float2bfloat16(r < rows ? src[(long) r * cols + c] : 0.f);
}

// out[c][r] = in[r][c] for r < rows, c < cols (32x32 tiles through shared memory)
__global__ void k_transpose(const bf16 *__restrict__ in, int rows, int cols, int ldi,
                            bf16 *__restrict__ out, int ldo) {
  __shared__ bf16 t[32][33];
  int r0 = blockIdx.y * 32, c0 = blockIdx.x * 32;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int r = r0 + k, c = c0 + threadIdx.x;
    t[k][threadIdx.x] = (r < rows && c < cols) ? in[(long) r * ldi + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    int c = c0 + k, r = r0 + threadIdx.x;
    if (c < cols && r < rows) out[(long) c * ldo + r] = t[threadIdx.x][k];
  }
}

// column sums of a bf16 [rows][ld] matrix, added into fp32 out[cols] (zeroed
// by the caller): block (x, y) sums 256 rows of 32 columns
__global__ void k_colsum(const bf16 *__restrict__ g, int rows, int cols, int ld,
                         float *__restrict__ out) {
  __shared__ float red[8][33];
  const int c = blockIdx.x * 32 + threadIdx.x;
  const int r0 = blockIdx.y * 256, r1 = min(rows, r0 + 256);
  float s = 0.f;
  if (c < cols)
    for (int r = r0 + threadIdx.y; r < r1; r += blockDim.y) s += __bfloat162float(g[(long) r * ld + c]);
  red[threadIdx.y][threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.y == 0 && c < cols) {
    float t = 0.f;
    for (int k = 0; k < (int) blockDim.y; k++) t += red[k][threadIdx.x];
    atomicAdd(out + c, t);
  }
}

// g4 = 2 (y - t) / (n_valid * 24) as bf16 [B][64] (zero padding and rows), and
// per-block partial sums of (y - t)^2
__global__ void k_loss_grad(const float *__restrict__ y, const float *__restrict__ t, int B,
                            int n_valid, bf16 *__restrict__ g4, double *__restrict__ part) {
  __shared__ double red[256];
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  double sq = 0.0;
  if (i < (long) B * NGP) {
    int r = (int) (i / NGP), c = (int) (i % NGP);
    float gv = 0.f;
    if (r < n_valid && c < NOUT) {
      float d = y[(long) r * NOUT + c] - t[(long) r * NOUT + c];
      sq = (double) d * d;
      gv = 2.f * d / ((float) n_valid * NOUT);
    }
    g4[i] = __float2bfloat16(gv);
  }
  red[threadIdx.x] = sq;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if ((int) threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

__global__ void k_adam(float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, long n, float lr, float b1, float b2, float eps,
                       float bc1, float bc2) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= n) return;
  float gi = g[i];
  float mi = b1 * m[i] + (1.f - b1) * gi;
  float vi = b2 * v[i] + (1.f - b2) * gi * gi;
  m[i] = mi;
  v[i] = vi;
  p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
}

// normalised features as bf16 [n][64]: (x - mean) * inv_std, zero padded
__global__ void k_features(const float *__restrict__ x, long n, const float *__restrict__ norm,
                           bf16 *__restrict__ out) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= n * NINP) return;
  long r = i / NINP;
  int c = (int) (i % NINP);
  float v = 0.f;
  if (c < NIN) v = (x[r * NIN + c] - norm[c]) * norm[NIN + c];
  out[i] = __float2bfloat16(v);
}

// normalised targets: (t - out_mean) / out_std
__global__ void k_targets(const float *__restrict__ t, long n, const float *__restrict__ norm,
                          float *__restrict__ out) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= n * NOUT) return;
  int c = (int) (i % NOUT);
  out[i] = (t[i] - norm[2 * NIN + c]) / norm[2 * NIN + NOUT + c];
}

// rows of a permutation into a contiguous batch (features bf16, targets fp32)
__global__ void k_gather(const bf16 *__restrict__ xall, const float *__restrict__ tall,
                         const int *__restrict__ idx, int nb, bf16 *__restrict__ x0,
                         float *__restrict__ tb) {
  long i = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (i >= (long) nb * NINP) return;
  int r = (int) (i / NINP), c = (int) (i % NINP);
  int src = idx[r];
  x0[i] = src >= 0 ? xall[(long) src * NINP + c] : __float2bfloat16(0.f);
  if (c < NOUT) tb[(long) r * NOUT + c] = src >= 0 ? tall[(long) src * NOUT + c] : 0.f;
}

// ensemble mean (denormalised) and spread: max over outputs of the members'
// standard deviation, in force units
__global__ void k_ensemble(const float *__restrict__ y, long n, int members, long mstride,
                           const float *__restrict__ norm, float *__restrict__ mean,
                           float *__restrict__ spread) {
  long r = blockIdx.x * (long) blockDim.x + threadIdx.x;
  if (r >= n) return;
  float smax = 0.f;
  for (int c = 0; c < NOUT; c++) {
    float s1 = 0.f, s2 = 0.f;
    for (int k = 0; k < members; k++) {
      float v = y[k * mstride + r * NOUT + c];
      s1 += v;
      s2 += v * v;
    }
    float mu = s1 / members;
    float var = fmaxf(s2 / members - mu * mu, 0.f);
    float sd = norm[2 * NIN + NOUT + c];
    mean[r * NOUT + c] = mu * sd + norm[2 * NIN + c];
    smax = fmaxf(smax, sqrtf(var) * sd);
  }
  spread[r] = smax;
}

// splitmix64: seeded, platform-independent initialisation
struct Rng {
  unsigned long long s;
  unsigned long long next() {
    unsigned long long z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (next() >> 11) * (1.0 / 9007199254740992.0); }
};

}  // namespace

struct Member {
  DBuf<float> p, m, v, g;
  DBuf<bf16> w1, w2, w3, w4, w2t, w3t, w4t;
};

struct Net {
  int device = 0, members = 0;
  cudaStream_t stream = nullptr;
  std::vector<Member> mem;
  float norm[2 * NIN + 2 * NOUT];  // in_mean, in_inv_std, out_mean, out_std
  double force_scale = 1.0;        // rms nodal-force magnitude of the training targets
  long long adam_steps = 0;
  std::string err;
  DBuf<float> d_norm;
  int bcap = 0;
  DBuf<bf16> x0, h1, h2, h3, g4, g3, g2, g1, x0t, h1t, h2t, h3t, g1t, g2t, g3t, g4t;
  DBuf<float> z1, z2, z3, y, tb, db;
  DBuf<double> part;
  DBuf<int> errflag;
  // inference buffers
  long long icap = 0;
  DBuf<bf16> ix0, ih1, ih2, ih3;
  DBuf<float> iy, iw1b;
  DBuf<bf16> iw1;  // all members' W1 stacked [members*256][64]

  void sync() { check(cudaStreamSynchronize(stream), "mlp sync"); }

  void ensure_err(cudaStream_t s) {
    if (errflag.p) return;
    errflag.ensure(1, s);
    check(cudaMemsetAsync(errflag.p, 0, sizeof(int), s), "errflag");
  }

  void upload_norm() {
    d_norm.ensure(2 * NIN + 2 * NOUT, stream);
    check(cudaMemcpyAsync(d_norm.p, norm, sizeof(norm), cudaMemcpyHostToDevice, stream), "norm");
  }

  void init_params(unsigned long long seed) {
    Rng rng{seed};
    std::vector<float> h(NPARAM);
    for (int k = 0; k < members; k++) {
      Member &M = mem[k];
      auto fill = [&](long off, int rows, int cols, double gain) {
        double a = gain * std::sqrt(3.0 / cols);
        for (long i = 0; i < (long) rows * cols; i++) h[off + i] = (float) ((2 * rng.uniform() - 1) * a);
      };
      std::fill(h.begin(), h.end(), 0.f);
      fill(oW1, NH, NIN, 1.0);
      fill(oW2, NH, NH, 1.0);
      fill(oW3, NH, NH, 1.0);
      fill(oW4, NOUT, NH, 0.1);
      M.p.ensure(NPARAM, stream);
      M.m.ensure(NPARAM, stream);
      M.v.ensure(NPARAM, stream);
      M.g.ensure(NPARAM, stream);
      check(cudaMemcpyAsync(M.p.p, h.data(), sizeof(float) * NPARAM, cudaMemcpyHostToDevice, stream), "params");
      check(cudaMemsetAsync(M.m.p, 0, sizeof(float) * NPARAM, stream), "adam m");
      check(cudaMemsetAsync(M.v.p, 0, sizeof(float) * NPARAM, stream), "adam v");
      refresh(k);
    }
    sync();
  }

  // bf16 copies of member k's weights (forward and transposed)
  void refresh(int k) {
    Member &M = mem[k];
    stacked = false;
    cudaStream_t s = stream;
    M.w1.ensure((size_t) NH * NINP, s);
    M.w2.ensure((size_t) NH * NH, s);
    M.w3.ensure((size_t) NH * NH, s);
    M.w4.ensure((size_t) NOUT * NH, s);
    M.w2t.ensure((size_t) NH * NH, s);
    M.w3t.ensure((size_t) NH * NH, s);
    M.w4t.ensure((size_t) NH * NGP, s);
    k_cast_pad<<<nblk((long) NH * NINP, 256), 256, 0, s>>>(M.p.p + oW1, NH, NIN, NIN, M.w1.p, NINP, NH);
    k_cast_pad<<<nblk((long) NH * NH, 256), 256, 0, s>>>(M.p.p + oW2, NH, NH, NH, M.w2.p, NH, NH);
    k_cast_pad<<<nblk((long) NH * NH, 256), 256, 0, s>>>(M.p.p + oW3, NH, NH, NH, M.w3.p, NH, NH);
    k_cast_pad<<<nblk((long) NOUT * NH, 256), 256, 0, s>>>(M.p.p + oW4, NOUT, NH, NH, M.w4.p, NH, NOUT);
    k_cast_transpose<<<nblk((long) NH * NH, 256), 256, 0, s>>>(M.p.p + oW2, NH, NH, M.w2t.p, NH);
    k_cast_transpose<<<nblk((long) NH * NH, 256), 256, 0, s>>>(M.p.p + oW3, NH, NH, M.w3t.p, NH);
    k_cast_transpose<<<nblk((long) NH * NGP, 256), 256, 0, s>>>(M.p.p + oW4, NOUT, NH, M.w4t.p, NGP);
    check(cudaGetLastError(), "mlp refresh");
  }

  void ensure_batch(int B) {
    if (B <= bcap) return;
    cudaStream_t s = stream;
    size_t b = (size_t) B;
    x0.ensure(b * NINP, s);
    for (DBuf<bf16> *p : {&h1, &h2, &h3, &g3, &g2, &g1}) p->ensure(b * NH, s);
    g4.ensure(b * NGP, s);
    x0t.ensure(b * NINP, s);
    for (DBuf<bf16> *p : {&h1t, &h2t, &h3t, &g1t, &g2t, &g3t}) p->ensure(b * NH, s);
    g4t.ensure(b * NOUT, s);
    for (DBuf<float> *p : {&z1, &z2, &z3}) p->ensure(b * NH, s);
    y.ensure(b * NOUT, s);
    tb.ensure(b * NOUT, s);
    db.ensure(NH, s);
    part.ensure(nblk(b * NGP, 256), s);
    ensure_err(s);
    bcap = B;
  }

  void transpose(const bf16 *in, int rows, int cols, int ldi, bf16 *out, int ldo) {
    dim3 g(nblk(cols, 32), nblk(rows, 32)), b(32, 8);
    k_transpose<<<g, b, 0, stream>>>(in, rows, cols, ldi, out, ldo);
    check(cudaGetLastError(), "transpose");
  }

  void colsum(const bf16 *g, int rows, int cols, int ld, float *out) {
    check(cudaMemsetAsync(out, 0, sizeof(float) * cols, stream), "colsum zero");
    k_colsum<<<dim3(nblk(cols, 32), nblk(rows, 256)), dim3(32, 8), 0, stream>>>(g, rows, cols, ld, out);
    check(cudaGetLastError(), "colsum");
  }

  // forward of member k on x0 (B rows), keeping z and h for the backward pass
  void forward_train(int k, int B) {
    Member &M = mem[k];
    int *e = errflag.p;
    gemm::gemm_tn(x0.p, NINP, M.w1.p, NINP, B, NH, NINP, 2, M.p.p + ob1, z1.p, NH, h1.p, NH, e, stream);
    gemm::gemm_tn(h1.p, NH, M.w2.p, NH, B, NH, NH, 2, M.p.p + ob2, z2.p, NH, h2.p, NH, e, stream);
    gemm::gemm_tn(h2.p, NH, M.w3.p, NH, B, NH, NH, 2, M.p.p + ob3, z3.p, NH, h3.p, NH, e, stream);
    gemm::gemm_tn(h3.p, NH, M.w4.p, NH, B, NOUT, NH, 1, M.p.p + ob4, y.p, NOUT, nullptr, 0, e, stream);
  }

  // loss against tb (n_valid of B rows) and all gradients of member k into M.g
  double backward(int k, int B, int n_valid, bool want_loss) {
    Member &M = mem[k];
    int *e = errflag.p;
    cudaStream_t s = stream;
    const int nb = nblk((long) B * NGP, 256);
    k_loss_grad<<<nb, 256, 0, s>>>(y.p, tb.p, B, n_valid, g4.p, part.p);
    check(cudaGetLastError(), "loss");
    // backward through the layers: g_{l} = (g_{l+1} W_{l+1}) * silu'(z_l)
    gemm::gemm_tn(g4.p, NGP, M.w4t.p, NGP, B, NH, NGP, 3, nullptr, z3.p, NH, g3.p, NH, e, s);
    gemm::gemm_tn(g3.p, NH, M.w3t.p, NH, B, NH, NH, 3, nullptr, z2.p, NH, g2.p, NH, e, s);
    gemm::gemm_tn(g2.p, NH, M.w2t.p, NH, B, NH, NH, 3, nullptr, z1.p, NH, g1.p, NH, e, s);
    // weight gradients dW_l = g_l^T h_{l-1} (operands transposed to K = batch)
    transpose(x0.p, B, NINP, NINP, x0t.p, B);
    transpose(h1.p, B, NH, NH, h1t.p, B);
    transpose(h2.p, B, NH, NH, h2t.p, B);
    transpose(h3.p, B, NH, NH, h3t.p, B);
    transpose(g1.p, B, NH, NH, g1t.p, B);
    transpose(g2.p, B, NH, NH, g2t.p, B);
    transpose(g3.p, B, NH, NH, g3t.p, B);
    transpose(g4.p, B, NOUT, NGP, g4t.p, B);
    // dW1 lands in a [256][64] scratch (z1 is free now), then compacts to [256][32]
    gemm::gemm_tn(g1t.p, B, x0t.p, B, NH, NINP, B, 0, nullptr, z1.p, NINP, nullptr, 0, e, s);
    check(cudaMemcpy2DAsync(M.g.p + oW1, sizeof(float) * NIN, z1.p, sizeof(float) * NINP,
                            sizeof(float) * NIN, NH, cudaMemcpyDeviceToDevice, s), "dW1");
    gemm::gemm_tn(g2t.p, B, h1t.p, B, NH, NH, B, 0, nullptr, M.g.p + oW2, NH, nullptr, 0, e, s);
    gemm::gemm_tn(g3t.p, B, h2t.p, B, NH, NH, B, 0, nullptr, M.g.p + oW3, NH, nullptr, 0, e, s);
    gemm::gemm_tn(g4t.p, B, h3t.p, B, NOUT, NH, B, 0, nullptr, M.g.p + oW4, NH, nullptr, 0, e, s);
    colsum(g1.p, B, NH, NH, M.g.p + ob1);
    colsum(g2.p, B, NH, NH, M.g.p + ob2);
    colsum(g3.p, B, NH, NH, M.g.p + ob3);
    colsum(g4.p, B, NOUT, NGP, M.g.p + ob4);
    if (!want_loss) return 0.0;
    std::vector<double> h(nb);
    check(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * nb, cudaMemcpyDeviceToHost, s), "loss");
    sync();
    double l = 0.0;
    for (double v : h) l += v;
    return l / ((double) n_valid * NOUT);
  }

  void check_err() {
    int v = 0;
    check(cudaMemcpyAsync(&v, errflag.p, sizeof(int), cudaMemcpyDeviceToHost, stream), "errflag");
    sync();
    if (v) throw CudaError{cudaErrorLaunchTimeout, "tensor-core GEMM: a bounded wait ran out"};
  }

  void adam(int k, float lr) {
    Member &M = mem[k];
    const float b1 = 0.9f, b2 = 0.999f;
    const double t = (double) adam_steps + 1;
    k_adam<<<nblk(NPARAM, 256), 256, 0, stream>>>(M.p.p, M.g.p, M.m.p, M.v.p, NPARAM, lr, b1, b2,
                                                  1e-8f, (float) (1 - std::pow(b1, t)),
                                                  (float) (1 - std::pow(b2, t)));
    check(cudaGetLastError(), "adam");
    refresh(k);
  }

  bool stacked = false;  // iw1/iw1b hold the current first layers

  // ensemble prediction on normalised bf16 features already on the device:
  // one fused launch over all members and layers (gemm::mlp_ensemble)
  DBuf<bf16> iw2, iw3, iw4;
  DBuf<float> ibias;
  void predict_device(const bf16 *xf, long long n, float *mean, float *spread, cudaStream_t s,
                      const int *dcount = nullptr) {
    if (n <= 0) return;
    ensure_err(s);
    if (!stacked) {
      const int BS = 3 * NH + NOUT;
      iw1.ensure((size_t) members * NH * NINP, s);
      iw2.ensure((size_t) members * NH * NH, s);
      iw3.ensure((size_t) members * NH * NH, s);
      iw4.ensure((size_t) members * NOUT * NH, s);
      ibias.ensure((size_t) members * BS, s);
      for (int k = 0; k < members; k++) {
        Member &M = mem[k];
        check(cudaMemcpyAsync(iw1.p + (size_t) k * NH * NINP, M.w1.p, sizeof(bf16) * NH * NINP, cudaMemcpyDeviceToDevice, s), "w1s");
        check(cudaMemcpyAsync(iw2.p + (size_t) k * NH * NH, M.w2.p, sizeof(bf16) * NH * NH, cudaMemcpyDeviceToDevice, s), "w2s");
        check(cudaMemcpyAsync(iw3.p + (size_t) k * NH * NH, M.w3.p, sizeof(bf16) * NH * NH, cudaMemcpyDeviceToDevice, s), "w3s");
        check(cudaMemcpyAsync(iw4.p + (size_t) k * NOUT * NH, M.w4.p, sizeof(bf16) * NOUT * NH, cudaMemcpyDeviceToDevice, s), "w4s");
        float *b = ibias.p + (size_t) k * BS;
        check(cudaMemcpyAsync(b, M.p.p + ob1, sizeof(float) * NH, cudaMemcpyDeviceToDevice, s), "b1s");
        check(cudaMemcpyAsync(b + NH, M.p.p + ob2, sizeof(float) * NH, cudaMemcpyDeviceToDevice, s), "b2s");
        check(cudaMemcpyAsync(b + 2 * NH, M.p.p + ob3, sizeof(float) * NH, cudaMemcpyDeviceToDevice, s), "b3s");
        check(cudaMemcpyAsync(b + 3 * NH, M.p.p + ob4, sizeof(float) * NOUT, cudaMemcpyDeviceToDevice, s), "b4s");
      }
      stacked = true;
    }
    gemm::mlp_ensemble(xf, (int) n, iw1.p, iw2.p, iw3.p, iw4.p, ibias.p, members, d_norm.p, mean,
                       spread, errflag.p, s, dcount);
  }
};

Net *net_of(cacg_mlp_t *m);
const float *norm_device(const Net *n) { return n->d_norm.p; }
double force_scale(const Net *n) { return n->force_scale; }
int members(const Net *n) { return n->members; }
void predict(Net *n, const void *xf, long long count, float *mean, float *spread, cudaStream_t s,
             const int *dcount) {
  n->ensure_err(s);
  n->predict_device(static_cast<const bf16 *>(xf), count, mean, spread, s, dcount);
}
void check_error(Net *n, cudaStream_t s) {
  int v = 0;
  check(cudaMemcpyAsync(&v, n->errflag.p, sizeof(int), cudaMemcpyDeviceToHost, s), "errflag");
  check(cudaStreamSynchronize(s), "errflag sync");
  if (v) throw CudaError{cudaErrorLaunchTimeout, "tensor-core GEMM: a bounded wait ran out"};
}

void features_bf16(const float *x, long long n, const float *norm, bf16 *out, cudaStream_t s) {
  k_features<<<nblk(n * NINP, 256), 256, 0, s>>>(x, n, norm, out);
  check(cudaGetLastError(), "features");
}

void targets(const float *t, long long n, const float *norm, float *out, cudaStream_t s) {
  k_targets<<<nblk(n * NOUT, 256), 256, 0, s>>>(t, n, norm, out);
  check(cudaGetLastError(), "targets");
}

void gather(const bf16 *xall, const float *tall, const int *idx, int nb, bf16 *x0, float *tb,
            cudaStream_t s) {
  k_gather<<<nblk((long) nb * NINP, 256), 256, 0, s>>>(xall, tall, idx, nb, x0, tb);
  check(cudaGetLastError(), "gather");
}

}  // namespace mlp
}  // namespace cacg

// ------------------------------------------------------------------ C ABI

using cacg::CudaError;
using cacg::mlp::Net;
using cacg::mlp::bf16;

struct cacg_mlp_t {
  Net net;
};

namespace cacg {
namespace mlp {
Net *net_of(cacg_mlp_t *m) { return m ? &m->net : nullptr; }
}  // namespace mlp
}  // namespace cacg

namespace {

struct MlpError {
  int code;
  std::string msg;
};

#define MLP_BEGIN             \
  if (!m) return CACG_EINVAL; \
  try {                       \
    cacg::check(cudaSetDevice(m->net.device), "cudaSetDevice");
#define MLP_END                                                            \
  return CACG_OK;                                                          \
  }                                                                        \
  catch (const MlpError &e) {                                              \
    m->net.err = e.msg;                                                    \
    return e.code;                                                         \
  }                                                                        \
  catch (const CudaError &e) {                                             \
    m->net.err = std::string(e.where) + ": " + cudaGetErrorString(e.code); \
    return CACG_ECUDA;                                                     \
  }                                                                        \
  catch (const std::bad_alloc &) {                                         \
    m->net.err = "host allocation failed";                                 \
    return CACG_ENOMEM;                                                    \
  }

void need(bool ok, const char *msg) {
  if (!ok) throw MlpError{CACG_EINVAL, msg};
}

using namespace cacg::mlp;

constexpr int MLP_IN = cacg::MLP_IN, MLP_OUT = cacg::MLP_OUT, MLP_HIDDEN = cacg::MLP_HIDDEN;
constexpr long kNParam = (long) MLP_HIDDEN * MLP_IN + MLP_HIDDEN +
                         2L * (MLP_HIDDEN * MLP_HIDDEN + MLP_HIDDEN) + (long) MLP_OUT * MLP_HIDDEN +
                         MLP_OUT;

// upload normalised features (bf16 [n][64]) and targets (fp32 [n][24])
void upload_set(Net &N, const float *x, const float *t, long long n, cacg::DBuf<bf16> &xf,
                cacg::DBuf<float> &tf) {
  cudaStream_t s = N.stream;
  cacg::DBuf<float> raw;
  raw.ensure((size_t) n * MLP_IN + 1, s);
  cacg::check(cudaMemcpyAsync(raw.p, x, sizeof(float) * n * MLP_IN, cudaMemcpyHostToDevice, s), "x");
  xf.ensure((size_t) n * 64 + 64, s);
  cacg::mlp::features_bf16(raw.p, n, N.d_norm.p, xf.p, s);
  if (t) {
    cacg::DBuf<float> rt;
    rt.ensure((size_t) n * MLP_OUT + 1, s);
    cacg::check(cudaMemcpyAsync(rt.p, t, sizeof(float) * n * MLP_OUT, cudaMemcpyHostToDevice, s), "t");
    tf.ensure((size_t) n * MLP_OUT + 1, s);
    cacg::mlp::targets(rt.p, n, N.d_norm.p, tf.p, s);
    N.sync();
    rt.release();
  }
  N.sync();
  raw.release();
}

}  // namespace

extern "C" {

int cacg_mlp_create(cacg_mlp *out, int device, int members, unsigned long long seed) {
  if (!out || members < 1 || members > 4) return CACG_EINVAL;
  *out = nullptr;
  cacg_mlp m = new (std::nothrow) cacg_mlp_t;
  if (!m) return CACG_ENOMEM;
  m->net.device = device;
  m->net.members = members;
  int rc = CACG_OK;
  try {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
      throw MlpError{CACG_ECUDA, "no CUDA device"};
    cacg::check(cudaSetDevice(device), "cudaSetDevice");
    cacg::check(cudaStreamCreateWithFlags(&m->net.stream, cudaStreamNonBlocking), "stream");
    for (int i = 0; i < MLP_IN; i++) m->net.norm[i] = 0.f, m->net.norm[MLP_IN + i] = 1.f;
    for (int i = 0; i < MLP_OUT; i++)
      m->net.norm[2 * MLP_IN + i] = 0.f, m->net.norm[2 * MLP_IN + MLP_OUT + i] = 1.f;
    m->net.upload_norm();
    m->net.mem.resize(members);
    m->net.init_params(seed);
  } catch (const MlpError &e) {
    rc = e.code;
  } catch (const CudaError &) {
    rc = CACG_ECUDA;
  }
  if (rc != CACG_OK) {
    delete m;
    return rc;
  }
  *out = m;
  return CACG_OK;
}

int cacg_mlp_destroy(cacg_mlp m) {
  if (!m) return CACG_OK;
  cudaSetDevice(m->net.device);
  if (m->net.stream) cudaStreamSynchronize(m->net.stream);
  Net &N = m->net;
  for (Member &M : N.mem)
    for (auto *b : {&M.p, &M.m, &M.v, &M.g}) b->release();
  for (Member &M : N.mem)
    for (auto *b : {&M.w1, &M.w2, &M.w3, &M.w4, &M.w2t, &M.w3t, &M.w4t}) b->release();
  for (auto *b : {&N.x0, &N.h1, &N.h2, &N.h3, &N.g4, &N.g3, &N.g2, &N.g1, &N.x0t, &N.h1t, &N.h2t,
                  &N.h3t, &N.g1t, &N.g2t, &N.g3t, &N.g4t, &N.ix0, &N.ih1, &N.ih2, &N.ih3, &N.iw1})
    b->release();
  for (auto *b : {&N.d_norm, &N.z1, &N.z2, &N.z3, &N.y, &N.tb, &N.db, &N.iy, &N.iw1b, &N.ibias})
    b->release();
  for (auto *b : {&N.iw2, &N.iw3, &N.iw4}) b->release();
  N.part.release();
  N.errflag.release();
  if (N.stream) cudaStreamDestroy(N.stream);
  delete m;
  return CACG_OK;
}

const char *cacg_mlp_error(cacg_mlp m) { return m ? m->net.err.c_str() : "null handle"; }

int cacg_mlp_sizes(cacg_mlp m, long long *sizes, int n) {
  MLP_BEGIN
  need(sizes && n > 0, "bad output array");
  long long v[6] = {m->net.members, kNParam, MLP_IN, MLP_OUT, MLP_HIDDEN, m->net.adam_steps};
  for (int i = 0; i < n && i < 6; i++) sizes[i] = v[i];
  MLP_END
}

int cacg_mlp_get_params(cacg_mlp m, int member, float *p) {
  MLP_BEGIN
  need(p && member >= 0 && member < m->net.members, "bad member or array");
  cacg::check(cudaMemcpyAsync(p, m->net.mem[member].p.p, sizeof(float) * kNParam,
                              cudaMemcpyDeviceToHost, m->net.stream), "params");
  m->net.sync();
  MLP_END
}

int cacg_mlp_set_params(cacg_mlp m, int member, const float *p) {
  MLP_BEGIN
  need(p && member >= 0 && member < m->net.members, "bad member or array");
  cacg::check(cudaMemcpyAsync(m->net.mem[member].p.p, p, sizeof(float) * kNParam,
                              cudaMemcpyHostToDevice, m->net.stream), "params");
  m->net.refresh(member);
  m->net.sync();
  MLP_END
}

int cacg_mlp_set_normalization(cacg_mlp m, const float *in_mean, const float *in_std,
                               const float *out_mean, const float *out_std, double force_scale) {
  MLP_BEGIN
  need(in_mean && in_std && out_mean && out_std && force_scale > 0, "bad normalization");
  for (int i = 0; i < MLP_IN; i++) {
    need(in_std[i] > 0, "input std must be positive");
    m->net.norm[i] = in_mean[i];
    m->net.norm[MLP_IN + i] = 1.f / in_std[i];
  }
  for (int i = 0; i < MLP_OUT; i++) {
    need(out_std[i] > 0, "output std must be positive");
    m->net.norm[2 * MLP_IN + i] = out_mean[i];
    m->net.norm[2 * MLP_IN + MLP_OUT + i] = out_std[i];
  }
  m->net.force_scale = force_scale;
  m->net.upload_norm();
  m->net.sync();
  MLP_END
}

int cacg_mlp_get_normalization(cacg_mlp m, float *in_mean, float *in_std, float *out_mean,
                               float *out_std, double *force_scale) {
  MLP_BEGIN
  for (int i = 0; i < MLP_IN; i++) {
    if (in_mean) in_mean[i] = m->net.norm[i];
    if (in_std) in_std[i] = 1.f / m->net.norm[MLP_IN + i];
  }
  for (int i = 0; i < MLP_OUT; i++) {
    if (out_mean) out_mean[i] = m->net.norm[2 * MLP_IN + i];
    if (out_std) out_std[i] = m->net.norm[2 * MLP_IN + MLP_OUT + i];
  }
  if (force_scale) *force_scale = m->net.force_scale;
  MLP_END
}

int cacg_mlp_loss_grad(cacg_mlp m, int member, const float *x, const float *t, int n,
                       double *loss, float *grad) {
  MLP_BEGIN
  Net &N = m->net;
  need(x && t && n > 0 && member >= 0 && member < N.members, "bad arguments");
  const int B = (n + 127) / 128 * 128;
  N.ensure_batch(B);
  cacg::DBuf<bf16> xf;
  cacg::DBuf<float> tf;
  upload_set(N, x, t, n, xf, tf);
  cacg::check(cudaMemsetAsync(N.x0.p, 0, sizeof(bf16) * (size_t) B * 64, N.stream), "x0");
  cacg::check(cudaMemsetAsync(N.tb.p, 0, sizeof(float) * (size_t) B * MLP_OUT, N.stream), "tb");
  cacg::check(cudaMemcpyAsync(N.x0.p, xf.p, sizeof(bf16) * (size_t) n * 64, cudaMemcpyDeviceToDevice, N.stream), "x0");
  cacg::check(cudaMemcpyAsync(N.tb.p, tf.p, sizeof(float) * (size_t) n * MLP_OUT, cudaMemcpyDeviceToDevice, N.stream), "tb");
  N.forward_train(member, B);
  double l = N.backward(member, B, n, true);
  N.check_err();
  if (loss) *loss = l;
  if (grad) {
    cacg::check(cudaMemcpyAsync(grad, N.mem[member].g.p, sizeof(float) * kNParam,
                                cudaMemcpyDeviceToHost, N.stream), "grad");
    N.sync();
  }
  xf.release();
  tf.release();
  MLP_END
}

int cacg_mlp_train(cacg_mlp m, const float *x, const float *t, long long n, int epochs, int batch,
                   float lr, unsigned long long seed, double *epoch_loss) {
  MLP_BEGIN
  Net &N = m->net;
  need(x && t && epochs > 0 && batch >= 128 && batch % 128 == 0 && n >= batch && lr > 0,
       "bad training arguments (batch a positive multiple of 128, n >= batch)");
  N.ensure_batch(batch);
  cacg::DBuf<bf16> xf;
  cacg::DBuf<float> tf;
  upload_set(N, x, t, n, xf, tf);
  cacg::DBuf<int> didx;
  const long long nbatch = n / batch;  // whole batches only
  didx.ensure((size_t) batch * std::max<long long>(nbatch, 1), N.stream);
  cacg::mlp::Rng rng{seed};
  std::vector<int> perm(n);
  for (int ep = 0; ep < epochs; ep++) {
    // cosine schedule from lr to lr/20
    const float lr_ep = (float) (lr * (0.05 + 0.95 * 0.5 * (1 + std::cos(M_PI * ep / epochs))));
    double lsum = 0.0;
    for (int k = 0; k < N.members; k++) {
      for (long long i = 0; i < n; i++) perm[i] = (int) i;
      for (long long i = n - 1; i > 0; i--) std::swap(perm[i], perm[rng.next() % (unsigned long long) (i + 1)]);
      cacg::check(cudaMemcpyAsync(didx.p, perm.data(), sizeof(int) * batch * nbatch,
                                  cudaMemcpyHostToDevice, N.stream), "perm");
      for (long long b = 0; b < nbatch; b++) {
        cacg::mlp::gather(xf.p, tf.p, didx.p + b * batch, batch, N.x0.p, N.tb.p, N.stream);
        N.forward_train(k, batch);
        bool last = ep == epochs - 1 && epoch_loss;
        double l = N.backward(k, batch, batch, last);
        lsum += l;
        N.adam(k, lr_ep);
      }
      N.sync();  // perm is reused for the next member
    }
    N.adam_steps += nbatch;
    if (epoch_loss && ep == epochs - 1) *epoch_loss = lsum / (double) (N.members * nbatch);
  }
  N.check_err();
  xf.release();
  tf.release();
  didx.release();
  MLP_END
}

int cacg_mlp_predict(cacg_mlp m, const float *x, long long n, float *mean, float *spread) {
  MLP_BEGIN
  Net &N = m->net;
  need(x && n > 0 && (mean || spread), "bad arguments");
  cacg::DBuf<bf16> xf;
  cacg::DBuf<float> tf, dm, ds;
  upload_set(N, x, nullptr, n, xf, tf);
  dm.ensure((size_t) n * MLP_OUT, N.stream);
  ds.ensure((size_t) n, N.stream);
  N.ensure_err(N.stream);
  N.predict_device(xf.p, n, dm.p, ds.p, N.stream);
  N.check_err();
  if (mean)
    cacg::check(cudaMemcpyAsync(mean, dm.p, sizeof(float) * n * MLP_OUT, cudaMemcpyDeviceToHost, N.stream), "mean");
  if (spread)
    cacg::check(cudaMemcpyAsync(spread, ds.p, sizeof(float) * n, cudaMemcpyDeviceToHost, N.stream), "spread");
  N.sync();
  xf.release();
  dm.release();
  ds.release();
  MLP_END
}

int cacg_gemm_bf16_tn(const void *a, int lda, const void *b, int ldb, float *c, int ldc, int m_,
                      int n_, int k_, int *err, void *stream) {
  if (!a || !b || !c || !err || m_ <= 0 || n_ <= 0 || k_ <= 0 || ldc < n_) return CACG_EINVAL;
  try {
    cacg::gemm::gemm_tn(a, lda, b, ldb, m_, n_, k_, 0, nullptr, c, ldc, nullptr, 0, err,
                        static_cast<cudaStream_t>(stream));
  } catch (const CudaError &e) {
    return e.code == cudaErrorInvalidValue ? CACG_EINVAL : CACG_ECUDA;
  }
  return CACG_OK;
}

}  // extern "C"
