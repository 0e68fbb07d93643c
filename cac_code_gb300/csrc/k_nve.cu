// Velocity-Verlet for atoms and element nodes, rebuild check and element-size
// reduction (sm_103a).  Compiled without contraction so the exact mode's
// updates are the reference's own multiply-then-add sequences (FixNVE,
// fix_nve.cpp:54-242); the other modes fuse them explicitly.
#include "internal.h"

namespace cacg {

namespace {

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

// dt/(2m) of a type: a select over constant indices, so that the table stays
// in the parameter space (a runtime index into a by-value parameter array
// would copy it to each thread's local memory)
__device__ __forceinline__ double type_scale(const TypeScale &t, int ty) {
  double d = t.v[0];
#pragma unroll
  for (int k = 1; k <= MAXT; k++) d = ty == k ? t.v[k] : d;
  return d;
}

// a + b * c: the reference's multiply-then-add, or one fused multiply-add in
// the FP64 (FMA) and mixed modes (FP64 instructions are scarce on this GPU:
// the integrators are bound by their FP64 issue, not by HBM)
template <bool FUSED>
__device__ __forceinline__ double madd(double a, double b, double c) {
  return FUSED ? fma(b, c, a) : a + b * c;
}

// FixNVE::initial_integrate, fix_nve.cpp:54-98 (per-type mass branch).  One
// thread per component, so the v and f loads of a warp are 256 contiguous
// bytes; x is the padded double4 array.
template <bool FUSED>
__global__ void k_nve_atoms_initial(double4 *__restrict__ x, double *__restrict__ v,
                                    const double *__restrict__ f, const int *__restrict__ type,
                                    TypeScale dtfm_t, int n, double dtv) {
  const long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x;
  if (t >= 3LL * n) return;
  const long long i = t / 3;
  const int d = (int) (t - 3 * i);
  const double vv = madd<FUSED>(v[t], type_scale(dtfm_t, type[i]), f[t]);
  v[t] = vv;
  double *xp = reinterpret_cast<double *>(x) + 4 * i + d;
  *xp = madd<FUSED>(*xp, dtv, vv);
}

// FixNVE::final_integrate, fix_nve.cpp:181-212 (one thread per component)
template <bool FUSED>
__global__ void k_nve_atoms_final(double *__restrict__ v, const double *__restrict__ f,
                                  const int *__restrict__ type, TypeScale dtfm_t, int n) {
  const long long t = blockIdx.x * (long long) blockDim.x + threadIdx.x;
  if (t >= 3LL * n) return;
  v[t] = madd<FUSED>(v[t], type_scale(dtfm_t, type[t / 3]), f[t]);
}

// FixNVE::einitial_integrate, fix_nve.cpp:100-157: nodal mass M_e/8, then the
// centre is recomputed as the mean of the nodes.  One thread per node for the
// update (its three components contiguous, so a warp's loads cover four
// elements' 768 bytes); the new positions of the block's 32 elements are
// staged in shared memory and one warp sums each element's nodes in node
// order, as the reference's loop adds them (one summing thread per element
// keeps the FP64 additions at 24 per element).
static_assert(NPE == 8, "eight nodes per element");
constexpr int NODE_BLOCK = 256, NODE_ELEMS = NODE_BLOCK / NPE;
template <bool FUSED>
__global__ void __launch_bounds__(NODE_BLOCK)
k_nve_nodes_initial(double *__restrict__ ex, double *__restrict__ nodex,
                    double *__restrict__ nodev, const double *__restrict__ nodef,
                    const int *__restrict__ etype, TypeScale dtfm_t, int n, double dtv) {
  __shared__ double sx[NODE_ELEMS][3 * NPE + 1];
  const long long t = blockIdx.x * (long long) NODE_BLOCK + threadIdx.x;
  const long long i = t >> 3;
  const int q = (int) (t & 7), le = threadIdx.x >> 3;
  if (i < n) {
    const double dtfm = type_scale(dtfm_t, etype[i]);
    for (int d = 0; d < 3; d++) {
      const size_t k = 24 * (size_t) i + 3 * q + d;
      const double vv = madd<FUSED>(nodev[k], dtfm, nodef[k]);
      nodev[k] = vv;
      const double xn = madd<FUSED>(nodex[k], dtv, vv);
      nodex[k] = xn;
      sx[le][3 * q + d] = xn;
    }
  }
  __syncthreads();
  const long long e = blockIdx.x * (long long) NODE_ELEMS + threadIdx.x;
  if (threadIdx.x < NODE_ELEMS && e < n) {
    for (int d = 0; d < 3; d++) {
      double c = 0.0;
      for (int r = 0; r < NPE; r++) c += sx[threadIdx.x][3 * r + d];
      ex[3 * e + d] = c / NPE;
    }
  }
}

// FixNVE::efinal_integrate, fix_nve.cpp:216-242
template <bool FUSED>
__global__ void k_nve_nodes_final(double *__restrict__ nodev, const double *__restrict__ nodef,
                                  const int *__restrict__ etype, TypeScale dtfm_t, int n) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 24) return;
  int i = t / 24;
  nodev[t] = madd<FUSED>(nodev[t], type_scale(dtfm_t, etype[i]), nodef[t]);
}

// Neighbor::check_distance, neighbor.cpp:1176-1217.  Bits of *flag: 1 an
// atom moved more than the trigger distance since its list build, 2 a node
// did since the element list build, 4 an element centre lies outside the box
// in a periodic dimension (Domain::elepbc would wrap it).
// With gate (the device step loop's state, gate[0] = steps since setup before
// this one), the kernel returns at once unless this step reaches a decision.
__global__ void k_check_distance(const double4 *__restrict__ x, const double *__restrict__ xh,
                                 int n, const double *__restrict__ nodex,
                                 const double *__restrict__ nodexh, int ne,
                                 const double *__restrict__ ex, BoxWrap box, double triggersq,
                                 int *__restrict__ flag, const int *__restrict__ gate, int every,
                                 int delay) {
  if (gate) {
    const int ago = gate[0] + 1;
    if (ago < delay || ago % every != 0) return;  // uniform over the grid
  }
  const long long t = (long long) blockIdx.x * blockDim.x + threadIdx.x;
  const long long nn = (long long) ne * NPE;
  int bit = 0;
  if (t < n) {
    double4 p = x[t];
    double dx = p.x - xh[3 * t], dy = p.y - xh[3 * t + 1], dz = p.z - xh[3 * t + 2];
    if (dx * dx + dy * dy + dz * dz > triggersq) bit = 1;
  } else if (t < n + nn) {
    size_t k = 3 * (size_t) (t - n);
    double dx = nodex[k] - nodexh[k], dy = nodex[k + 1] - nodexh[k + 1],
           dz = nodex[k + 2] - nodexh[k + 2];
    if (dx * dx + dy * dy + dz * dz > triggersq) bit = 2;
  } else if (ex && t < n + nn + ne) {
    const size_t e = (size_t) (t - n - nn);
#pragma unroll
    for (int d = 0; d < 3; d++) {
      const double c = ex[3 * e + d];
      if (box.periodic[d] && (c < box.lo[d] || c >= box.hi[d])) bit = 4;
    }
  }
  const unsigned m = __reduce_or_sync(0xffffffffu, (unsigned) bit);
  if (m && (threadIdx.x & 31) == 0) atomicOr(flag, (int) m);
}

__global__ void k_hold_atoms(const double4 *__restrict__ x, double *__restrict__ xh, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = x[i];
  xh[3 * i] = p.x;
  xh[3 * i + 1] = p.y;
  xh[3 * i + 2] = p.z;
}

// Per-element longest body diagonal (Element::element_size, element.cpp:567-625)
// and the centre-versus-node-mean check (element.cpp:608-622).
__global__ void k_elem_diag(const double *__restrict__ nodex, const double *__restrict__ ex,
                            int n, double *__restrict__ diag, int *__restrict__ bad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double *nx = nodex + 24 * (size_t) i;
  double length = 0.0;
  for (int j = 0; j < 4; j++) {
    int o = j < 2 ? j + 6 : j + 2;
    double lx = nx[3 * j] - nx[3 * o], ly = nx[3 * j + 1] - nx[3 * o + 1],
           lz = nx[3 * j + 2] - nx[3 * o + 2];
    double l = sqrt(lx * lx + ly * ly + lz * lz);
    length = length > l ? length : l;
  }
  diag[i] = length;
  double c[3] = {0.0, 0.0, 0.0};
  for (int q = 0; q < NPE; q++)
    for (int d = 0; d < 3; d++) c[d] += nx[3 * q + d];
  for (int d = 0; d < 3; d++) c[d] = c[d] / NPE;
  double dist = (c[0] - ex[3 * i]) * (c[0] - ex[3 * i]) +
                (c[1] - ex[3 * i + 1]) * (c[1] - ex[3 * i + 1]) +
                (c[2] - ex[3 * i + 2]) * (c[2] - ex[3 * i + 2]);
  if (dist > 0.01) atomicAdd(bad, 1);
}

// [n][3] <-> double4 layout changes for host transfers, done on the device so
// that a host-resident caller moves plain arrays with one DMA each way
__global__ void k_pack3to4(const double *__restrict__ in, double4 *__restrict__ out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = make_double4(in[3 * i], in[3 * i + 1], in[3 * i + 2], 0.0);
}

__global__ void k_unpack4to3(const double4 *__restrict__ in, double *__restrict__ out, int n) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = in[i];
  out[3 * i] = p.x;
  out[3 * i + 1] = p.y;
  out[3 * i + 2] = p.z;
}

// Dependent chains of FP64 fused multiply-adds: 8 independent chains per
// thread keep the FP64 pipe busy; the result is written so nothing is elided.
__global__ void k_fma_loop(double *out, int iters) {
  double a0 = threadIdx.x * 1e-9, a1 = a0 + 1e-9, a2 = a0 + 2e-9, a3 = a0 + 3e-9;
  double a4 = a0 + 4e-9, a5 = a0 + 5e-9, a6 = a0 + 6e-9, a7 = a0 + 7e-9;
  const double b = 0.999999, c = 1e-7;
  for (int k = 0; k < iters; k++) {
    a0 = fma(a0, b, c); a1 = fma(a1, b, c); a2 = fma(a2, b, c); a3 = fma(a3, b, c);
    a4 = fma(a4, b, c); a5 = fma(a5, b, c); a6 = fma(a6, b, c); a7 = fma(a7, b, c);
  }
  out[blockIdx.x * blockDim.x + threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

}  // namespace

void launch_nve_atoms_initial(double4 *x, double *v, const double *f, const int *type,
                              const TypeScale &dtfm, int n, double dtv, bool fused,
                              cudaStream_t s) {
  if (n <= 0) return;
  auto k = fused ? k_nve_atoms_initial<true> : k_nve_atoms_initial<false>;
  k<<<nblk(3LL * n, 256), 256, 0, s>>>(x, v, f, type, dtfm, n, dtv);
  check(cudaGetLastError(), "nve_atoms_initial");
}

void launch_nve_atoms_final(double *v, const double *f, const int *type, const TypeScale &dtfm,
                            int n, bool fused, cudaStream_t s) {
  if (n <= 0) return;
  auto k = fused ? k_nve_atoms_final<true> : k_nve_atoms_final<false>;
  k<<<nblk(3LL * n, 256), 256, 0, s>>>(v, f, type, dtfm, n);
  check(cudaGetLastError(), "nve_atoms_final");
}

void launch_nve_nodes_initial(double *ex, double *nodex, double *nodev, const double *nodef,
                              const int *etype, const TypeScale &dtfm, int n, double dtv,
                              bool fused, cudaStream_t s) {
  if (n <= 0) return;
  auto k = fused ? k_nve_nodes_initial<true> : k_nve_nodes_initial<false>;
  k<<<nblk((long long) n * NPE, NODE_BLOCK), NODE_BLOCK, 0, s>>>(ex, nodex, nodev, nodef, etype,
                                                                  dtfm, n, dtv);
  check(cudaGetLastError(), "nve_nodes_initial");
}

void launch_nve_nodes_final(double *nodev, const double *nodef, const int *etype,
                            const TypeScale &dtfm, int n, bool fused, cudaStream_t s) {
  if (n <= 0) return;
  auto k = fused ? k_nve_nodes_final<true> : k_nve_nodes_final<false>;
  k<<<nblk((long long) n * 24, 256), 256, 0, s>>>(nodev, nodef, etype, dtfm, n);
  check(cudaGetLastError(), "nve_nodes_final");
}

void launch_check_distance(const double4 *x, const double *xhold, int n,
                           const double *nodex, const double *nodexhold, int ne,
                           const double *ex, const BoxWrap &box, double triggersq, int *flag,
                           cudaStream_t s) {
  long long tot = (long long) n + (long long) ne * NPE + (ex ? ne : 0);
  if (tot <= 0) return;
  k_check_distance<<<nblk(tot, 256), 256, 0, s>>>(x, xhold, n, nodex, nodexhold, ne, ex, box,
                                                   triggersq, flag, nullptr, 1, 0);
  check(cudaGetLastError(), "check_distance");
}

void launch_loop_check(const double4 *x, const double *xhold, int n, const double *nodex,
                       const double *nodexhold, int ne, const double *ex, const BoxWrap &box,
                       double triggersq, int *loop, int every, int delay, cudaStream_t s) {
  long long tot = (long long) n + (long long) ne * NPE + (ex ? ne : 0);
  if (tot <= 0) return;
  k_check_distance<<<nblk(tot, 256), 256, 0, s>>>(x, xhold, n, nodex, nodexhold, ne, ex, box,
                                                   triggersq, loop + LOOP_BITS, loop, every, delay);
  check(cudaGetLastError(), "loop check");
}

// Neighbor::decide (neighbor.cpp:1150-1163) inside the device step loop: one
// thread.  ago counts steps since setup (not reset by a rebuild); a decision
// step whose check found an atom or a node past the trigger (or any decision
// step without the check) ends the loop before the step's force passes, with
// the flags left for the host's rebuild; any other step runs on and counts
// as done.  The loop also ends when the wanted steps are done, and never runs
// more iterations than steps wanted.
__global__ void k_loop_decide(int *__restrict__ loop, int every, int delay, int dist_check,
                              cudaGraphConditionalHandle again, cudaGraphConditionalHandle proceed) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int ago = loop[LOOP_AGO] + 1;
  const int it = loop[LOOP_ITERS] + 1;
  loop[LOOP_AGO] = ago;
  loop[LOOP_ITERS] = it;
  int flags = 0;
  if (ago >= delay && ago % every == 0) {
    if (!dist_check) {
      flags = 1;
    } else {
      const int b = loop[LOOP_BITS];
      flags = (b & 3) ? b : 0;  // a wrap alone needs no rebuild
    }
    loop[LOOP_BITS] = 0;
  }
  if (flags) {
    loop[LOOP_PENDING] = flags;
    cudaGraphSetConditional(proceed, 0u);
    cudaGraphSetConditional(again, 0u);
    return;
  }
  const int done = loop[LOOP_DONE] + 1;
  loop[LOOP_DONE] = done;
  cudaGraphSetConditional(proceed, 1u);
  cudaGraphSetConditional(again, (done < loop[LOOP_WANT] && it < loop[LOOP_WANT]) ? 1u : 0u);
}

void launch_loop_decide(int *loop, int every, int delay, int dist_check,
                        cudaGraphConditionalHandle again, cudaGraphConditionalHandle proceed,
                        cudaStream_t s) {
  k_loop_decide<<<1, 32, 0, s>>>(loop, every, delay, dist_check, again, proceed);
  check(cudaGetLastError(), "loop decide");
}

void launch_hold_atoms(const double4 *x, double *xhold, int n, cudaStream_t s) {
  if (n <= 0) return;
  k_hold_atoms<<<nblk(n, 256), 256, 0, s>>>(x, xhold, n);
  check(cudaGetLastError(), "hold_atoms");
}

void launch_elem_diag(const double *nodex, const double *ex, int n, double *diag,
                      int *centre_bad, cudaStream_t s) {
  if (n <= 0) return;
  k_elem_diag<<<nblk(n, 128), 128, 0, s>>>(nodex, ex, n, diag, centre_bad);
  check(cudaGetLastError(), "elem_diag");
}

void launch_pack3to4(const double *in, double4 *out, int n, cudaStream_t s) {
  if (n <= 0) return;
  k_pack3to4<<<nblk(n, 256), 256, 0, s>>>(in, out, n);
  check(cudaGetLastError(), "pack3to4");
}

void launch_unpack4to3(const double4 *in, double *out, int n, cudaStream_t s) {
  if (n <= 0) return;
  k_unpack4to3<<<nblk(n, 256), 256, 0, s>>>(in, out, n);
  check(cudaGetLastError(), "unpack4to3");
}

namespace {
__global__ void k_setforce(double *__restrict__ f, const int *__restrict__ mask, int n, int per,
                           int bit, int sx, int sy, int sz, double vx, double vy, double vz) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * per || !(mask[i / per] & bit)) return;
  if (sx) f[3 * (size_t) i] = vx;
  if (sy) f[3 * (size_t) i + 1] = vy;
  if (sz) f[3 * (size_t) i + 2] = vz;
}

__global__ void k_viscous(double *__restrict__ f, const double *__restrict__ v,
                          const int *__restrict__ mask, int n, int per, int bit, double drag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * per || !(mask[i / per] & bit)) return;
  for (int d = 0; d < 3; d++) f[3 * (size_t) i + d] -= drag * v[3 * (size_t) i + d];
}
__global__ void k_affine(double *__restrict__ x, int n, int stride, double olo, double nlo,
                         double f) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) x[(size_t) i * stride] = nlo + (x[(size_t) i * stride] - olo) * f;
}
}  // namespace

void launch_affine(double *x, int n, int stride, double olo, double nlo, double f, cudaStream_t s) {
  if (n <= 0) return;
  k_affine<<<nblk(n, 256), 256, 0, s>>>(x, n, stride, olo, nlo, f);
  check(cudaGetLastError(), "affine");
}

void launch_setforce(double *f, const int *mask, int n, int per_item, int bit, const int *set,
                     const double *val, cudaStream_t s) {
  if (n <= 0) return;
  k_setforce<<<nblk((long long) n * per_item, 256), 256, 0, s>>>(f, mask, n, per_item, bit, set[0], set[1],
                                                              set[2], val[0], val[1], val[2]);
  check(cudaGetLastError(), "setforce");
}

void launch_viscous(double *f, const double *v, const int *mask, int n, int per_item, int bit,
                    double gamma, cudaStream_t s) {
  if (n <= 0) return;
  k_viscous<<<nblk((long long) n * per_item, 256), 256, 0, s>>>(f, v, mask, n, per_item, bit, gamma);
  check(cudaGetLastError(), "viscous");
}

double fp64_fma_rate(cudaStream_t s) {
  int dev = 0;
  check(cudaGetDevice(&dev), "getdevice");
  int nsm = 0;
  check(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev), "attr");
  const int threads = 256, blocks = nsm * 8, iters = 4096;
  double *out = nullptr;
  check(cudaMalloc(&out, sizeof(double) * threads * blocks), "malloc fma");
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  k_fma_loop<<<blocks, threads, 0, s>>>(out, iters);  // warm-up
  cudaEventRecord(a, s);
  k_fma_loop<<<blocks, threads, 0, s>>>(out, iters);
  cudaEventRecord(b, s);
  check(cudaEventSynchronize(b), "fma sync");
  float ms = 0;
  cudaEventElapsedTime(&ms, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(out);
  double flops = 2.0 * 8.0 * (double) iters * threads * blocks;
  return ms > 0 ? flops / (ms * 1e-3) : 0.0;
}

}  // namespace cacg
