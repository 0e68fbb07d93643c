// Kinetic-energy sums without any device allocation.
//
// A variant of the kinetic kernel in k_thermo.cu for callers that may not
// allocate device memory at the point of the call: a host MD driver that
// reports thermo from its per-step output hook (cudaMalloc and cudaFree
// synchronise the whole device and would stall the step pipeline), or a
// driver whose device memory is already reserved by another framework's
// caching allocator, so that a fresh allocation fails or evicts its pool.
// The handle-based cacg_compute_thermo grows a per-handle buffer for its
// per-block partial sums; this entry point keeps them in a fixed file-scope
// device array instead and reduces them on the device, so it calls neither
// cudaMalloc nor cudaFree nor any library that allocates.
//
// Scratch: NOALLOC_MAX_BLOCKS blocks x 7 partial sums (448 KiB).  One block
// covers 256 items, so n is limited to CACG_NOALLOC_MAX_ITEMS; a larger n is
// rejected with CACG_ESCRATCH before anything is launched.
//
// Nothing in the scratch has to start at zero: the first kernel writes every
// partial slot the second one reads, and the second one stores out[] rather
// than adding to it.
//
// All calls on one device share the one scratch array.  Calls that can
// overlap (different streams, or different host threads, with no ordering
// between them) overwrite each other's partial sums: serialise them on one
// stream or with events.
//
// The scratch address is resolved once per device ordinal, with that device
// current, by cudaGetSymbolAddress on the first call, and cached: it belongs
// to the device's primary context, so it does not survive cudaDeviceReset and
// does not serve a caller that made another context current.  Make that first
// call (n = 0 is enough) before any stream capture begins.
//
// A CUDA error left pending by earlier, unrelated work is reported
// (CACG_ECUDA) and left in place for its owner; the call then launches
// nothing.
#include <mutex>

#include "cacg.h"
#include "internal.h"

constexpr int NOALLOC_TB = 256;
constexpr int NOALLOC_NQ = 7;  // energy, m vx vx, m vy vy, m vz vz, m vx vy, m vx vz, m vy vz
constexpr int NOALLOC_MAX_BLOCKS = CACG_NOALLOC_MAX_ITEMS / NOALLOC_TB;
constexpr int NOALLOC_MAX_DEVICES = 64;

static_assert(CACG_NOALLOC_MAX_ITEMS % NOALLOC_TB == 0, "scratch holds whole blocks");

// 8192 blocks x 7 doubles = 458,752 bytes
static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_MAX_BLOCKS * NOALLOC_NQ];

namespace {

std::mutex g_noalloc_mu;
double *g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// per-block partial sums of 1/2 m v^2 and m v_a v_b (mass by type of item / per_item)
__global__ void __launch_bounds__(NOALLOC_TB)
k_kinetic_partials(const double *__restrict__ v, const int *__restrict__ type,
                   const double *__restrict__ mass, int n, int per_item, double scale,
                   double *__restrict__ part) {
  __shared__ double sh[NOALLOC_NQ][NOALLOC_TB / 32];
  double q[NOALLOC_NQ] = {0, 0, 0, 0, 0, 0, 0};
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) {
    const double m = mass[type[i / per_item]] * scale;
    const double vx = v[3 * i], vy = v[3 * i + 1], vz = v[3 * i + 2];
    q[0] = 0.5 * m * (vx * vx + vy * vy + vz * vz);
    q[1] = m * vx * vx;
    q[2] = m * vy * vy;
    q[3] = m * vz * vz;
    q[4] = m * vx * vy;
    q[5] = m * vx * vz;
    q[6] = m * vy * vz;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NOALLOC_NQ; k++) {
    double s = q[k];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) sh[k][wid] = s;
  }
  __syncthreads();
  if (threadIdx.x < NOALLOC_NQ) {
    double s = 0.0;
    for (int w = 0; w < NOALLOC_TB / 32; w++) s += sh[threadIdx.x][w];
    part[(size_t) blockIdx.x * NOALLOC_NQ + threadIdx.x] = s;
  }
}

// out[k] = mvv2e * (the partials of quantity k summed): one block, each
// thread sums a stride of the partials, then a tree over the threads
constexpr int NOALLOC_FINISH = 256;

__global__ void __launch_bounds__(NOALLOC_FINISH)
k_kinetic_finish(const double *__restrict__ part, int nblocks, double mvv2e,
                 double *__restrict__ out) {
  __shared__ double sh[NOALLOC_NQ][NOALLOC_FINISH];
  double q[NOALLOC_NQ] = {0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += NOALLOC_FINISH)
#pragma unroll
    for (int k = 0; k < NOALLOC_NQ; k++) q[k] += part[(size_t) b * NOALLOC_NQ + k];
#pragma unroll
  for (int k = 0; k < NOALLOC_NQ; k++) sh[k][threadIdx.x] = q[k];
  __syncthreads();
  for (int w = NOALLOC_FINISH / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
#pragma unroll
      for (int k = 0; k < NOALLOC_NQ; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x < NOALLOC_NQ) out[threadIdx.x] = sh[threadIdx.x][0] * mvv2e;
}

// the scratch address on the current device, resolved once per device
int noalloc_scratch(double **ptr) {
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return CACG_ECUDA;
  std::lock_guard<std::mutex> lock(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return CACG_ECUDA;
    g_noalloc_ptr[dev] = static_cast<double *>(p);
  }
  *ptr = g_noalloc_ptr[dev];
  return CACG_OK;
}

}  // namespace

extern "C" int cacg_kinetic_noalloc(const double *v, const int *type, const double *mass, int n,
                                    int per_item, double scale, double mvv2e, double *out,
                                    void *stream) {
  if (n < 0 || per_item < 1 || !out || (n > 0 && (!v || !type || !mass))) return CACG_EINVAL;
  if (n > CACG_NOALLOC_MAX_ITEMS) return CACG_ESCRATCH;
  // an error pending from earlier work is its owner's: report it, keep it
  if (cudaPeekAtLastError() != cudaSuccess) return CACG_ECUDA;
  double *part = nullptr;
  int rc = noalloc_scratch(&part);
  if (rc != CACG_OK) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int nblocks = (n + NOALLOC_TB - 1) / NOALLOC_TB;
  if (nblocks > 0)
    k_kinetic_partials<<<nblocks, NOALLOC_TB, 0, s>>>(v, type, mass, n, per_item, scale, part);
  k_kinetic_finish<<<1, NOALLOC_FINISH, 0, s>>>(part, nblocks, mvv2e, out);
  // nothing was pending before the launches: an error now is theirs
  return cudaGetLastError() == cudaSuccess ? CACG_OK : CACG_ECUDA;
}
