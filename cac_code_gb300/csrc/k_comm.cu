// Ghost images, periodic wrap, binning and scans (sm_103a).
//
// The reference builds ghosts with six sequential slab swaps per rebuild
// (CommBrick::borders, comm_brick.cpp:641-914) and refreshes them every step
// with the same swap chain (forward_comm, comm_brick.cpp:1051-1112).  Here a
// swap is a stable stream compaction over the source range followed by an
// append, so ghost k lands at the same index as in the reference and keeps
// the reference's x + pbc*prd arithmetic.  Bins are a counting sort whose
// members are re-sorted by index, reproducing the forward-linked bin lists of
// Neighbor::bin_atoms (neighbor.cpp:656-674).
#include "internal.h"

namespace cacg {

namespace {

constexpr int SCAN_THREADS = 512;
constexpr int SCAN_ITEMS = 4;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int warp_incl_scan(int v) {
  const unsigned lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, v, o);
    if (lane >= (unsigned) o) v += t;
  }
  return v;
}

// Exclusive scan of one tile per block; block totals to sums[blockIdx.x].
__global__ void k_scan_tile(const int *__restrict__ in, int *__restrict__ out, int n,
                            int *__restrict__ sums) {
  __shared__ int warp_tot[SCAN_THREADS / 32];
  const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int run = 0;
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    int idx = base + k;
    v[k] = idx < n ? in[idx] : 0;
    run += v[k];
  }
  int incl = warp_incl_scan(run);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 31) warp_tot[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    int t = lane < SCAN_THREADS / 32 ? warp_tot[lane] : 0;
    t = warp_incl_scan(t);
    if (lane < SCAN_THREADS / 32) warp_tot[lane] = t;
  }
  __syncthreads();
  int excl = incl - run + (wid > 0 ? warp_tot[wid - 1] : 0);
#pragma unroll
  for (int k = 0; k < SCAN_ITEMS; k++) {
    int idx = base + k;
    if (idx < n) out[idx] = excl;
    excl += v[k];
  }
  if (threadIdx.x == SCAN_THREADS - 1) sums[blockIdx.x] = warp_tot[SCAN_THREADS / 32 - 1];
}

__global__ void k_add_offsets(int *__restrict__ out, int n, const int *__restrict__ offs) {
  int idx = blockIdx.x * SCAN_TILE + threadIdx.x;
  int add = offs[blockIdx.x];
  for (int k = 0; k < SCAN_ITEMS; k++, idx += SCAN_THREADS)
    if (idx < n) out[idx] += add;
}

__global__ void k_total(const int *in, const int *out, int n, int *total) {
  *total = n > 0 ? out[n - 1] + in[n - 1] : 0;
}

void scan_rec(const int *in, int *out, int n, DBuf<int> &scratch, size_t off,
              cudaStream_t s) {
  int nb = (n + SCAN_TILE - 1) / SCAN_TILE;
  if (nb < 1) nb = 1;
  int *sums = scratch.p + off;
  int *sums_scan = sums + nb;
  k_scan_tile<<<nb, SCAN_THREADS, 0, s>>>(in, out, n, sums);
  if (nb > 1) {
    scan_rec(sums, sums_scan, nb, scratch, off + 2 * (size_t) nb, s);
    k_add_offsets<<<nb, SCAN_THREADS, 0, s>>>(out, n, sums_scan);
  }
}

}  // namespace

void scan_exclusive(const int *in, int *out, int n, int *total, DBuf<int> &scratch,
                    cudaStream_t s) {
  // scratch: 2*nb per level, geometric
  size_t need = 0, m = (size_t) n;
  do {
    size_t nb = (m + SCAN_TILE - 1) / SCAN_TILE;
    if (nb < 1) nb = 1;
    need += 2 * nb;
    m = nb;
  } while (m > 1);
  scratch.ensure(need + 16, s);
  if (n > 0) scan_rec(in, out, n, scratch, 0, s);
  if (total) k_total<<<1, 1, 0, s>>>(in, out, n, total);
  check(cudaGetLastError(), "scan");
}

// ------------------------------------------------------------------ borders

namespace {

__global__ void k_border_flags_atoms(const double4 *__restrict__ x, int nfirst, int nlast,
                                     int dim, double lo, double hi, int *__restrict__ flags) {
  int i = nfirst + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlast) return;
  double4 p = x[i];
  double c = dim == 0 ? p.x : (dim == 1 ? p.y : p.z);
  flags[i - nfirst] = (c >= lo && c <= hi) ? 1 : 0;
}

struct TypeSlabs {
  double lo[MAXT + 1], hi[MAXT + 1];
};

__global__ void k_border_flags_elems(const double *__restrict__ ex, const int *__restrict__ et,
                                     int nfirst, int nlast, int dim, TypeSlabs sl,
                                     int *__restrict__ flags) {
  int i = nfirst + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlast) return;
  double c = ex[3 * i + dim];
  int t = et[i];
  flags[i - nfirst] = (c >= sl.lo[t] && c <= sl.hi[t]) ? 1 : 0;
}

__global__ void k_border_scatter_atoms(double4 *__restrict__ x, int *__restrict__ type,
                                       int *__restrict__ tag, int *__restrict__ root,
                                       int *__restrict__ sendlist,
                                       const int *__restrict__ flags,
                                       const int *__restrict__ pos, int nfirst, int nlast,
                                       int n0, double dx, double dy, double dz) {
  int i = nfirst + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlast) return;
  int k = i - nfirst;
  if (!flags[k]) return;
  int m = pos[k];
  int g = n0 + m;
  double4 p = x[i];
  // AtomVecAtomic::pack_border: x + dx with dx = pbc*prd (atom_vec_atomic.cpp:212-214)
  p.x = p.x + dx;
  p.y = p.y + dy;
  p.z = p.z + dz;
  x[g] = p;
  type[g] = type[i];
  tag[g] = tag[i];
  root[g] = root[i];
  sendlist[m] = i;
}

__global__ void k_border_scatter_elems(double *__restrict__ ex, double *__restrict__ nodex,
                                       int *__restrict__ et, int *__restrict__ etag,
                                       int *__restrict__ eroot, int *__restrict__ sendlist,
                                       const int *__restrict__ flags,
                                       const int *__restrict__ pos, int nfirst, int nlast,
                                       int n0, double dx, double dy, double dz) {
  int i = nfirst + blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlast) return;
  int k = i - nfirst;
  if (!flags[k]) return;
  int m = pos[k];
  int g = n0 + m;
  const double d[3] = {dx, dy, dz};
  // Element::pack_border: centre and every node + pbc*prd (element.cpp:923-955)
  for (int c = 0; c < 3; c++) ex[3 * g + c] = ex[3 * i + c] + d[c];
  for (int q = 0; q < NPE; q++)
    for (int c = 0; c < 3; c++) nodex[24 * g + 3 * q + c] = nodex[24 * i + 3 * q + c] + d[c];
  et[g] = et[i];
  etag[g] = etag[i];
  eroot[g] = eroot[i];
  sendlist[m] = i;
}

__global__ void k_forward_atoms(double4 *__restrict__ x, const int *__restrict__ send, int n,
                                int first, double dx, double dy, double dz) {
  int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= n) return;
  double4 p = x[send[m]];
  p.x = p.x + dx;
  p.y = p.y + dy;
  p.z = p.z + dz;
  x[first + m] = p;
}

__global__ void k_forward_elems(double *__restrict__ nodex, const int *__restrict__ send, int n,
                                int first, double dx, double dy, double dz) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n * 24) return;
  int m = t / 24, r = t % 24;
  int c = r % 3;
  double d = c == 0 ? dx : (c == 1 ? dy : dz);
  nodex[24 * (first + m) + r] = nodex[24 * send[m] + r] + d;
}

// All swaps of a forward communication in one launch: each ghost follows its
// chain of sources back to the owned item (ghost g was sent from
// send[g - nfirst], an owned item or an earlier swap's ghost) and applies the
// swaps' shifts in the order the swaps ran, so every ghost value is the same
// sum of the same doubles as swap-by-swap communication.
__device__ __forceinline__ int swap_of(const SwapChain &c, int g) {
  int w = 0;
  for (int k = 1; k < c.n; k++)
    if (g >= c.first[k]) w = k;
  return w;
}

__global__ void k_forward_atoms_all(double4 *__restrict__ x, const int *__restrict__ send,
                                    int nlocal, int nghost, SwapChain c) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nghost) return;
  int chain[MAX_SWAPS], depth = 0, src = nlocal + t;
  while (src >= nlocal && depth < MAX_SWAPS) {
    chain[depth++] = swap_of(c, src);
    src = send[src - nlocal];
  }
  double4 p = x[src];
  for (int k = depth - 1; k >= 0; k--) {
    const int w = chain[k];
    p.x = p.x + c.d[w][0];
    p.y = p.y + c.d[w][1];
    p.z = p.z + c.d[w][2];
  }
  x[nlocal + t] = p;
}

__global__ void k_forward_elems_all(double *__restrict__ nodex, const int *__restrict__ send,
                                    int nlocal, int nghost, SwapChain c) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nghost * 24) return;
  const int m = t / 24, r = t % 24, dim = r % 3;
  int chain[MAX_SWAPS], depth = 0, src = nlocal + m;
  while (src >= nlocal && depth < MAX_SWAPS) {
    chain[depth++] = swap_of(c, src);
    src = send[src - nlocal];
  }
  double v = nodex[24 * (size_t) src + r];
  for (int k = depth - 1; k >= 0; k--) v = v + c.d[chain[k]][dim];
  nodex[24 * (size_t) (nlocal + m) + r] = v;
}

template <class T>
__global__ void k_copy_root(T *__restrict__ a, int width, const int *__restrict__ root, int gfirst,
                            int gn) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= gn * width) return;
  int g = gfirst + t / width, c = t % width;
  a[(size_t) g * width + c] = a[(size_t) root[g] * width + c];
}

struct Box {
  double lo[3], hi[3], prd[3];
  int per[3];
};

// Domain::pbc for periodic dims, domain.cpp:535-645
__global__ void k_pbc_atoms(double4 *__restrict__ x, int n, Box b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = x[i];
  double c[3] = {p.x, p.y, p.z};
  for (int d = 0; d < 3; d++) {
    if (!b.per[d]) continue;
    if (c[d] < b.lo[d]) c[d] += b.prd[d];
    if (c[d] >= b.hi[d]) {
      c[d] -= b.prd[d];
      c[d] = c[d] > b.lo[d] ? c[d] : b.lo[d];
    }
  }
  p.x = c[0];
  p.y = c[1];
  p.z = c[2];
  x[i] = p;
}

// Domain::elepbc, domain.cpp:647-745, periodic dims; nodes move with the centre
__global__ void k_pbc_elems(double *__restrict__ ex, double *__restrict__ nodex, int n, Box b) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  for (int d = 0; d < 3; d++) {
    if (!b.per[d]) continue;
    double c = ex[3 * i + d];
    if (c < b.lo[d]) {
      c += b.prd[d];
      for (int q = 0; q < NPE; q++) nodex[24 * i + 3 * q + d] += b.prd[d];
    }
    if (c >= b.hi[d]) {
      c -= b.prd[d];
      for (int q = 0; q < NPE; q++) nodex[24 * i + 3 * q + d] -= b.prd[d];
      c = c > b.lo[d] ? c : b.lo[d];
    }
    ex[3 * i + d] = c;
  }
}

// Neighbor::coord2bin, neighbor.cpp:688-717
__device__ __forceinline__ int coord2bin(double x, double y, double z, const BinGeom &g) {
  const double c[3] = {x, y, z};
  int ix[3];
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (c[d] >= g.hi[d]) ix[d] = (int) ((c[d] - g.hi[d]) * g.bininv[d]) + g.nbin[d];
    else if (c[d] >= g.lo[d]) {
      ix[d] = (int) ((c[d] - g.lo[d]) * g.bininv[d]);
      ix[d] = ix[d] < g.nbin[d] - 1 ? ix[d] : g.nbin[d] - 1;
    } else ix[d] = (int) ((c[d] - g.lo[d]) * g.bininv[d]) - 1;
  }
  return (ix[2] - g.mlo[2]) * g.mbin[1] * g.mbin[0] + (ix[1] - g.mlo[1]) * g.mbin[0] +
         (ix[0] - g.mlo[0]);
}

// A coordinate outside the bin grid would index outside binhead in the
// reference; here it is counted in *oob (the host turns it into an error) and
// parked in bin 0 so no access leaves the arrays.
__global__ void k_coord2bin_atoms(const double4 *__restrict__ x, int n, BinGeom g,
                                  int *__restrict__ bin, int *__restrict__ oob) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double4 p = x[i];
  int b = coord2bin(p.x, p.y, p.z, g);
  bool ok = b >= 0 && b < g.mbins;
  bin[i] = ok ? b : 0;
  if (!ok) atomicAdd(oob, 1);
}

__global__ void k_coord2bin_elems(const double *__restrict__ ex, int n, BinGeom g,
                                  int *__restrict__ bin, int *__restrict__ oob) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int b = coord2bin(ex[3 * i], ex[3 * i + 1], ex[3 * i + 2], g);
  bool ok = b >= 0 && b < g.mbins;
  bin[i] = ok ? b : 0;
  if (!ok) atomicAdd(oob, 1);
}

__global__ void k_bin_count(const int *__restrict__ bin, int n, int *__restrict__ count) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) atomicAdd(&count[bin[i]], 1);
}

__global__ void k_bin_fill(const int *__restrict__ bin, int n, const int *__restrict__ start,
                           int *__restrict__ cursor, int *__restrict__ members) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int b = bin[i];
  int slot = atomicAdd(&cursor[b], 1);
  members[start[b] + slot] = i;
}

// Sort each bin's members ascending (the reference's forward linked order).
// One thread per member: its rank in its bin is the number of smaller members
// of that bin.  The work follows the members, not the bins (a long box has far
// more bins than members).
__global__ void k_bin_sort(const int *__restrict__ bin, int n, const int *__restrict__ start,
                           const int *__restrict__ count, const int *__restrict__ members_in,
                           int *__restrict__ members_out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = bin[i];
  const int s0 = start[b], c = count[b];
  int rank = 0;
  for (int a = 0; a < c; a++) rank += members_in[s0 + a] < i;
  members_out[s0 + rank] = i;
}

__global__ void k_gather_bx_atoms(const int *__restrict__ mem, const double4 *__restrict__ x,
                                  double4 *__restrict__ bx, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) bx[p] = x[mem[p]];
}

__global__ void k_gather_bx_elems(const int *__restrict__ mem, const double *__restrict__ ex,
                                  double4 *__restrict__ bx, int n) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int i = mem[p];
  bx[p] = make_double4(ex[3 * i], ex[3 * i + 1], ex[3 * i + 2], 0.0);
}

inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }

}  // namespace

void launch_border_flags_atoms(const double4 *x, int nfirst, int nlast, int dim, double lo,
                               double hi, int *flags, cudaStream_t s) {
  int n = nlast - nfirst;
  if (n <= 0) return;
  k_border_flags_atoms<<<nblk(n, 256), 256, 0, s>>>(x, nfirst, nlast, dim, lo, hi, flags);
  check(cudaGetLastError(), "border_flags_atoms");
}

void launch_border_flags_elems(const double *ex, const int *etype, int nfirst, int nlast,
                               int dim, const double *mlo, const double *mhi, int *flags,
                               cudaStream_t s) {
  int n = nlast - nfirst;
  if (n <= 0) return;
  TypeSlabs sl;
  for (int t = 0; t <= MAXT; t++) {
    sl.lo[t] = mlo[t];
    sl.hi[t] = mhi[t];
  }
  k_border_flags_elems<<<nblk(n, 256), 256, 0, s>>>(ex, etype, nfirst, nlast, dim, sl, flags);
  check(cudaGetLastError(), "border_flags_elems");
}

void launch_border_scatter_atoms(double4 *x, int *type, int *tag, int *root, int *sendlist,
                                 const int *flags, const int *pos, int nfirst, int nlast,
                                 int n0, double dx, double dy, double dz, cudaStream_t s) {
  int n = nlast - nfirst;
  if (n <= 0) return;
  k_border_scatter_atoms<<<nblk(n, 256), 256, 0, s>>>(x, type, tag, root, sendlist, flags, pos,
                                                       nfirst, nlast, n0, dx, dy, dz);
  check(cudaGetLastError(), "border_scatter_atoms");
}

void launch_border_scatter_elems(double *ex, double *nodex, int *etype, int *etag, int *eroot,
                                 int *sendlist, const int *flags, const int *pos, int nfirst,
                                 int nlast, int n0, double dx, double dy, double dz,
                                 cudaStream_t s) {
  int n = nlast - nfirst;
  if (n <= 0) return;
  k_border_scatter_elems<<<nblk(n, 128), 128, 0, s>>>(ex, nodex, etype, etag, eroot, sendlist,
                                                       flags, pos, nfirst, nlast, n0, dx, dy,
                                                       dz);
  check(cudaGetLastError(), "border_scatter_elems");
}

void launch_forward_atoms(double4 *x, const int *sendlist, int n, int first, double dx,
                          double dy, double dz, cudaStream_t s) {
  if (n <= 0) return;
  k_forward_atoms<<<nblk(n, 256), 256, 0, s>>>(x, sendlist, n, first, dx, dy, dz);
  check(cudaGetLastError(), "forward_atoms");
}

void launch_forward_atoms_all(double4 *x, const int *send, int nlocal, int nghost,
                              const SwapChain &c, cudaStream_t s) {
  if (nghost <= 0) return;
  k_forward_atoms_all<<<nblk(nghost, 256), 256, 0, s>>>(x, send, nlocal, nghost, c);
  check(cudaGetLastError(), "forward_atoms_all");
}

void launch_forward_elems_all(double *nodex, const int *send, int nlocal, int nghost,
                              const SwapChain &c, cudaStream_t s) {
  if (nghost <= 0) return;
  k_forward_elems_all<<<nblk((long long) nghost * 24, 256), 256, 0, s>>>(nodex, send, nlocal,
                                                                         nghost, c);
  check(cudaGetLastError(), "forward_elems_all");
}

void launch_forward_elems(double *nodex, const int *sendlist, int n, int first, double dx,
                          double dy, double dz, cudaStream_t s) {
  if (n <= 0) return;
  k_forward_elems<<<nblk((long long) n * 24, 256), 256, 0, s>>>(nodex, sendlist, n, first, dx,
                                                                 dy, dz);
  check(cudaGetLastError(), "forward_elems");
}

void launch_copy_root(double *a, int width, const int *root, int gfirst, int gn,
                      cudaStream_t s) {
  if (gn <= 0) return;
  k_copy_root<double><<<nblk((long long) gn * width, 256), 256, 0, s>>>(a, width, root, gfirst, gn);
  check(cudaGetLastError(), "copy_root");
}

void launch_copy_root(float *a, int width, const int *root, int gfirst, int gn, cudaStream_t s) {
  if (gn <= 0) return;
  k_copy_root<float><<<nblk((long long) gn * width, 256), 256, 0, s>>>(a, width, root, gfirst, gn);
  check(cudaGetLastError(), "copy_root");
}

void launch_pbc_atoms(double4 *x, int n, const double *lo, const double *hi,
                      const double *prd, const int *periodic, cudaStream_t s) {
  if (n <= 0) return;
  Box b;
  for (int d = 0; d < 3; d++) {
    b.lo[d] = lo[d];
    b.hi[d] = hi[d];
    b.prd[d] = prd[d];
    b.per[d] = periodic[d];
  }
  k_pbc_atoms<<<nblk(n, 256), 256, 0, s>>>(x, n, b);
  check(cudaGetLastError(), "pbc_atoms");
}

void launch_pbc_elems(double *ex, double *nodex, int n, const double *lo, const double *hi,
                      const double *prd, const int *periodic, cudaStream_t s) {
  if (n <= 0) return;
  Box b;
  for (int d = 0; d < 3; d++) {
    b.lo[d] = lo[d];
    b.hi[d] = hi[d];
    b.prd[d] = prd[d];
    b.per[d] = periodic[d];
  }
  k_pbc_elems<<<nblk(n, 128), 128, 0, s>>>(ex, nodex, n, b);
  check(cudaGetLastError(), "pbc_elems");
}

void launch_coord2bin_atoms(const double4 *x, int n, const BinGeom &g, int *bin, int *oob,
                            cudaStream_t s) {
  if (n <= 0) return;
  k_coord2bin_atoms<<<nblk(n, 256), 256, 0, s>>>(x, n, g, bin, oob);
  check(cudaGetLastError(), "coord2bin_atoms");
}

void launch_coord2bin_elems(const double *ex, int n, const BinGeom &g, int *bin, int *oob,
                            cudaStream_t s) {
  if (n <= 0) return;
  k_coord2bin_elems<<<nblk(n, 256), 256, 0, s>>>(ex, n, g, bin, oob);
  check(cudaGetLastError(), "coord2bin_elems");
}

void build_bins(const int *bin, int n, int mbins, DBuf<int> &count, DBuf<int> &start,
                DBuf<int> &members, DBuf<int> &scratch, cudaStream_t s) {
  count.ensure((size_t) mbins + 1, s);
  start.ensure((size_t) mbins + 1, s);
  members.ensure((size_t) 2 * (n > 0 ? n : 1), s);
  check(cudaMemsetAsync(count.p, 0, sizeof(int) * ((size_t) mbins + 1), s), "bin memset");
  if (n > 0) k_bin_count<<<nblk(n, 256), 256, 0, s>>>(bin, n, count.p);
  scan_exclusive(count.p, start.p, mbins, start.p + mbins, scratch, s);
  // cursor reuses count after the scan consumed it; restore counts afterwards
  DBuf<int> &cursor = count;
  int *unsorted = members.p + n;
  check(cudaMemsetAsync(cursor.p, 0, sizeof(int) * (size_t) mbins, s), "cursor memset");
  if (n > 0) {
    k_bin_fill<<<nblk(n, 256), 256, 0, s>>>(bin, n, start.p, cursor.p, unsorted);
    k_bin_sort<<<nblk(n, 256), 256, 0, s>>>(bin, n, start.p, cursor.p, unsorted, members.p);
  }
  check(cudaGetLastError(), "build_bins");
}

void launch_gather_bin_x_atoms(const int *members, const double4 *x, double4 *bx, int n,
                               cudaStream_t s) {
  if (n <= 0) return;
  k_gather_bx_atoms<<<nblk(n, 256), 256, 0, s>>>(members, x, bx, n);
  check(cudaGetLastError(), "gather_bx_atoms");
}

void launch_gather_bin_x_elems(const int *members, const double *ex, double4 *bx, int n,
                               cudaStream_t s) {
  if (n <= 0) return;
  k_gather_bx_elems<<<nblk(n, 256), 256, 0, s>>>(members, ex, bx, n);
  check(cudaGetLastError(), "gather_bx_elems");
}

}  // namespace cacg
