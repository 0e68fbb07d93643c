// Internal declarations shared by the host orchestration (host.cpp) and the
// CUDA kernels (k_*.cu) of libcacg.so.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

struct cacg_mlp_t;

namespace cacg {

constexpr int NPE = 8;    // nodes per 3-d element (element.cpp:41)
constexpr int MAXT = 8;   // atom / element types supported

// Error from a CUDA call, turned into CACG_ECUDA at the ABI boundary.
struct CudaError {
  cudaError_t code;
  const char *where;
};

inline void check(cudaError_t e, const char *where) {
  if (e != cudaSuccess) throw CudaError{e, where};
}

// Allocation epochs: bumped whenever a device array is allocated or freed, so
// that a CUDA graph captured under an older value (it may hold pointers that
// are gone) is dropped.  An allocation made inside a call on a handle counts
// in that handle's epoch (the C ABI's entry points install it for the calling
// thread), any other in the global one; a handle's graphs are checked against
// the sum of both.  Handles driven from threads of their own thus do not drop
// each other's graphs.
inline std::atomic<unsigned long long> &dbuf_global_epoch() {
  static std::atomic<unsigned long long> e{0};
  return e;
}
inline std::atomic<unsigned long long> *&dbuf_epoch_slot() {
  static thread_local std::atomic<unsigned long long> *p = nullptr;
  return p;
}
inline void dbuf_bump() {
  if (std::atomic<unsigned long long> *p = dbuf_epoch_slot()) ++*p;
  else ++dbuf_global_epoch();
}
inline unsigned long long dbuf_epoch() {
  const std::atomic<unsigned long long> *p = dbuf_epoch_slot();
  return (p ? p->load() : 0ULL) + dbuf_global_epoch().load();
}
// installs a handle's epoch for the calling thread for the scope of a call
struct EpochScope {
  std::atomic<unsigned long long> *prev;
  explicit EpochScope(std::atomic<unsigned long long> *e) : prev(dbuf_epoch_slot()) {
    dbuf_epoch_slot() = e;
  }
  ~EpochScope() { dbuf_epoch_slot() = prev; }
  EpochScope(const EpochScope &) = delete;
  EpochScope &operator=(const EpochScope &) = delete;
};

// Growable device array.  Growth keeps contents when asked (ghost appends).
template <class T>
struct DBuf {
  T *p = nullptr;
  size_t cap = 0;
  void ensure(size_t n, cudaStream_t s, bool keep = false) {
    if (n <= cap) return;
    dbuf_bump();
    size_t ncap = cap ? cap : 256;
    while (ncap < n) ncap = ncap + ncap / 2 + 256;
    T *q = nullptr;
    check(cudaMalloc(&q, ncap * sizeof(T)), "cudaMalloc");
    if (keep && p && cap) check(cudaMemcpyAsync(q, p, cap * sizeof(T), cudaMemcpyDeviceToDevice, s), "grow copy");
    if (p) {
      check(cudaStreamSynchronize(s), "grow sync");
      cudaFree(p);
    }
    p = q;
    cap = ncap;
  }
  void release() {
    if (p) {
      cudaFree(p);
      dbuf_bump();
    }
    p = nullptr;
    cap = 0;
  }
};

// Bin geometry of Neighbor::setup_bins (neighbor.cpp:828-976); coord2bin uses
// the domain box lo/hi as bboxlo/bboxhi.
struct BinGeom {
  double lo[3], hi[3];
  double bininv[3];
  int nbin[3];
  int mlo[3];
  int mbin[3];
  int mbins;
};

// Shape-function and sub-element tables on the device (element.cpp:725-1423).
struct ElemTables {
  const double *spa_int;        // [sum numint][8], rows of type t start at int_off[t]
  const double *weight;         // [sum numint]
  const double *spa_inter;      // [sum ninter][8], type t starts at inter_off[t]
  const int *int_off;           // [MAXT+1]
  const int *inter_off;         // [MAXT+1]
  const int *numint;            // [MAXT+1]
  const int *inter_num;         // [MAXT+1]
  const int *node_list;         // [(MAXT+1)*8]
  const double *spa_center_sub; // [nsub][8]
  const double *spa_inter_sub;  // [total][8]
  const int *list_inter_sub;    // [total]
  const int *sub_first;         // [nsub+1]
  int nsub;
};

struct EamTables {
  const double *frho;  // [(nrho+1)*7]
  const double *rhor;  // [(nr+1)*7]
  const double *z2r;   // [(nr+1)*7]
  int nr, nrho;
  double rdr, rdrho, cutforcesq;
};

// ---- scan / compaction (k_comm.cu) ----
void scan_exclusive(const int *in, int *out, int n, int *total, DBuf<int> &scratch,
                    cudaStream_t s);

// ---- ghosts, wrap, bins (k_comm.cu) ----
void launch_border_flags_atoms(const double4 *x, int nfirst, int nlast, int dim, double lo,
                               double hi, int *flags, cudaStream_t s);
void launch_border_flags_elems(const double *ex, const int *etype, int nfirst, int nlast,
                               int dim, const double *mlo, const double *mhi, int *flags,
                               cudaStream_t s);
void launch_border_scatter_atoms(double4 *x, int *type, int *tag, int *root, int *sendlist,
                                 const int *flags, const int *pos, int nfirst, int nlast,
                                 int n0, double dx, double dy, double dz, cudaStream_t s);
void launch_border_scatter_elems(double *ex, double *nodex, int *etype, int *etag, int *eroot,
                                 int *sendlist, const int *flags, const int *pos, int nfirst,
                                 int nlast, int n0, double dx, double dy, double dz,
                                 cudaStream_t s);
// the swaps of a forward communication: first ghost index and shift of each
constexpr int MAX_SWAPS = 8;
struct SwapChain {
  int n;
  int first[MAX_SWAPS];
  double d[MAX_SWAPS][3];
};
// every swap in one launch, each ghost value computed as swap by swap
void launch_forward_atoms_all(double4 *x, const int *send, int nlocal, int nghost,
                              const SwapChain &c, cudaStream_t s);
void launch_forward_elems_all(double *nodex, const int *send, int nlocal, int nghost,
                              const SwapChain &c, cudaStream_t s);
void launch_forward_atoms(double4 *x, const int *sendlist, int n, int first, double dx,
                          double dy, double dz, cudaStream_t s);
void launch_forward_elems(double *nodex, const int *sendlist, int n, int first, double dx,
                          double dy, double dz, cudaStream_t s);
void launch_copy_root(float *a, int width, const int *root, int gfirst, int gn, cudaStream_t s);
void launch_copy_root(double *a, int width, const int *root, int gfirst, int gn,
                      cudaStream_t s);
void launch_pbc_atoms(double4 *x, int n, const double *lo, const double *hi,
                      const double *prd, const int *periodic, cudaStream_t s);
void launch_pbc_elems(double *ex, double *nodex, int n, const double *lo, const double *hi,
                      const double *prd, const int *periodic, cudaStream_t s);
void launch_coord2bin_atoms(const double4 *x, int n, const BinGeom &g, int *bin, int *oob,
                            cudaStream_t s);
void launch_coord2bin_elems(const double *ex, int n, const BinGeom &g, int *bin, int *oob,
                            cudaStream_t s);
// counting sort by bin, members of a bin in ascending index order
void build_bins(const int *bin, int n, int mbins, DBuf<int> &count, DBuf<int> &start,
                DBuf<int> &members, DBuf<int> &scratch, cudaStream_t s);
void launch_gather_bin_x_atoms(const int *members, const double4 *x, double4 *bx, int n,
                               cudaStream_t s);
void launch_gather_bin_x_elems(const int *members, const double *ex, double4 *bx, int n,
                               cudaStream_t s);

// ---- neighbor lists (k_neigh.cu) ----
void launch_atom_list(const double4 *x, const int *bin, const int *bstart, const int *bmem,
                      const double4 *bx, const int *stencil, int nstencil, int mbins, int nlocal,
                      double cutsq, int maxneigh, int stride, int *num, int *list,
                      int *overflow, cudaStream_t s);
void launch_elem_list(const double *ex, const int *bin, const int *bstart, const int *bmem,
                      const double4 *bx, const int *stencil, int nstencil, int mbins, int nlocal,
                      double cutsq, int maxneigh, int stride, int *num, int *list,
                      int *overflow, cudaStream_t s);
// site_h (may be null): float copy of each site for the FP32 pre-tests
void launch_sites(const double *nodex, const int *etype, const int *site_base, int nelem,
                  ElemTables t, double4 *site_x, float4 *site_h, cudaStream_t s);
void launch_split_hi(const double4 *x, float4 *xh, int n, cudaStream_t s);
void launch_sub_centres(const double *nodex, int nelem, ElemTables t, double4 *subc,
                        cudaStream_t s);
void launch_ip_list(const double *nodex, const double *ex, const int *etype,
                    const int *row_elem, const int *row_jj, int nrows, const int *enum_,
                    const int *elist, int estride, const double4 *subc, const double4 *site_x,
                    const int *site_base, ElemTables t, double cut_elesq, double cut_subelesq,
                    double cutsq, int maxip, int rowstride, int *ipnum, int *ipent,
                    int *overflow, cudaStream_t s);

// ---- forces: same kernels in two translation units (force_fp64.cuh) ----
// fp64_exact (k_force_exact.cu, -fmad=false) and fp64_fma (k_force_fma.cu).
#define CACG_FORCE_DECLS                                                                   \
  void lj_atoms(const double4 *x, const int *type, const int *num, const int *list,         \
                int stride, int nlocal, const void *tab, double *f, cudaStream_t s);        \
  void eam_rho_atoms(const double4 *x, const int *num, const int *list, int stride,         \
                     int nlocal, EamTables e, double *rho, double *fp, cudaStream_t s);     \
  void eam_force_atoms(const double4 *x, const int *num, const int *list, int stride,       \
                       int nlocal, EamTables e, const double *fp, double *f,                \
                       cudaStream_t s);                                                     \
  void lj_ip(const double *nodex, const int *etype, const int *row_elem, const int *row_jj, \
             int nrows, const int *ipnum, const int *ipent, int rowstride,                  \
             const double4 *site_x, ElemTables t, double lj1, double lj2, double cutsq,      \
             double *fip, cudaStream_t s);                                                  \
  void eam_erho(const double *nodex, const int *etype, const int *row_first, int nlocal_e,  \
                const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,   \
                ElemTables t, EamTables e, double *erho, cudaStream_t s);                   \
  void eam_site_fp(const double *erho, const int *etype, const int *site_base, int nelem,   \
                   ElemTables t, EamTables e, double *site_fp, cudaStream_t s);             \
  void eam_ip(const double *nodex, const double *erho, const int *etype,                    \
              const int *row_elem, const int *row_jj, int nrows, const int *ipnum,          \
              const int *ipent, int rowstride, const double4 *site_x,                       \
              const double *site_fp, ElemTables t, EamTables e, double *fip,                \
              cudaStream_t s);                                                              \
  void gather_nodef(const double *fip, const int *etype, const int *row_first,              \
                    int nlocal_e, ElemTables t, double *nodef, cudaStream_t s);

namespace fp64_exact {
CACG_FORCE_DECLS
}
// fp64_fma (k_force_fma.cu): FP32 pre-test against cut_pass on the float
// copies (xh, site_h), Newton-refined reciprocals, weight-0 rows skipped.
namespace fp64_fma {
void lj_atoms(const double4 *x, const float4 *xh, const int *type, const int *num,
              const int *list, int stride, int nlocal, const void *tab, float cut_pass,
              double *f, cudaStream_t s);
void eam_rho_atoms(const double4 *x, const float4 *xh, const int *num, const int *list,
                   int stride, int nlocal, EamTables e, float cut_pass, double *rho,
                   double *fp, cudaStream_t s);
void eam_force_atoms(const double4 *x, const float4 *xh, const int *num, const int *list,
                     int stride, int nlocal, EamTables e, float cut_pass, const double *fp,
                     double *f, cudaStream_t s);
void lj_ip(const double *nodex, const int *etype, const int *row_elem, const int *row_jj,
           int nrows, const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,
           const float4 *site_h, ElemTables t, double lj1, double lj2, double cutsq,
           float cut_pass, const int *rows, double *fip, cudaStream_t s);
void eam_erho(const double *nodex, const int *etype, const int *row_first, int nlocal_e,
              const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,
              const float4 *site_h, ElemTables t, EamTables e, float cut_pass, double *erho,
              cudaStream_t s);
void eam_site_fp(const double *erho, const int *etype, const int *site_base, int nelem,
                 ElemTables t, EamTables e, double *site_fp, cudaStream_t s);
void eam_ip(const double *nodex, const double *erho, const int *etype, const int *row_elem,
            const int *row_jj, int nrows, const int *ipnum, const int *ipent, int rowstride,
            const double4 *site_x, const float4 *site_h, const double *site_fp, ElemTables t,
            EamTables e, float cut_pass, const int *rows, double *fip, cudaStream_t s);
void gather_nodef(const double *fip, const int *etype, const int *row_first, int nlocal_e,
                  ElemTables t, double *nodef, cudaStream_t s);
void sites(const double *nodex, const int *etype, const int *site_base, int nelem, ElemTables t,
           double4 *site_x, float4 *site_h, cudaStream_t s);
// the sites any integration-point list references (computed per rebuild)
void mark_sites(const int *ipnum, const int *ipent, int nrows, int rowstride, int *flag,
                cudaStream_t s);
void need_compact(const int *flag, const int *pos, int nsites, const int *site_base, int nall,
                  int *need, int *need_elem, cudaStream_t s);
void sites_needed(const double *nodex, const int *etype, const int *site_base, const int *need,
                  const int *need_elem, int nneed, ElemTables t, double4 *site_x, float4 *site_h,
                  cudaStream_t s);
void site_fp_needed(const double *erho, const int *etype, const int *site_base, const int *need,
                    const int *need_elem, int nneed, ElemTables t, EamTables e, double *site_fp,
                    cudaStream_t s);
// per-step short lists (FP32 guarded cutoff test), used by both FP64 modes
void filter_atoms(const float4 *xh, const int *num, const int *list, int stride, int nlocal,
                  float cut_pass, int *snum, int *slist, cudaStream_t s);
void filter_rows(const double *nodex, const int *etype, const int *row_elem, const int *row_jj,
                 int nrows, const int *ipnum, const int *ipent, int rowstride,
                 const float4 *site_h, ElemTables t, float cut_pass, int only_needed, int *snum,
                 int *sent, cudaStream_t s, const int *row_list = nullptr,
                 const unsigned char *skip = nullptr);
}  // namespace fp64_fma

// ---- mixed precision (k_mixed.cu): FP32 pair terms, FP64 accumulation ----
namespace mixed {
struct MixedAtoms {
  const double4 *x;
  // cell-relative coordinates: xyz = x - (L0 + g * cell) in FP32, w = the cell
  // (12 + 10 + 10 bits); a pair vector is (q_i - q_j) + g * (cell_i - cell_j)
  const float4 *xq;
  float qg;
  const int *num, *list;
  int stride, nlocal;
  float cutsq_f, band_lo, band_hi;  // FP32 test; [band_lo, band_hi] re-tested in FP64
  double cutsq;
  int *snum, *slist;  // EAM: short list written by the density pass, read by the force pass
  // EAM density pass over a reordered list: nnear[i] entries lie within the
  // cutoff + 1 A at the reorder; dmax2 = the largest squared displacement
  // since (float bits); null: every entry is scanned
  const int4 *nnear = nullptr;
  const unsigned *dmax2 = nullptr;
  int block = 512;    // threads per block of the persistent grids (autotuned)
  bool fprime64 = true;  // F'(rho) of the atoms from the FP64 spline ("tune fprime")
  const float2 *frho_ds = nullptr;  // its F' coefficients as double-single pairs
};
// Displacement culling of the mixed passes: list entries beyond r_c + d at
// the last reorder are skipped while twice the largest displacement since
// then, plus CULL_MARGIN, stays within d, for the levels d = CULL_D1, CULL_D2,
// CULL_DELTA (A); beyond CULL_DELTA the lists are reordered.
constexpr float CULL_D1 = 0.25f, CULL_D2 = 0.5f, CULL_DELTA = 1.0f, CULL_MARGIN = 0.01f;

// the culling level the device kernels choose (1..3; 4: no culling), from
// the squared displacement and the reordered-this-step flag
inline int cull_level_host(float d2, unsigned reordered) {
  if (reordered) return 1;
  const float d = 2.0f * __builtin_sqrtf(d2) + CULL_MARGIN;
  return d <= CULL_D1 ? 1 : d <= CULL_D2 ? 2 : d <= CULL_DELTA ? 3 : 4;
}
// float4 per knot of the FP32 EAM force table: (rho c0, c1, c2, r*phi c3),
// (r*phi c4, c5, c6, 0)
constexpr int FTAB_W = 2;

// The packing grid of the cell-relative coordinates: cells of a power-of-two
// size g from the corner l0 (split into double-single floats); *oob counts
// positions outside the 4096 x 1024 x 1024-cell range.
struct PackGrid {
  float l0h[3], l0l[3];
  float g, ig;
  int *oob;
};
// lattice sizes per type ([3 * type + axis]) and the fractions k / (n - 1)
// per type and axis as double-single floats ([(3 * type + axis) * fstride + k])
struct Lattice {
  const int *nae;
  const float2 *frac;
  int fstride;
  int kb = 6;  // bits of the site index kk in a list entry's line code
};
struct MixedElems {
  const float4 *line_pos;  // lattice lines of this step: U, D double-single (3 float4)
  const float2 *line_rho;  // nodal-density lines of this step (EAM force pass)
  const float4 *fp4;       // FP32 F' spline, c0..c2 per knot
  int nrho = 0;
  float rdrho = 0.f;
  const float4 *ip_q;         // packed integration-point positions, per row
  const float4 *ip_h, *ip_l;  // their double-single positions
  const float *row_fp;        // FP32 F'(rho) at the rows of nonzero weight (EAM force pass)
  const int *etype, *row_elem, *row_first, *node_list;
  // integration-point lists, row-major: line codes (element * maxlines + line)
  // << lat.kb | kk, each row's culling parts in order
  const int *row_start, *ent;
  const int4 *nnear_row = nullptr;  // culled entry counts per row (null: no culling)
  const unsigned *eflags = nullptr;  // [node displacement^2 bits, reordered this step]
  int nlocal_e;
  const int *rows;  // rows of nonzero weight (force passes), count nforce
  int nforce;
  float cutsq_f, band_lo, band_hi;
  double cutsq;
  const unsigned char *skip = nullptr;  // elements whose forces come from the surrogate
  Lattice lat;
  PackGrid pg;
  int block = 512;  // threads per block of the persistent grids
  int group = 8;    // lanes per integration point (4, 8 or 16)
};
// cell-relative packed coordinates for the atom passes; *oob counts atoms
// outside the 4096 x 1024 x 1024-cell range
PackGrid make_pack_grid(const double l0[3], double g, int *oob);
// with ref (packed coordinates of the list reorder, same grid): the largest
// squared displacement of the first nref atoms is max-folded into *dmax2
void pack_rel(const double4 *x, int n, const PackGrid &pg, float4 *xq, const float4 *ref, int nref,
              unsigned *dmax2, cudaStream_t s);
// with ref: the largest squared node displacement against ref -> *dmax2 (atomic max)
void node_split(const double *nodex, int n, float2 *hl, const float2 *ref, unsigned *dmax2,
                cudaStream_t s);
// Lattice lines: U, D (double-single, relative to l0) of every line that
// mask (mask_near while culling holds) marks; FP32 nodal-density lines
// (with gate: only in a step whose node displacement calls for a list reorder)
void lines(const float2 *node_hl, const int *etype, const Lattice &lat, int max_nax,
           const unsigned long long *mask, const unsigned long long *mask_near,
           const unsigned *eflags, int maxlines, const PackGrid &pg, int nelem, float4 *line_pos,
           cudaStream_t s, const unsigned *gate = nullptr);
void line_rho(const double *erho, const int *etype, const Lattice &lat,
              const unsigned long long *mask, const unsigned long long *mask_near,
              const unsigned *eflags, int maxlines, int nelem, float2 *out, cudaStream_t s);
// the integration-point lists' site ids turned into line codes in place
void ent_codes(int *ent, long long n, const int *site_base, int nall_e, const int *etype,
               const int *nae, int maxlines, int kb, cudaStream_t s);
// line masks (bit kk per line) of the rows' entries (all rows; force rows);
// with nnear_row, of the culled parts; with gate, only after a reorder
void line_masks(const int *row_start, const int *ent, const int4 *nnear_row, int nrows,
                const Lattice &lat, const unsigned char *isforce, unsigned long long *mask,
                unsigned long long *mask_f, long long nmask, const unsigned *gate,
                cudaStream_t s);
// the fused element passes (every list entry references its row's own
// element): per element, one warp evaluates the node rows (pass 1: nodal
// densities) or the rows of nonzero weight with the nodal gather (pass 2: EAM
// forces; pass 0: LJ), pair vectors from the element's trilinear coefficient
// vectors and lattice-index differences; guard-band pairs are decided in FP64
struct FusedTables {
  const float2 *node_hl;      // split nodes of this step
  const double *nodex;        // FP64 nodes
  const int *int_off, *inter_off;  // first row / site of each type in the per-type tables
  const int4 *intp;           // lattice indices of the rows, per type
  const double *spa_int;      // FP64 shape functions of the rows
  const double *spa_inter;    // FP64 shape functions of the sites
  const int *fjj, *fjj_off;   // per type: rows of nonzero weight (at most 32), ascending
  const float *wn;            // weight x shape function per row and node
  int maxlines;
  int variant;                // 0: coefficients in registers; 1, 2: in shared memory
  const float2 *spa_int_hl;   // the rows' shape functions as double-single pairs
  const float2 *frho_ds;      // F' spline c0..c2 per knot as double-single pairs
  const float *wnf;           // wn of the rows of nonzero weight, per type in fjj order
  int *band;                  // guard-band list: count, blocks done, elements re-run so
                              // far, then the listed elements (3 + nlocal_e ints, zeroed once)
  const float4 *lat_rec;      // per type 1/(n_a-1), 1/(n_b-1), 1/(n_c-1), 1/n_b
};
bool fused_fits(int nr, int nrho);
// elements [e_begin, e_end) (e_end < 0: all local elements); the guard-band
// exact pass runs after each launch
void elem_fused(const MixedElems &m, const FusedTables &t, int pass, const float4 *tab,
                const EamTables &e, float lj1, float lj2, const double *erho_in,
                double *erho_out, double *nodef, cudaStream_t s, int e_begin = 0,
                int e_end = -1);
// list entries that reference a site of another element than their row's
long long self_check(const int *row_start, const int *ent, const int *row_elem, int nrows,
                     const Lattice &lat, int maxlines, unsigned long long *scratch,
                     cudaStream_t s);
// lattice lines with a referenced site: count[0] in mask, count[1] in mask_f
void count_lines(const unsigned long long *mask, const unsigned long long *mask_f, long long n,
                 unsigned long long *count, cudaStream_t s);
// displacement culling of the integration-point lists: reorder (gated on the
// node displacement in eflags[0]) into ent_near / nnear_row and keep the
// nodes as the reference (eflags[1] = 1, eflags[2] counts reorders)
void ip_reorder(const int *row_start, const int *ent, int nrows, const float4 *ip_q,
                const float4 *line_pos, const Lattice &lat, const PackGrid &pg, float cutoff,
                int *ent_near, int4 *nnear_row, const float2 *node_hl, int nall_e,
                float2 *node_ref, unsigned *eflags, cudaStream_t s);
// each atom's list reordered in its culling parts when the displacement since
// the last reorder (dmax2[0], against ref) no longer allows culling; it then
// sets ref to the positions and dmax2[1] = 1
void list_partition(const float4 *xq, float g, const int *num, const int *list, int stride,
                    int nlocal, float cut_rsq, float cutoff, int *out, int4 *nnear, float4 *ref,
                    unsigned *dmax2, unsigned *reorders, cudaStream_t s);
// neighbor unions of 32-atom groups staged in shared memory (EAM atom passes)
int union_max();
void union_build(const int *num, const int *list, int stride, int nlocal, int *union_j,
                 int *union_n, unsigned short *slot, cudaStream_t s);
void eam_rho_union(const MixedAtoms &m, const int *union_j, const int *union_n,
                   const unsigned short *slot, unsigned short *sslot, const float4 *rhor_val,
                   const EamTables &e, const float4 *fp4, double *rho, float *fp,
                   cudaStream_t s);
void eam_force_union(const MixedAtoms &m, const int *union_j, const int *union_n,
                     const unsigned short *sslot, const float4 *ftab, const EamTables &e,
                     const float *fp, double *f, cudaStream_t s);
// fp: FP32 F'(rho) from the FP32 coefficient table fp4 (c0..c2 per knot)
void eam_rho_atoms(const MixedAtoms &m, const float4 *rhor_val, const EamTables &e,
                   const float4 *fp4, double *rho, float *fp, cudaStream_t s);
void eam_force_atoms(const MixedAtoms &m, const float4 *ftab, const EamTables &e,
                     const float *fp, double *f, cudaStream_t s);
void lj_atoms(const MixedAtoms &m, const int *type, const float *lj1, const float *lj2,
              const float *cutsq_t, const double *cutsq64, double *f, cudaStream_t s);
// every row's integration point: packed, and its double-single position
void row_q(const int *row_elem, const int *row_jj, const int *etype, const int *int_off,
           const float2 *spa_int_hl, const float2 *node_hl, int nrows, const PackGrid &pg,
           float4 *ip_q, float4 *ip_h, float4 *ip_l, cudaStream_t s,
           const unsigned *gate = nullptr);
// FP32 F'(rho) at the rows of nonzero weight, rho in FP64 from the nodal densities
void row_fp(const int *rows, int nforce, const int *row_elem, const int *row_jj,
            const int *etype, const int *int_off, const double *spa_int, const double *erho,
            const EamTables &e, float *fp, cudaStream_t s);
// row-major copy of the integration-point lists (row_start: exclusive scan of ipnum)
void ip_csr(const int *ipnum, const int *ipent, int nrows, int rowstride, const int *row_start,
            int *ent, cudaStream_t s);
// pass 0: LJ forces -> outf[3*rows]; 1: EAM nodal densities -> out[8*nlocal_e]
// (FP64); 2: EAM forces -> outf[3*rows] (double-single floats)
void ip_pass(const MixedElems &m, int pass, const float4 *tab, const EamTables &e, float lj1,
             float lj2, double *out, float2 *outf, cudaStream_t s);
// nodal forces from the double-single row forces; wn = weight x shape function
// (FP32) per type row and node
void gather_nodef(const float2 *fipf, const int *etype, const int *row_first, const int *numint,
                  const int *int_off, const float *wn, int nlocal_e, double *nodef,
                  cudaStream_t s);
}  // namespace mixed

// ---- energy, virial, kinetic energy (k_thermo.cu); 7 partial sums per block ----
namespace thermo {
int partial_blocks(long long n);
void atoms_lj(const double4 *x, const int *type, const int *num, const int *list, int stride,
              int n, const double *lj, double *part, cudaStream_t s);
void atoms_eam(const double4 *x, const int *num, const int *list, int stride, int n,
               EamTables e, const double *rho, const double *fp, double *part, cudaStream_t s);
void ip(const double *nodex, const double *erho, const int *etype, const int *row_elem,
        const int *row_jj, const int *rows, int nforce, const int *ipnum, const int *ipent,
        int rowstride, const double4 *site_x, const double *site_fp, ElemTables t, EamTables e,
        int eam, double lj1, double lj2, double lj3, double lj4, double ljcutsq, double *part,
        cudaStream_t s);
void kinetic(const double *v, const int *type, const double *mass, int n, int per_item,
             double scale, double *part, cudaStream_t s);
}  // namespace thermo

// ---- analysis (k_analysis.cu, -fmad=false) ----
namespace analysis {
// centro-symmetry of atoms i0 .. i0+n-1; scratch dsq/near hold maxn x chunk
// entries (column-major, chunk >= n)
void centro(const double4 *x, const int *num, const int *list, int stride, int i0, int n,
            double cutsq, double *dsq, int *near, int chunk, double *out, cudaStream_t s);
}  // namespace analysis

// ---- tensor-core GEMM (k_gemm.cu) and the surrogate MLP (mlp.cu) ----
namespace gemm {
// C = A B^T, bf16 operands (K-major), fp32 accumulation; kind: 0 store C,
// 1 C = acc + bias, 2 Z = acc + bias and H = silu(Z), 3 H = acc * silu'(Z),
// 4 H = silu(acc + bias)
void gemm_tn(const void *A, int lda, const void *B, int ldb, int M, int N, int K, int kind,
             const float *bias, float *c, int ldc, void *h, int ldh, int *err, cudaStream_t s);
// all members and layers of the surrogate in one launch (k_mlp_ensemble)
void mlp_ensemble(const void *xf, int n, const void *w1s, const void *w2s, const void *w3s,
                  const void *w4s, const float *bias, int members, const float *norm, float *mean,
                  float *spread, int *err, cudaStream_t s,
                  const int *count = nullptr);
}  // namespace gemm
constexpr int MLP_IN = 32, MLP_HIDDEN = 256, MLP_OUT = 24;
namespace mlp {
struct Net;
Net *net_of(cacg_mlp_t *m);
const float *norm_device(const Net *n);  // in_mean[32], in_inv_std[32], out_mean[24], out_std[24]
double force_scale(const Net *n);
int members(const Net *n);
// ensemble prediction on normalised bf16 features [count][64] on the device
// count: rows to evaluate (device), or null for all
void predict(Net *n, const void *xf, long long count, float *mean, float *spread, cudaStream_t s,
             const int *dcount = nullptr);
// throws when a bounded wait inside a GEMM ran out (reads a device flag)
void check_error(Net *n, cudaStream_t s);
}  // namespace mlp
namespace surrogate {
// elems[i] for i < *count (count null: i < n)
void features(const double *nodex, const double *nodex0, const double *erho, const int *elems,
              int n, const int *count, const float *norm, void *xf, cudaStream_t s);
// the far elements due for a test this step (indices into far) and their
// number; wait[i] counts down the steps to a far element's next test
void due(int nfar, const int *far, unsigned char *wait, unsigned char *skip, int *due_list,
         int *count, cudaStream_t s);
void raw_features(const double *nodex, const double *nodex0, const double *erho, int n, float *x,
                  cudaStream_t s);
void accept(const float *spread, const int *far, const int *due_list, const int *count, int nfar,
            float thr, unsigned char *skip, unsigned char *wait, unsigned char *streak,
            unsigned long long *counters, cudaStream_t s);
void write_forces(const float *mean, const int *far, const int *due_list, const int *count,
                  int nfar, const unsigned char *skip, double *nodef, cudaStream_t s);
// out[i] = far[due_list[i]] for i < *count
void gather_far(const int *far, const int *due_list, const int *count, int nfar, int *out,
                cudaStream_t s);
void to_float(const double *src, long long n, float *dst, cudaStream_t s);
}  // namespace surrogate

// ---- integration and reductions (k_nve.cu) ----
// dtf / m per type (FixNVE's dtfm, fix_nve.cpp:54-99), the same IEEE quotient
// the host forms: no FP64 division per atom on the device
struct TypeScale {
  double v[MAXT + 1];
};
// fused: one FMA per update (FP64 FMA and mixed modes); else the exact mode's
// multiply-then-add
void launch_nve_atoms_initial(double4 *x, double *v, const double *f, const int *type,
                              const TypeScale &dtfm, int n, double dtv, bool fused,
                              cudaStream_t s);
void launch_nve_atoms_final(double *v, const double *f, const int *type, const TypeScale &dtfm,
                            int n, bool fused, cudaStream_t s);
void launch_nve_nodes_initial(double *ex, double *nodex, double *nodev, const double *nodef,
                              const int *etype, const TypeScale &dtfm, int n, double dtv,
                              bool fused, cudaStream_t s);
// fix setforce / fix viscous on the items (atoms, or elements x 8 nodes) whose
// group mask has `bit` (fix_setforce.cpp:107-161, fix_viscous.cpp:73-123)
void launch_setforce(double *f, const int *mask, int n, int per_item, int bit, const int *set,
                     const double *val, cudaStream_t s);
// x[i * stride] = nlo + (x[i * stride] - olo) * f for i < n (fix deform remap)
void launch_affine(double *x, int n, int stride, double olo, double nlo, double f, cudaStream_t s);
void launch_viscous(double *f, const double *v, const int *mask, int n, int per_item, int bit,
                    double gamma, cudaStream_t s);
void launch_nve_nodes_final(double *nodev, const double *nodef, const int *etype,
                            const TypeScale &dtfm, int n, bool fused, cudaStream_t s);
// the box for the element wrap test of the distance check
struct BoxWrap {
  double lo[3], hi[3];
  int periodic[3];
};
// bits of *flag: 1 atoms, 2 nodes moved past the trigger; 4 (with ex) an
// element centre outside the box in a periodic dimension
void launch_check_distance(const double4 *x, const double *xhold, int n,
                           const double *nodex, const double *nodexhold, int ne,
                           const double *ex, const BoxWrap &box, double triggersq, int *flag,
                           cudaStream_t s);
// the device step loop's state (int slots): steps since setup, steps done in
// this launch, steps wanted, flags of a pending rebuild (0: none), loop
// iterations, check_distance bits of the current step
enum { LOOP_AGO = 0, LOOP_DONE, LOOP_WANT, LOOP_PENDING, LOOP_ITERS, LOOP_BITS, LOOP_SLOTS };
// check_distance for the device loop: only on steps that reach a decision,
// bits into loop[LOOP_BITS]
void launch_loop_check(const double4 *x, const double *xhold, int n, const double *nodex,
                       const double *nodexhold, int ne, const double *ex, const BoxWrap &box,
                       double triggersq, int *loop, int every, int delay, cudaStream_t s);
// the decision of the device loop: sets the loop's conditions (again: run
// another iteration; proceed: this step's force passes run)
void launch_loop_decide(int *loop, int every, int delay, int dist_check,
                        cudaGraphConditionalHandle again, cudaGraphConditionalHandle proceed,
                        cudaStream_t s);
void launch_hold_atoms(const double4 *x, double *xhold, int n, cudaStream_t s);
void launch_elem_diag(const double *nodex, const double *ex, int n, double *diag,
                      int *centre_bad, cudaStream_t s);
double fp64_fma_rate(cudaStream_t s);
void launch_pack3to4(const double *in, double4 *out, int n, cudaStream_t s);
void launch_unpack4to3(const double4 *in, double *out, int n, cudaStream_t s);

}  // namespace cacg
