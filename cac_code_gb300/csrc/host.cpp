// Host side of libcacg.so: the C ABI in include/cacg.h.
//
// The handle mirrors the reference's objects for this path -- Domain box,
// Atom/Element arrays, Neighbor settings and lists, Pair tables, FixNVE -- but
// the arrays live on the GPU from cacg_init on.  Host code does only what the
// reference does once per rebuild on scalars (cutoffs, bin geometry, swap
// slabs, element-size maximum) and drives the kernels on one stream.
//
// Parsing follows the reference's command and file formats so an input
// script written for the reference runs unchanged:
//   Input::execute_command  input.cpp:362-404
//   ReadData::command       read_data.cpp:70-246, 277-367, 379-688
//   PairLJCut::settings/coeff/init_one  pair_lj_cut.cpp:75-198
//   PairEAM::coeff/read_file/file2array/array2spline  pair_eam.cpp:119-580
//   Neighbor::set/modify_params/init/setup_bins  neighbor.cpp:188-481, 828-976
//   Element tables  element.cpp:725-906, 1170-1423
//   CommBrick::setup  comm_brick.cpp:182-367
#include "../../include/cacg.h"
#include "internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

using namespace cacg;

namespace {

struct ApiError {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const char *fmt, ...) {
  char buf[1024];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  throw ApiError{code, buf};
}

struct SwapDef {
  int dim = 0, pbc = 0;
  double lo = 0, hi = 0;
  double mlo[MAXT + 1] = {}, mhi[MAXT + 1] = {};
  int nsend = 0, firstrecv = 0, send_off = 0;
  int ensend = 0, efirstrecv = 0, esend_off = 0;
  double d[3] = {0, 0, 0};
};

double numeric(const std::string &s) {
  char *end = nullptr;
  double v = strtod(s.c_str(), &end);
  if (end == s.c_str() || *end) fail(CACG_EINVAL, "Expected floating point parameter instead of '%s'", s.c_str());
  return v;
}

int inumeric(const std::string &s) {
  char *end = nullptr;
  long v = strtol(s.c_str(), &end, 10);
  if (end == s.c_str() || *end) fail(CACG_EINVAL, "Expected integer parameter instead of '%s'", s.c_str());
  return (int) v;
}

// Force::bounds: "*", "n", "*n", "n*", "m*n" over 1..nmax (force.cpp:182-210)
void bounds(const std::string &s, int nmax, int &lo, int &hi) {
  size_t p = s.find('*');
  if (p == std::string::npos) {
    lo = hi = inumeric(s);
  } else if (s.size() == 1) {
    lo = 1;
    hi = nmax;
  } else if (p == 0) {
    lo = 1;
    hi = inumeric(s.substr(1));
  } else if (p == s.size() - 1) {
    lo = inumeric(s.substr(0, p));
    hi = nmax;
  } else {
    lo = inumeric(s.substr(0, p));
    hi = inumeric(s.substr(p + 1));
  }
  if (lo < 1 || hi > nmax || lo > hi) fail(CACG_EINVAL, "Numeric index is out of bounds");
}

std::vector<std::string> split_words(const std::string &line) {
  std::vector<std::string> w;
  std::istringstream is(line);
  std::string t;
  while (is >> t) w.push_back(t);
  return w;
}

void shape8(double px, double py, double pz, double *N) {
  // element.cpp:1340-1347, evaluated left to right
  N[0] = 0.125 * (1 - px) * (1 - py) * (1 - pz);
  N[1] = 0.125 * (1 + px) * (1 - py) * (1 - pz);
  N[2] = 0.125 * (1 + px) * (1 + py) * (1 - pz);
  N[3] = 0.125 * (1 - px) * (1 + py) * (1 - pz);
  N[4] = 0.125 * (1 - px) * (1 - py) * (1 + pz);
  N[5] = 0.125 * (1 + px) * (1 - py) * (1 + pz);
  N[6] = 0.125 * (1 + px) * (1 + py) * (1 + pz);
  N[7] = 0.125 * (1 - px) * (1 + py) * (1 + pz);
}

template <class T>
void upload(DBuf<T> &b, const std::vector<T> &h, cudaStream_t s) {
  b.ensure(h.size() > 0 ? h.size() : 1, s);
  if (!h.empty())
    check(cudaMemcpyAsync(b.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s),
          "upload");
}

}  // namespace

struct LJTabHost {
  double lj1[(MAXT + 1) * (MAXT + 1)];
  double lj2[(MAXT + 1) * (MAXT + 1)];
  double cutsq[(MAXT + 1) * (MAXT + 1)];
};

struct cacg_context {
  std::string err;
  int device = 0;
  cudaStream_t stream = nullptr;

  // units (update.cpp:83-132)
  double ftm2v = 1.0, dt = 0.005, skin = 0.3;
  bool metal = false;
  // neighbor settings (neighbor.cpp:45-55 defaults)
  int every = 1, delay = 10, dist_check = 1, oneatom = 2000, pgsize = 100000;
  double binsize_user = 0.0;
  int nsplit = 2;
  int mode = CACG_FP64_EXACT;
  bool fix_nve = false;

  // box
  double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, prd[3] = {0, 0, 0};
  int periodic[3] = {1, 1, 1};
  bool box_set = false;

  // atoms (host staging until init)
  int ntypes = 0;
  double amass[MAXT + 1] = {};
  double up_mass[MAXT + 1] = {}, up_emass[MAXT + 1] = {};  // the masses on the device
  std::vector<double> h_x, h_v;
  std::vector<int> h_type, h_tag;
  int nlocal = 0, nghost = 0;

  // element types
  int netypes = 0;
  int nae[MAXT + 1][3] = {};
  int numint[MAXT + 1] = {};
  std::vector<int> intp[MAXT + 1];
  std::vector<double> weight[MAXT + 1];
  double emass[MAXT + 1] = {};
  std::vector<double> h_ex, h_nodex, h_nodev;
  std::vector<int> h_etype, h_etag;
  int enlocal = 0, enghost = 0;

  // pair
  int pair_style = 0;  // 1 lj/cut, 2 eam
  bool eam_setfl = false;  // eam/alloy: the tables come from a setfl file
  double cut_global = 0.0;
  double eps[MAXT + 1][MAXT + 1] = {}, sig[MAXT + 1][MAXT + 1] = {}, cutp[MAXT + 1][MAXT + 1] = {};
  int setflag[MAXT + 1][MAXT + 1] = {};
  // LJ tables handed over by cacg_set_lj (the caller's PairLJCut after
  // init_one): used as given instead of forming them from epsilon and sigma
  bool lj_raw = false;
  std::vector<double> raw_lj1, raw_lj2, raw_cutsq;  // [(ntypes + 1)^2]
  LJTabHost ljtab;
  // eam
  int nr = 0, nrho = 0;
  double dr = 0, drho = 0, rdr = 0, rdrho = 0, cutforcesq = 0, eam_mass = 0, eam_cut = 0;
  std::vector<double> frho_sp, rhor_sp, z2r_sp;

  // derived cutoffs
  double cutneighmax = 0, cutneighmaxsq = 0, triggersq = 0;
  double esize[MAXT + 1] = {}, max_size = 0.0;
  double cut_all = 0, cut_allsq = 0, cut_ele = 0, cut_elesq = 0, cut_subele = 0, cut_subelesq = 0;
  double cutghost[3] = {}, cutghostmulti[MAXT + 1] = {};
  std::vector<SwapDef> swaps;
  BinGeom bins{};
  std::vector<int> stencil;

  // element tables (host)
  int nsub = 0;
  std::vector<int> int_off, inter_off, inter_num, numint_v, node_list, sub_first, list_isub;
  std::vector<double> spa_int, w_all, spa_inter, spa_csub, spa_isub;
  std::vector<int> h_site_base, h_row_first, h_eroot;
  int nrows = 0, nsites = 0;

  // device arrays: atoms
  DBuf<double4> d_x;
  DBuf<float4> d_xh, d_site_h;  // float copies for the FP32 cutoff pre-tests
  // mixed precision: FP32 spline tables, double-single element nodes and
  // integration-point shape functions, packed site positions and site F'(rho),
  // the referenced sites of each lattice line, lattice sizes per type
  DBuf<float4> d_xl, d_rhor_val4, d_ftab, d_fp4, d_line_pos;
  DBuf<float2> d_frho_ds;  // F' spline coefficients c0..c2 per knot, double-single
  DBuf<float2> d_node_hl, d_spa_int_hl;
  DBuf<float> d_u, d_ljf, d_fpf;
  DBuf<float2> d_line_rho;
  DBuf<unsigned long long> d_line_mask, d_line_mask_f;  // all rows; rows of nonzero weight
  DBuf<int> d_nae;
  DBuf<float2> d_frac, d_fipf;  // lattice fractions; double-single row forces
  DBuf<float> d_wn;             // weight x shape function per type row and node (FP32)
  DBuf<float> d_wnf;            // the same for the rows of nonzero weight, per type in order
  DBuf<int> d_band;             // elements with a guard-band pair: count, blocks done, list
  DBuf<float4> d_lat_rec;       // per type 1/(n_a-1), 1/(n_b-1), 1/(n_c-1), 1/n_b
  int fstride = 1;
  // mixed precision, per row: packed and double-single integration points,
  // F'(rho) of the force rows; the integration-point lists row-major
  DBuf<float4> d_ip_q, d_ip_h, d_ip_l;
  DBuf<float> d_row_fpf;
  DBuf<int> d_row_start, d_ent;
  // displacement culling of the integration-point lists: rows' near entries
  // first, their count, the nodes at the reorder, near-site masks, the line
  // code of every site, force-row flags; reordered once per element list build
  // and whenever a node has moved 0.495 A since
  DBuf<int> d_ent_near;
  bool codes_ok = false;  // the lists fit the line codes of the mixed element passes
  int code_kb = 6;        // bits of kk in a line code
  DBuf<int4> d_nnear_row;
  DBuf<float2> d_node_ref;
  DBuf<unsigned long long> d_line_mask_n, d_line_mask_nf;
  DBuf<unsigned char> d_row_isforce;
  long long elist_builds = 0, epart_of = -1;
  bool ereorders_zeroed = false;  // the reorder counter (d_misc slot 15)
  bool areorders_zeroed = false;  // the atom-list reorder counter (d_misc slot 16)
  // lattice lines that the integration-point lists reference (all rows; force
  // rows), counted at each element list build
  DBuf<unsigned long long> d_nlines;
  unsigned long long h_nlines[2] = {0, 0};
  // fused element passes ("tune fused yes|no"): one warp per element when every
  // list entry references its row's own element (checked at each element list
  // build) and no type has more than 32 rows of nonzero weight
  bool fused_on = true, self_contained = false, fused_types_ok = false, fused_used = false;
  // "tune fused_variant 0|1|2", the kernel arrangement (same arithmetic): the
  // element's coefficients in registers (0, 512 threads a block), read from
  // shared memory at every entry (1, 768 threads: more warps per SM; at C5
  // 2.48 against 3.18 ms for the force pass), or as 1 with two entries in
  // flight per lane (2)
  int fused_variant = 1;
  // half-width of the guard band of the mixed cutoff decisions ("tune band")
  float band_eps = 1.0e-4f;
  // run_host: the fused element force pass in out_parts parts, each part's node
  // velocities integrated and copied out while the next part's forces run
  // ("tune out_parts 0..8", 0: 4 parts from 65,536 elements on, else 1);
  // out_split is set while run_host enqueues such a step, parts_done /
  // part_bounds report what the force pass did
  int out_parts = 0, parts_done = 1;
  bool out_split = false;
  std::vector<int> part_bounds;
  cudaEvent_t ev_nvpart[8] = {};
  // "tune fprime fp64|fp32": F'(rho) of the atoms in the mixed density pass
  // from the FP64 spline at the FP64 density (default), or from the FP32 copy
  bool fprime64 = true;
  DBuf<int> d_fjj, d_fjj_off;
  DBuf<int4> d_intp4;  // lattice indices (i, j, k) of every type's rows
  // lanes per integration point ("tune ip_group N"; 0: from the row count, so
  // that rows x lanes reach the GPU's resident threads)
  int mixed_ip_group = 0;
  int maxlines = 0, max_nax = 0, max_naz = 0;
  DBuf<double> d_cutsq64, d_stage, d_part, d_lj5;
  std::vector<double> h_lj5;
  // regions, groups and post-force fixes (region_block.cpp, region_sphere.cpp,
  // group.cpp, fix_setforce.cpp, fix_viscous.cpp)
  struct Region {
    std::string id;
    int sphere = 0, interior = 1;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0}, c[3] = {0, 0, 0}, r = 0;
    bool match(double x, double y, double z) const {
      int in;
      if (sphere) {
        double dx = x - c[0], dy = y - c[1], dz = z - c[2];
        in = std::sqrt(dx * dx + dy * dy + dz * dz) <= r;
      } else {
        in = x >= lo[0] && x <= hi[0] && y >= lo[1] && y <= hi[1] && z >= lo[2] && z <= hi[2];
      }
      return !(in ^ interior);  // Region::match, region.cpp:96-99
    }
  };
  struct PostFix {
    int viscous = 0, bit = 1;
    int set[3] = {0, 0, 0};
    double val[3] = {0, 0, 0}, gamma = 0;
  };
  std::vector<Region> regions;
  std::vector<std::string> groups{"all"};
  std::vector<int> h_amask, h_emask;  // group bits of the local atoms / elements
  std::vector<PostFix> post_fixes;
  // fix deform: L(t) = L0 (1 + erate t) about the box centre, affine remap of
  // atom and node positions at the end of every step
  bool deform_on = false;
  double erate[3] = {0, 0, 0}, dL0[3] = {0, 0, 0}, dc0[3] = {0, 0, 0};
  long long deform_t0 = 0;
  DBuf<int> d_amask, d_emask;
  bool masks_dirty = true;
  // nodal-force surrogate (elements far from the atoms)
  cacg_mlp_t *sur = nullptr;
  double sur_tol = 1e-4, sur_dist = 0.0;
  DBuf<double> d_nodex0;
  bool have_x0 = false;
  DBuf<int> d_far;
  int nfar = 0;
  DBuf<unsigned char> d_skip;
  // re-test back-off of the far elements: steps to the next test, rejections
  // in a row; the elements due this step (indices into d_far) and their number
  DBuf<unsigned char> d_swait, d_sstreak;
  DBuf<int> d_sdue, d_sdue_n, d_sfar_due;
  DBuf<unsigned short> d_sfeat;  // bf16 features [nfar][64]
  DBuf<float> d_smean, d_sspread, d_sraw;
  DBuf<unsigned long long> d_scount;  // evaluated, accepted element-steps
  DBuf<double> d_v, d_f, d_xhold, d_rho, d_fp, d_mass;
  DBuf<int> d_type, d_tag, d_root, d_send;
  DBuf<int> d_abin, d_bcount, d_bstart, d_bmem, d_stencil;
  DBuf<double4> d_bx;
  DBuf<int> d_num, d_list;
  DBuf<int> d_snum, d_slist;  // per-step short lists (FP32 guarded cutoff test)
  int maxneigh = 64, stride = 0;
  // elements
  DBuf<double> d_ex, d_nodex, d_nodev, d_nodef, d_nodexhold, d_erho, d_emass, d_diag, d_fip,
      d_site_fp;
  DBuf<int> d_etype, d_etag, d_eroot, d_esend;
  DBuf<int> d_ebin, d_ebcount, d_ebstart, d_ebmem;
  DBuf<double4> d_ebx, d_site_x, d_subc;
  DBuf<int> d_enum, d_elist;
  int maxeneigh = 32, estride = 0;
  DBuf<int> d_row_elem, d_row_jj, d_row_first, d_site_base, d_ipnum, d_ipent;
  DBuf<int> d_sipnum, d_sipent;
  DBuf<int> d_force_rows, d_need, d_need_elem, d_site_flag, d_site_pos;
  int nforce = 0, nneed = 0;
  int maxip = 128, rowstride = 0;
  // tables
  DBuf<double> d_spa_int, d_weight, d_spa_inter, d_spa_csub, d_spa_isub, d_frho, d_rhor, d_z2r;
  DBuf<int> d_int_off, d_inter_off, d_numint, d_inter_num, d_node_list, d_list_isub,
      d_sub_first;
  DBuf<LJTabHost> d_ljtab;
  // scratch
  DBuf<int> d_flags, d_pos, d_scan, d_misc;
  int *h_pin = nullptr;  // pinned readback slots

  // state
  bool inited = false, setup_done = false, list_built = false, elists_built = false;
  long long ntimestep = 0, launches = 0;
  int ago = 0, nrebuild = 0;
  // rebuilds that kept the element lists (atoms alone moved past the trigger)
  long long nrebuild_atoms = 0;
  // a rebuild that only atoms triggered keeps the element lists and element
  // ghosts when no node has moved past the trigger since the element lists
  // were built and no element needs a periodic wrap: every pair within the
  // cutoff is then still in the lists (a site moves at most as far as the
  // farthest node of its element), so forces are unchanged.  Off in the
  // bit-exact mode, which follows the reference's full rebuild.
  bool lazy_elists = true;
  // device time of every rebuild (events around it)
  cudaEvent_t rb_ev[2] = {nullptr, nullptr};
  double rebuild_ms_total = 0.0;
  cudaEvent_t ev[10] = {};
  double t_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  bool timing = false;
  // CUDA graph of a step without a rebuild decision (captured once, replayed
  // until a rebuild, a reallocation or a configuration change)
  int mixed_block = 512;  // threads per block of the mixed persistent kernels ("tune block N")
  // a mixed step as two chains on two streams ("tune streams yes|no"): atoms
  // and element sites do not interact, so the atom chain (initial
  // integration, ghost update, density and force passes) and the element
  // chain meet only before the fixes and the final integration
  bool two_streams = true;
  cudaStream_t astream = nullptr;  // the atom chain's stream (higher priority)
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  // host-resident stepping (run_host): copy-in and copy-out streams and the
  // events that order the copies against the step's two chains
  cudaStream_t cin = nullptr, cout_s = nullptr;
  cudaEvent_t ev_ain = nullptr, ev_nin = nullptr, ev_xout = nullptr, ev_nxout = nullptr,
              ev_nvout = nullptr, ev_end = nullptr, ev_hstart = nullptr, ev_hdone = nullptr,
              ev_vout = nullptr, ev_acheck = nullptr, ev_apass = nullptr;
  // graph of a whole single-step run_host call on pinned buffers
  cudaGraphExec_t hexec = nullptr;
  bool hgraph_valid = false, hgraph_ok = true;
  unsigned long long hgraph_epoch = 0;
  long long hgraph_launches = 0;
  const void *hgraph_bufs[4] = {nullptr, nullptr, nullptr, nullptr};
  const void *hlast_bufs[4] = {nullptr, nullptr, nullptr, nullptr};  // the previous call's
  // neighbor unions staged in shared memory ("tune union yes"): the same pair
  // arithmetic over the build-order lists (the direct passes walk the
  // reordered lists, so sums differ in order only); at C2 they run at 8 warps
  // per SM and lose to the direct kernels (1.71 vs 0.77 ms for the density
  // pass when measured), so off by default
  bool mixed_union = false;
  long long list_builds = 0, union_of = -1;
  // the atom lists reordered for the mixed EAM passes (in-range entries
  // first), once per list build
  long long part_of = -1;
  DBuf<int> d_mlist;
  DBuf<int4> d_nnear;
  // packed coordinates at the reorder and their grid: the density pass skips
  // the far part of each list while no atom has moved 0.495 A since then
  DBuf<float4> d_xq_ref;
  bool mixed_cull = true;  // "tune cull yes|no"
  double ref_l0[3] = {0, 0, 0}, ref_g = 0;
  DBuf<int> d_union_j, d_union_n;
  DBuf<unsigned short> d_slot, d_sslot;
  bool ran = false;  // steps taken since init (positions may have left the box)
  bool oob_zeroed = false;  // d_misc[9] (packed-range counter) initialised
  bool use_graphs = true, graph_ok = true, graph_valid = false;
  cudaGraphExec_t gexec = nullptr;
  unsigned long long graph_epoch = 0;
  long long graph_launches = 0, graph_steps = 0;
  int eager_since = 0;
  // device step loop ("tune loop device|host"): one graph launch runs steps
  // back to back, the rebuild decision taken on the device (a WHILE node
  // around the step, an IF node around its force passes), until the wanted
  // steps are done or a step needs a rebuild, which the host then performs
  std::atomic<unsigned long long> epoch{0};  // allocations made in calls on this handle
  bool loop_device = false;
  DBuf<int> d_loop;
  cudaGraphExec_t lexec = nullptr;
  bool lgraph_valid = false;
  unsigned long long lgraph_epoch = 0;
  long long lgraph_pre = 0, lgraph_post = 0;  // kernels per iteration before / after the decision
  long long loop_launches = 0, host_decisions = 0;
  void invalidate_graph() {
    graph_valid = false;
    hgraph_valid = false;
    lgraph_valid = false;
    eager_since = 0;
  }
  bool capture_plain_step();
  void loop_prepare();
  bool add_loop(cudaGraph_t top, long long &pre, long long &post, bool *destroyable);
  bool capture_loop();
  void loop_arm(int want);
  int loop_finish(int want, long long pre, long long post);
  int run_loop(int n);
  std::vector<cudaEvent_t> pev;  // per-step phase events
  // with timing on: events around the main kernels of each step; kernel k of
  // step j is bracketed by events 2 (j KT_N + k) and 2 (j KT_N + k) + 1
  enum {
    KT_ATOM1 = 0,   // atom pass 1: LJ forces or EAM densities + F'
    KT_ATOM2,       // atom pass 2: EAM forces
    KT_ELEM_RHO,    // nodal densities (EAM element density pass)
    KT_ELEM_FORCE,  // integration-point forces
    KT_SUR,         // surrogate: features, ensemble, acceptance
    KT_SITES,       // element sites (FP64) or lattice lines (mixed)
    KT_APART,       // mixed atom-list reorder (returns at once unless due)
    KT_EPREP,       // mixed integration-point rows, reorder and line masks
    KT_SITE_FP,     // site F'(rho): per site (FP64) or per lattice line (mixed)
    KT_N
  };
  double t_kern[KT_N] = {};
  std::vector<cudaEvent_t> kev;
  std::vector<char> kev_used;
  size_t cur_step = 0;
  bool capturing = false;
  void kmark(int k, int end) {
    if (!timing || capturing) return;
    const size_t at = 2 * (cur_step * KT_N + (size_t) k) + (size_t) end;
    while (kev.size() <= at) {
      cudaEvent_t e;
      check(cudaEventCreate(&e), "event");
      kev.push_back(e);
      kev_used.push_back(0);
    }
    check(cudaEventRecord(kev[at], stream), "event record");
    kev_used[at] = 1;
  }
  std::vector<char> pev_used;  // marks recorded in the current run
  void mark(size_t k) {
    if (!timing) return;
    while (pev.size() <= k) {
      cudaEvent_t e;
      check(cudaEventCreate(&e), "event");
      pev.push_back(e);
      pev_used.push_back(0);
    }
    check(cudaEventRecord(pev[k], stream), "event record");
    pev_used[k] = 1;
  }

  ~cacg_context();

  // ---- helpers ----
  void sync() { check(cudaStreamSynchronize(stream), "sync"); }
  ElemTables etab() const {
    ElemTables t;
    t.spa_int = d_spa_int.p;
    t.weight = d_weight.p;
    t.spa_inter = d_spa_inter.p;
    t.int_off = d_int_off.p;
    t.inter_off = d_inter_off.p;
    t.numint = d_numint.p;
    t.inter_num = d_inter_num.p;
    t.node_list = d_node_list.p;
    t.spa_center_sub = d_spa_csub.p;
    t.spa_inter_sub = d_spa_isub.p;
    t.list_inter_sub = d_list_isub.p;
    t.sub_first = d_sub_first.p;
    t.nsub = nsub;
    return t;
  }
  EamTables eamtab() const {
    EamTables e;
    e.frho = d_frho.p;
    e.rhor = d_rhor.p;
    e.z2r = d_z2r.p;
    e.nr = nr;
    e.nrho = nrho;
    e.rdr = rdr;
    e.rdrho = rdrho;
    e.cutforcesq = cutforcesq;
    return e;
  }

  // Float threshold for the FP32 pre-test of a pair against cutsq: any pair
  // with exact rsq < cutsq has float rsq <= the returned value.  Coordinates
  // are bounded by the box plus the ghost margin plus a motion allowance; each
  // float coordinate is within u|x| (u = 2^-24) of the double, the float
  // difference within a further u|dx|, and the float sum of squares within 3u.
  float cut_pass(double cutsq) const {
    double X = 0.0;
    for (int d = 0; d < 3; d++)
      X = std::max(X, std::max(std::fabs(lo[d]), std::fabs(hi[d])) + cutghost[d] + max_size +
                          10.0 * skin + 1.0);
    const double u = std::ldexp(1.0, -24);
    const double rn = std::max(cutneighmax, std::sqrt(cutsq));
    const double delta = 2.0 * u * X * 1.001 + u * (rn + 1.0);
    const double guard = 4.0 * u * cutsq + (1.0 + 4.0 * u) * (2.0 * std::sqrt(3.0) * rn * delta +
                                                              3.0 * delta * delta);
    float c = (float) (cutsq + guard);
    return std::nextafter(std::nextafter(c, 3.0e38f), 3.0e38f);
  }
  float atom_cut_pass() const {
    if (pair_style == 2) return cut_pass(cutforcesq);
    double mx = 0.0;
    int nt = std::max(ntypes, 1);
    for (int i = 1; i <= nt; i++)
      for (int j = 1; j <= nt; j++) mx = std::max(mx, ljtab.cutsq[i * (MAXT + 1) + j]);
    return cut_pass(mx);
  }
  bool fast() const { return mode != CACG_FP64_EXACT; }

  // ---- commands ----
  void command(const std::string &line);
  void read_data(const std::string &path);
  void read_eam(const std::string &path, bool setfl = false, const std::string &element = "");
  void set_units(const std::string &style);

  // ---- path ----
  void init();
  void element_tables();
  void mixed_tables();
  void element_size();
  void setup_cut();
  void comm_setup();
  void setup_bins();
  void borders();
  void forward_comm(int which = 3);  // 1 atoms, 2 elements, 3 both
  void pbc();
  void neighbor_build();
  void neighbor_ebuild();
  void neighbor_nbuild();
  void pair_compute();
  void pair_compute_pass(int pass);
  void pair_compute_mixed(int pass);
  void pair_ecompute_mixed();
  void pair_ecompute();
  void nve_initial(int which = 3);
  void nve_final(int which = 3);
  void nve_nodes_final_range(int b0, int b1);
  void compute_thermo(double *out);
  void compute_centro(double *out);
  void region_cmd(const std::vector<std::string> &a);
  void group_cmd(const std::vector<std::string> &a);
  void fix_cmd(const std::vector<std::string> &a);
  int group_bit(const std::string &name) const;
  void post_force();
  void upload_masks();
  void check_packed_range();
  void nve_scales(TypeScale &a, TypeScale &e) const;
  // cell-relative packed coordinates of the mixed passes: cells of a
  // power-of-two size g cover the box, its ghost shell and a margin in
  // 4096 x 1024 x 1024 cells from the corner l0
  void pack_grid(double l0[3], double &g) const {
    double ext[3];
    const double margin =
        std::max(cutghost[0], std::max(cutghost[1], cutghost[2])) + max_size + cutneighmax;
    for (int d = 0; d < 3; d++) {
      l0[d] = lo[d] - margin;
      ext[d] = prd[d] + 2.0 * margin;
    }
    g = 1.0 / 1024.0;
    while (ext[0] / g > 4096.0 || ext[1] / g > 1024.0 || ext[2] / g > 1024.0) g *= 2.0;
  }
  void set_group(const std::string &name, const int *atom_in, const int *elem_in);
  void deform_step();
  void dump_xyz(const char *path);
  void dump_elements(const char *path, int append);
  void surrogate_reference(const double *nodex0);
  void surrogate_samples(float *x, float *t);
  void surrogate_attach(cacg_mlp_t *m, double tol, double dist);
  void surrogate_predict(const EamTables &e);
  int decide();
  void rebuild(int flags = 3);
  void borders_atoms();
  void borders_elems();
  void run(int n);
  void force_passes(long long b);  // b: phase-mark base of the step, < 0 for none
  void run_host(int n, double *x, double *v, double *nodex, double *nodev);
  bool fork_ok() const {
    return two_streams && mode == CACG_MIXED && !timing && nlocal > 0 && enlocal > 0;
  }
  template <class A, class E>
  void forked(A atoms, E elems, bool elems_first = false);
  void setup();
  void require_init() {
    if (!inited) init();
  }
};

cacg_context::~cacg_context() {
  DBuf<double4> *b4[] = {&d_x, &d_bx, &d_ebx, &d_site_x, &d_subc};
  for (auto *b : b4) b->release();
  d_xh.release();
  d_site_h.release();
  d_xl.release();
  d_rhor_val4.release();
  d_ftab.release();
  d_u.release();
  d_fp4.release();
  d_line_pos.release();
  d_line_rho.release();
  d_node_hl.release();
  d_spa_int_hl.release();
  d_fpf.release();
  d_line_mask.release();
  d_line_mask_f.release();
  d_nae.release();
  d_frac.release();
  d_fipf.release();
  d_wn.release();
  d_wnf.release();
  d_band.release();
  d_lat_rec.release();
  d_ip_q.release();
  d_ip_h.release();
  d_ip_l.release();
  d_row_fpf.release();
  d_row_start.release();
  d_ent.release();
  d_ent_near.release();
  d_nnear_row.release();
  d_node_ref.release();
  d_line_mask_n.release();
  d_line_mask_nf.release();
  d_row_isforce.release();
  d_ljf.release();
  d_cutsq64.release();
  d_stage.release();
  d_part.release();
  d_lj5.release();
  d_nodex0.release();
  d_amask.release();
  d_emask.release();
  d_union_j.release();
  d_mlist.release();
  d_nnear.release();
  d_xq_ref.release();
  d_union_n.release();
  d_slot.release();
  d_sslot.release();
  d_far.release();
  d_skip.release();
  d_sfeat.release();
  d_smean.release();
  d_sspread.release();
  d_sraw.release();
  d_scount.release();
  DBuf<double> *bd[] = {&d_v, &d_f, &d_xhold, &d_rho, &d_fp, &d_mass, &d_ex, &d_nodex, &d_nodev,
                        &d_nodef, &d_nodexhold, &d_erho, &d_emass, &d_diag, &d_fip, &d_site_fp,
                        &d_spa_int, &d_weight, &d_spa_inter, &d_spa_csub, &d_spa_isub, &d_frho,
                        &d_rhor, &d_z2r};
  for (auto *b : bd) b->release();
  DBuf<int> *bi[] = {&d_type, &d_tag, &d_root, &d_send, &d_abin, &d_bcount, &d_bstart, &d_bmem,
                     &d_stencil, &d_num, &d_list, &d_etype, &d_etag, &d_eroot, &d_esend,
                     &d_ebin, &d_ebcount, &d_ebstart, &d_ebmem, &d_enum, &d_elist,
                     &d_row_elem, &d_row_jj, &d_row_first, &d_site_base, &d_ipnum, &d_ipent,
                     &d_int_off, &d_inter_off, &d_numint, &d_inter_num, &d_node_list,
                     &d_list_isub, &d_sub_first, &d_flags, &d_pos, &d_scan, &d_misc,
                     &d_snum, &d_slist, &d_sipnum, &d_sipent, &d_force_rows, &d_need,
                     &d_need_elem, &d_site_flag, &d_site_pos, &d_loop};
  for (auto *b : bi) b->release();
  d_ljtab.release();
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  for (auto &e : pev) cudaEventDestroy(e);
  for (auto &e : kev) cudaEventDestroy(e);
  if (gexec) cudaGraphExecDestroy(gexec);
  if (lexec) cudaGraphExecDestroy(lexec);
  if (h_pin) cudaFreeHost(h_pin);
  if (fork_ev) cudaEventDestroy(fork_ev);
  if (hexec) cudaGraphExecDestroy(hexec);
  for (cudaEvent_t e : ev_nvpart)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : {ev_ain, ev_nin, ev_xout, ev_nxout, ev_nvout, ev_end, ev_hstart, ev_hdone,
                        ev_vout, ev_acheck, ev_apass})
    if (e) cudaEventDestroy(e);
  if (cin) cudaStreamDestroy(cin);
  if (cout_s) cudaStreamDestroy(cout_s);
  if (join_ev) cudaEventDestroy(join_ev);
  if (astream) cudaStreamDestroy(astream);
  if (stream) cudaStreamDestroy(stream);
}

// ------------------------------------------------------------------ commands

void cacg_context::set_units(const std::string &style) {
  if (style == "lj") {
    metal = false;
    ftm2v = 1.0;
    dt = 0.005;
    skin = 0.3;
  } else if (style == "metal") {
    metal = true;
    ftm2v = 1.0 / 1.0364269e-4;
    dt = 0.001;
    skin = 2.0;
  } else {
    fail(CACG_EINVAL, "Illegal units command");
  }
}

void cacg_context::command(const std::string &raw) {
  invalidate_graph();  // any command may change what a captured step would do
  std::string line = raw;
  size_t hash = line.find('#');
  if (hash != std::string::npos) line = line.substr(0, hash);
  auto w = split_words(line);
  if (w.empty()) return;
  const std::string &c = w[0];
  std::vector<std::string> a(w.begin() + 1, w.end());
  if (c == "units") {
    if (a.size() != 1) fail(CACG_EINVAL, "Illegal units command");
    if (box_set) fail(CACG_EINVAL, "Units command after simulation box is defined");
    set_units(a[0]);
  } else if (c == "dimension") {
    if (a.size() != 1 || a[0] != "3") fail(CACG_EINVAL, "Only 3d CAC is supported");
  } else if (c == "atom_style") {
    if (a.empty() || a[0] != "atomic") fail(CACG_EINVAL, "Only atom_style atomic is supported");
  } else if (c == "newton" || c == "processors") {
    // single GPU: no processor grid; newton flag unused by the full lists
  } else if (c == "boundary") {
    if (a.size() != 3) fail(CACG_EINVAL, "Illegal boundary command");
    for (int d = 0; d < 3; d++) {
      char c0 = a[d][0], c1 = a[d].size() == 1 ? a[d][0] : a[d][1];
      if (!strchr("pfsm", c0) || !strchr("pfsm", c1)) fail(CACG_EINVAL, "Illegal boundary command");
      if ((c0 == 'p') != (c1 == 'p')) fail(CACG_EINVAL, "Both sides of boundary must be periodic");
      if (c0 == 's' || c0 == 'm' || c1 == 's' || c1 == 'm')
        fail(CACG_EINVAL, "Shrink-wrapped boundaries are not supported");
      periodic[d] = c0 == 'p';
    }
  } else if (c == "timestep") {
    if (a.size() != 1) fail(CACG_EINVAL, "Illegal timestep command");
    dt = numeric(a[0]);
  } else if (c == "elementsplit") {
    if (a.size() != 1) fail(CACG_EINVAL, "Illegal element_split command");
    nsplit = inumeric(a[0]);
    if (nsplit < 1) fail(CACG_EINVAL, "Illegal element_split command");
  } else if (c == "neighbor") {
    if (a.size() != 2) fail(CACG_EINVAL, "Illegal neighbor command");
    skin = numeric(a[0]);
    if (skin < 0.0) fail(CACG_EINVAL, "Illegal neighbor command");
    if (a[1] != "bin") fail(CACG_EINVAL, "Only neighbor style bin is supported");
  } else if (c == "neigh_modify") {
    size_t i = 0;
    while (i < a.size()) {
      if (i + 1 >= a.size()) fail(CACG_EINVAL, "Illegal neigh_modify command");
      const std::string &k = a[i], &v = a[i + 1];
      if (k == "every") {
        every = inumeric(v);
        if (every <= 0) fail(CACG_EINVAL, "Illegal neigh_modify command");
      } else if (k == "delay") {
        delay = inumeric(v);
        if (delay < 0) fail(CACG_EINVAL, "Illegal neigh_modify command");
      } else if (k == "check") {
        if (v == "yes") dist_check = 1;
        else if (v == "no") dist_check = 0;
        else fail(CACG_EINVAL, "Illegal neigh_modify command");
      } else if (k == "binsize") {
        binsize_user = numeric(v);
        if (binsize_user <= 0.0) binsize_user = 0.0;
      } else if (k == "one") {
        oneatom = inumeric(v);
      } else if (k == "page") {
        pgsize = inumeric(v);
      } else {
        fail(CACG_EINVAL, "Illegal neigh_modify command");
      }
      i += 2;
    }
  } else if (c == "read_data") {
    if (a.size() < 1) fail(CACG_EINVAL, "Illegal read_data command");
    read_data(a[0]);
  } else if (c == "pair_style") {
    if (a.empty()) fail(CACG_EINVAL, "Illegal pair_style command");
    lj_raw = false;
    if (a[0] == "lj/cut") {
      if (a.size() != 2) fail(CACG_EINVAL, "Illegal pair_style command");
      pair_style = 1;
      cut_global = numeric(a[1]);
    } else if (a[0] == "eam" || a[0] == "eam/alloy") {
      if (a.size() != 1) fail(CACG_EINVAL, "Illegal pair_style command");
      pair_style = 2;
      eam_setfl = a[0] == "eam/alloy";
    } else {
      fail(CACG_EINVAL, "Unknown pair style %s", a[0].c_str());
    }
    inited = false;
  } else if (c == "pair_coeff") {
    if (!box_set) fail(CACG_EINVAL, "Pair_coeff command before simulation box is defined");
    if (pair_style == 0) fail(CACG_EINVAL, "Pair_coeff command before pair_style is defined");
    int ilo, ihi, jlo, jhi;
    int nt = ntypes > 0 ? ntypes : 1;
    if (pair_style == 1) {
      if (a.size() < 4 || a.size() > 5) fail(CACG_EINVAL, "Incorrect args for pair coefficients");
      lj_raw = false;  // coefficients again, instead of handed-over tables
      bounds(a[0], nt, ilo, ihi);
      bounds(a[1], nt, jlo, jhi);
      double e = numeric(a[2]), s = numeric(a[3]);
      double cc = a.size() == 5 ? numeric(a[4]) : cut_global;
      int count = 0;
      for (int i = ilo; i <= ihi; i++)
        for (int j = std::max(jlo, i); j <= jhi; j++) {
          eps[i][j] = e;
          sig[i][j] = s;
          cutp[i][j] = cc;
          setflag[i][j] = 1;
          count++;
        }
      if (count == 0) fail(CACG_EINVAL, "Incorrect args for pair coefficients");
    } else if (eam_setfl) {
      // pair_coeff * * file el1 ... elN: one element name per atom type
      if (a.size() != 3 + (size_t) nt || a[0] != "*" || a[1] != "*")
        fail(CACG_EINVAL, "Incorrect args for pair coefficients");
      for (int t = 1; t < nt; t++)
        if (a[3 + t] != a[3]) fail(CACG_EINVAL, "one species per system on this path");
      read_eam(a[2], true, a[3]);
      for (int i = 1; i <= nt; i++) {
        setflag[i][i] = 1;
        amass[i] = eam_mass;
      }
    } else {
      if (a.size() != 3) fail(CACG_EINVAL, "Incorrect args for pair coefficients");
      bounds(a[0], nt, ilo, ihi);
      bounds(a[1], nt, jlo, jhi);
      read_eam(a[2]);
      int count = 0;
      for (int i = ilo; i <= ihi; i++)
        for (int j = std::max(jlo, i); j <= jhi; j++)
          if (i == j) {
            setflag[i][i] = 1;
            amass[i] = eam_mass;  // PairEAM::coeff sets the type mass (pair_eam.cpp:152-161)
            count++;
          }
      if (count == 0) fail(CACG_EINVAL, "Incorrect args for pair coefficients");
    }
    inited = false;
  } else if (c == "fix") {
    fix_cmd(a);
  } else if (c == "region") {
    region_cmd(a);
  } else if (c == "group") {
    group_cmd(a);
  } else if (c == "run") {
    if (a.size() < 1) fail(CACG_EINVAL, "Illegal run command");
    run(inumeric(a[0]));
  } else if (c == "tune") {
    // tune block 128|256|512: threads per block of the mixed-precision kernels
    // tune union yes|no: neighbor unions staged in shared memory (EAM atom passes)
    // tune ip_group 0|4|8|16: lanes per integration point in the mixed element
    //   passes (0: chosen from the row count)
    // tune cull yes|no: the mixed EAM density pass skips list entries that no
    //   displacement since the list reorder can bring within the cutoff
    // tune streams yes|no: a mixed step's atom and element chains on two streams
    // tune fprime fp64|fp32: F'(rho) of the atoms in the mixed density pass
    // tune fused yes|no: the mixed element passes one warp per element
    //   (when every list entry references its row's own element)
    // tune elists lazy|eager: in the FP64 and mixed modes a rebuild that only
    //   atoms triggered keeps the element lists and ghosts (lazy, the default)
    // tune loop device|host: steps run as one graph launch with the rebuild
    //   decision on the device (with graphs on, no box deformation), or one
    //   graph launch per step without a decision and eager decision steps
    //   (host, the default)
    // tune out_parts N: run_host splits the fused element force pass in N parts
    //   and copies each part's node velocities out while the next part runs
    //   (1 to 8; 0, the default: 4 from 65,536 elements on, else 1;
    //   bit-identical)
    // tune band W: the guard band of the mixed cutoff decisions, cutsq (1 +- W)
    //   (default 1e-4, at most 0.1); a wider band only moves more pairs to the
    //   FP64 decision, the decisions and forces stay the same
    if (a.size() != 2) fail(CACG_EINVAL, "Illegal tune command");
    if (a[0] == "block") {
      int b = inumeric(a[1]);
      if (b != 128 && b != 256 && b != 512) fail(CACG_EINVAL, "tune block takes 128, 256 or 512");
      mixed_block = b;
    } else if (a[0] == "ip_group") {
      int gsz = inumeric(a[1]);
      if (gsz != 0 && gsz != 4 && gsz != 8 && gsz != 16)
        fail(CACG_EINVAL, "tune ip_group takes 0, 4, 8 or 16");
      mixed_ip_group = gsz;
    } else if (a[0] == "cull") {
      if (a[1] != "yes" && a[1] != "no") fail(CACG_EINVAL, "tune cull takes yes or no");
      mixed_cull = a[1] == "yes";
    } else if (a[0] == "union") {
      if (a[1] != "yes" && a[1] != "no") fail(CACG_EINVAL, "tune union takes yes or no");
      mixed_union = a[1] == "yes";
    } else if (a[0] == "streams") {
      if (a[1] != "yes" && a[1] != "no") fail(CACG_EINVAL, "tune streams takes yes or no");
      two_streams = a[1] == "yes";
      invalidate_graph();
    } else if (a[0] == "fprime") {
      if (a[1] != "fp64" && a[1] != "fp32") fail(CACG_EINVAL, "tune fprime takes fp64 or fp32");
      fprime64 = a[1] == "fp64";
      invalidate_graph();
    } else if (a[0] == "band") {
      const double w = numeric(a[1]);
      if (!(w >= 1.0e-4 && w <= 0.1)) fail(CACG_EINVAL, "tune band takes 1e-4 to 0.1");
      band_eps = (float) w;
      invalidate_graph();
    } else if (a[0] == "out_parts") {
      const int v = inumeric(a[1]);
      if (v < 0 || v > 8) fail(CACG_EINVAL, "tune out_parts takes 0 to 8");
      out_parts = v;
      invalidate_graph();
    } else if (a[0] == "fused_variant") {
      const int v = inumeric(a[1]);
      if (v < 0 || v > 2) fail(CACG_EINVAL, "tune fused_variant takes 0, 1 or 2");
      fused_variant = v;
      invalidate_graph();
    } else if (a[0] == "fused") {
      if (a[1] != "yes" && a[1] != "no") fail(CACG_EINVAL, "tune fused takes yes or no");
      fused_on = a[1] == "yes";
      invalidate_graph();
    } else if (a[0] == "elists") {
      if (a[1] != "lazy" && a[1] != "eager") fail(CACG_EINVAL, "tune elists takes lazy or eager");
      lazy_elists = a[1] == "lazy";
    } else if (a[0] == "loop") {
      if (a[1] != "device" && a[1] != "host") fail(CACG_EINVAL, "tune loop takes device or host");
      loop_device = a[1] == "device";
      invalidate_graph();
    } else {
      fail(CACG_EINVAL, "Illegal tune command");
    }
  } else if (c == "thermo" || c == "thermo_style" || c == "dump" || c == "velocity") {
    // output and setup commands outside this path are accepted and ignored
  } else {
    fail(CACG_EINVAL, "Unknown command: %s", raw.c_str());
  }
}

// ------------------------------------------------------------------ regions, groups, fixes

// region ID block xlo xhi ylo yhi zlo zhi [side in|out] [units box|lattice]
// (region_block.cpp:15-67, INF = +-1e20, EDGE = the box face);
// region ID sphere xc yc zc r (region_sphere.cpp:15-32)
void cacg_context::region_cmd(const std::vector<std::string> &a) {
  if (a.size() < 2) fail(CACG_EINVAL, "Illegal region command");
  Region r;
  r.id = a[0];
  size_t iarg;
  if (a[1] == "block") {
    if (a.size() < 8) fail(CACG_EINVAL, "Illegal region block command");
    for (int d = 0; d < 3; d++) {
      for (int side = 0; side < 2; side++) {
        const std::string &v = a[2 + 2 * d + side];
        double &dst = side ? r.hi[d] : r.lo[d];
        if (v == "INF" || v == "EDGE") {
          if (!box_set) fail(CACG_EINVAL, "Cannot use region INF or EDGE when box does not exist");
          if (v == "INF") dst = side ? 1.0e20 : -1.0e20;
          else dst = side ? hi[d] : lo[d];
        } else {
          dst = numeric(v);
        }
      }
    }
    if (r.lo[0] > r.hi[0] || r.lo[1] > r.hi[1] || r.lo[2] > r.hi[2])
      fail(CACG_EINVAL, "Illegal region block command");
    iarg = 8;
  } else if (a[1] == "sphere") {
    if (a.size() < 6) fail(CACG_EINVAL, "Illegal region sphere command");
    r.sphere = 1;
    for (int d = 0; d < 3; d++) r.c[d] = numeric(a[2 + d]);
    r.r = numeric(a[5]);
    if (r.r < 0.0) fail(CACG_EINVAL, "Illegal region sphere command");
    iarg = 6;
  } else {
    fail(CACG_EINVAL, "Unknown region style %s", a[1].c_str());
  }
  for (; iarg < a.size(); iarg += 2) {  // Region::options, region.cpp:55-84
    if (iarg + 1 >= a.size()) fail(CACG_EINVAL, "Illegal region command");
    if (a[iarg] == "units") {
      if (a[iarg + 1] != "box" && a[iarg + 1] != "lattice") fail(CACG_EINVAL, "Illegal region command");
    } else if (a[iarg] == "side") {
      if (a[iarg + 1] == "in") r.interior = 1;
      else if (a[iarg + 1] == "out") r.interior = 0;
      else fail(CACG_EINVAL, "Illegal region command");
    } else {
      fail(CACG_EINVAL, "Illegal region command");
    }
  }
  for (auto &q : regions)
    if (q.id == r.id) fail(CACG_EINVAL, "Reuse of region ID");
  regions.push_back(r);
}

int cacg_context::group_bit(const std::string &name) const {
  for (size_t g = 0; g < groups.size(); g++)
    if (groups[g] == name) return 1 << g;
  return 0;
}

// group ID region RID | subtract G1 G2 ... | union G1 ... (group.cpp:80-200):
// atoms by position, elements by centre, at the time of the command
void cacg_context::group_cmd(const std::vector<std::string> &a) {
  if (a.size() < 2) fail(CACG_EINVAL, "Illegal group command");
  int bit = group_bit(a[0]);
  if (!bit) {
    if (groups.size() == 32) fail(CACG_EINVAL, "Too many groups");
    groups.push_back(a[0]);
    bit = 1 << (groups.size() - 1);
  }
  // current positions: the device copy once it exists
  std::vector<double> ax(h_x), ex(h_ex);
  if (inited) {
    std::vector<double4> x4(std::max(nlocal, 1));
    if (nlocal)
      check(cudaMemcpyAsync(x4.data(), d_x.p, sizeof(double4) * nlocal, cudaMemcpyDeviceToHost, stream), "x");
    ex.assign((size_t) 3 * enlocal, 0.0);
    if (enlocal)
      check(cudaMemcpyAsync(ex.data(), d_ex.p, sizeof(double) * 3 * enlocal, cudaMemcpyDeviceToHost, stream), "ex");
    sync();
    ax.assign((size_t) 3 * nlocal, 0.0);
    for (int i = 0; i < nlocal; i++) {
      ax[3 * i] = x4[i].x;
      ax[3 * i + 1] = x4[i].y;
      ax[3 * i + 2] = x4[i].z;
    }
  }
  const int na = (int) (ax.size() / 3), ne = (int) (ex.size() / 3);
  h_amask.resize(na, 1);
  h_emask.resize(ne, 1);
  if (a[1] == "region") {
    if (a.size() != 3) fail(CACG_EINVAL, "Illegal group command");
    const Region *r = nullptr;
    for (auto &q : regions)
      if (q.id == a[2]) r = &q;
    if (!r) fail(CACG_EINVAL, "Group region ID does not exist");
    for (int i = 0; i < na; i++)
      if (r->match(ax[3 * i], ax[3 * i + 1], ax[3 * i + 2])) h_amask[i] |= bit;
    for (int i = 0; i < ne; i++)
      if (r->match(ex[3 * i], ex[3 * i + 1], ex[3 * i + 2])) h_emask[i] |= bit;
  } else if (a[1] == "subtract" || a[1] == "union") {
    if (a.size() < (a[1] == "subtract" ? 4u : 3u)) fail(CACG_EINVAL, "Illegal group command");
    std::vector<int> bits;
    for (size_t k = 2; k < a.size(); k++) {
      int b = group_bit(a[k]);
      if (!b) fail(CACG_EINVAL, "Group ID does not exist");
      bits.push_back(b);
    }
    for (std::vector<int> *mk : {&h_amask, &h_emask}) {
      for (int &m : *mk) {
        if (a[1] == "union") {
          for (int b : bits)
            if (m & b) m |= bit;
        } else {
          if (m & bits[0]) m |= bit;
          for (size_t k = 1; k < bits.size(); k++)
            if (m & bits[k]) m &= ~bit;
        }
      }
    }
  } else {
    fail(CACG_EINVAL, "Illegal group command");
  }
  masks_dirty = true;
}

// fix ID group nve | setforce fx fy fz (NULL keeps a component) | viscous gamma
void cacg_context::fix_cmd(const std::vector<std::string> &a) {
  if (a.size() < 3) fail(CACG_EINVAL, "Illegal fix command");
  const int bit = group_bit(a[1]);
  if (!bit) fail(CACG_EINVAL, "Could not find fix group ID");
  if (a[2] == "nve") {
    if (a[1] != "all") fail(CACG_EINVAL, "fix nve applies to group all here");
    fix_nve = true;
  } else if (a[2] == "setforce") {  // fix_setforce.cpp:18-60
    if (a.size() < 6) fail(CACG_EINVAL, "Illegal fix setforce command");
    PostFix f;
    f.bit = bit;
    for (int d = 0; d < 3; d++)
      if (a[3 + d] != "NULL") {
        f.set[d] = 1;
        f.val[d] = numeric(a[3 + d]);
      }
    post_fixes.push_back(f);
  } else if (a[2] == "deform") {
    // fix ID all deform 1 x|y|z erate R ... [remap x]: the reference has no
    // box deformation; this follows the engineering strain-rate convention,
    // L(t) = L0 (1 + R t) with the centre fixed, positions remapped affinely
    if (a[1] != "all") fail(CACG_EINVAL, "fix deform applies to group all here");
    if (a.size() < 7 || inumeric(a[3]) != 1) fail(CACG_EINVAL, "Illegal fix deform command");
    if (!box_set) fail(CACG_EINVAL, "fix deform before the box is defined");
    double er[3] = {0, 0, 0};
    size_t k = 4;
    while (k < a.size()) {
      if (a[k] == "remap" && k + 1 < a.size() && a[k + 1] == "x") {
        k += 2;
        continue;
      }
      int d = a[k] == "x" ? 0 : a[k] == "y" ? 1 : a[k] == "z" ? 2 : -1;
      if (d < 0 || k + 2 >= a.size() || a[k + 1] != "erate") fail(CACG_EINVAL, "Illegal fix deform command");
      er[d] = numeric(a[k + 2]);
      k += 3;
    }
    for (int d = 0; d < 3; d++) {
      erate[d] = er[d];
      dL0[d] = hi[d] - lo[d];
      dc0[d] = 0.5 * (lo[d] + hi[d]);
    }
    deform_t0 = ntimestep;
    deform_on = er[0] != 0.0 || er[1] != 0.0 || er[2] != 0.0;
  } else if (a[2] == "viscous") {  // fix_viscous.cpp:14-30
    if (a.size() < 4) fail(CACG_EINVAL, "Illegal fix viscous command");
    PostFix f;
    f.viscous = 1;
    f.bit = bit;
    f.gamma = numeric(a[3]);
    post_fixes.push_back(f);
  } else {
    fail(CACG_EINVAL, "Fix style %s is not on this path", a[2].c_str());
  }
}

// Modify::post_force (modify.cpp:663-669): each fix in order, atoms then nodes
// group membership from flags per local atom / element (nonzero = member),
// e.g. clamped slabs of many replicas at once
void cacg_context::set_group(const std::string &name, const int *atom_in, const int *elem_in) {
  int bit = group_bit(name);
  if (!bit) {
    if (groups.size() == 32) fail(CACG_EINVAL, "Too many groups");
    groups.push_back(name);
    bit = 1 << (groups.size() - 1);
  }
  const int na = inited ? nlocal : (int) (h_x.size() / 3);
  const int ne = inited ? enlocal : (int) (h_ex.size() / 3);
  h_amask.resize(na, 1);
  h_emask.resize(ne, 1);
  for (int i = 0; i < na; i++) {
    if (atom_in && atom_in[i]) h_amask[i] |= bit;
    else h_amask[i] &= ~bit;
  }
  for (int i = 0; i < ne; i++) {
    if (elem_in && elem_in[i]) h_emask[i] |= bit;
    else h_emask[i] &= ~bit;
  }
  masks_dirty = true;
  invalidate_graph();
}

void cacg_context::upload_masks() {
  if (!masks_dirty || post_fixes.empty()) return;
  std::vector<int> am(h_amask), em(h_emask);
  am.resize(std::max(nlocal, 1), 1);
  em.resize(std::max(enlocal, 1), 1);
  upload(d_amask, am, stream);
  upload(d_emask, em, stream);
  masks_dirty = false;
}

void cacg_context::post_force() {
  if (post_fixes.empty()) return;
  cudaStream_t s = stream;
  upload_masks();
  for (const PostFix &f : post_fixes) {
    if (f.viscous) {
      if (nlocal) launch_viscous(d_f.p, d_v.p, d_amask.p, nlocal, 1, f.bit, f.gamma, s);
      if (enlocal) launch_viscous(d_nodef.p, d_nodev.p, d_emask.p, enlocal, NPE, f.bit, f.gamma, s);
    } else {
      if (nlocal) launch_setforce(d_f.p, d_amask.p, nlocal, 1, f.bit, f.set, f.val, s);
      if (enlocal) launch_setforce(d_nodef.p, d_emask.p, enlocal, NPE, f.bit, f.set, f.val, s);
    }
    launches += (nlocal > 0) + (enlocal > 0);
  }
}

void cacg_context::deform_step() {
  if (!deform_on) return;
  cudaStream_t s = stream;
  const double t = (double) (ntimestep - deform_t0) * dt;
  for (int d = 0; d < 3; d++) {
    if (erate[d] == 0.0) continue;
    const double L = dL0[d] * (1.0 + erate[d] * t);
    const double nlo = dc0[d] - 0.5 * L, olo = lo[d];
    const double f = L / prd[d];
    launch_affine(reinterpret_cast<double *>(d_x.p) + d, nlocal, 4, olo, nlo, f, s);
    launch_affine(d_nodex.p + d, NPE * enlocal, 3, olo, nlo, f, s);
    launch_affine(d_ex.p + d, enlocal, 3, olo, nlo, f, s);
    launches += 3;
    lo[d] = nlo;
    hi[d] = dc0[d] + 0.5 * L;
    prd[d] = L;
  }
  // ghost images are owners + pbc * prd: the shifts follow the new box, and
  // the ghosts follow their remapped owners now (the next step would refresh
  // them anyway; a force call between steps must not see the old images)
  for (auto &w : swaps)
    for (int d = 0; d < 3; d++) w.d[d] = (d == w.dim ? w.pbc : 0) * prd[d];
  forward_comm();
}

// ------------------------------------------------------------------ read_data

namespace {

void remap(double *x, const double *lo, const double *hi, const double *prd, const int *per) {
  // Domain::remap, domain.cpp:389-476
  for (int d = 0; d < 3; d++) {
    if (!per[d]) continue;
    while (x[d] < lo[d]) x[d] += prd[d];
    while (x[d] >= hi[d]) x[d] -= prd[d];
    x[d] = std::max(x[d], lo[d]);
  }
}

bool blank(const std::string &s) { return s.find_first_not_of(" \t\r\n") == std::string::npos; }

std::string trim(const std::string &s) {
  size_t a = s.find_first_not_of(" \t\r\n");
  if (a == std::string::npos) return "";
  size_t b = s.find_last_not_of(" \t\r\n");
  return s.substr(a, b - a + 1);
}

}  // namespace

void cacg_context::read_data(const std::string &path) {
  std::ifstream in(path);
  if (!in) fail(CACG_EIO, "Cannot open file %s", path.c_str());
  std::string line;
  std::getline(in, line);  // first line skipped
  long long natoms = 0, nelem = 0;
  int nat = 0, net = 0;
  double blo[3] = {0, 0, 0}, bhi[3] = {0, 0, 0};
  std::string keyword;
  // header (read_data.cpp:277-367)
  while (std::getline(in, line)) {
    std::string l = line;
    size_t hash = l.find('#');
    if (hash != std::string::npos) l = l.substr(0, hash);
    if (blank(l)) continue;
    if (l.find("atoms") != std::string::npos) natoms = atoll(l.c_str());
    else if (l.find("elements") != std::string::npos) nelem = atoll(l.c_str());
    else if (l.find("xlo xhi") != std::string::npos) sscanf(l.c_str(), "%lg %lg", &blo[0], &bhi[0]);
    else if (l.find("ylo yhi") != std::string::npos) sscanf(l.c_str(), "%lg %lg", &blo[1], &bhi[1]);
    else if (l.find("zlo zhi") != std::string::npos) sscanf(l.c_str(), "%lg %lg", &blo[2], &bhi[2]);
    else if (l.find("atom types") != std::string::npos) nat = atoi(l.c_str());
    else if (l.find("element types") != std::string::npos) net = atoi(l.c_str());
    else {
      keyword = trim(l);
      break;
    }
  }
  if (nat < 1 || nat > MAXT) fail(CACG_EINVAL, "unsupported number of atom types %d", nat);
  if (net > MAXT) fail(CACG_EINVAL, "unsupported number of element types %d", net);
  for (int d = 0; d < 3; d++) {
    if (!(blo[d] < bhi[d])) fail(CACG_EINVAL, "Box bounds are invalid");
    lo[d] = blo[d];
    hi[d] = bhi[d];
    prd[d] = hi[d] - lo[d];
  }
  box_set = true;
  ntypes = nat;
  netypes = net;
  h_x.clear(); h_v.clear(); h_type.clear(); h_tag.clear();
  h_amask.clear();
  masks_dirty = true;
  h_ex.clear(); h_nodex.clear(); h_nodev.clear(); h_etype.clear(); h_etag.clear();
  h_emask.clear();
  masks_dirty = true;
  std::vector<int> eid_to_index;
  auto next_lines = [&](long long n, std::vector<std::string> &out) {
    out.clear();
    // one blank line follows the keyword (parse_keyword reads it)
    std::getline(in, line);
    while ((long long) out.size() < n) {
      if (!std::getline(in, line)) fail(CACG_EIO, "Unexpected end of data file");
      out.push_back(line);
    }
  };
  std::vector<std::string> rows;
  while (!keyword.empty()) {
    if (keyword == "Masses") {
      next_lines(nat, rows);
      for (auto &r : rows) {
        int t;
        double m;
        if (sscanf(r.c_str(), "%d %lg", &t, &m) != 2 || t < 1 || t > nat)
          fail(CACG_EINVAL, "Invalid type for mass set");
        if (m <= 0.0) fail(CACG_EINVAL, "Invalid mass value");
        amass[t] = m;
      }
    } else if (keyword == "NAAE") {
      next_lines(net, rows);
      for (auto &r : rows) {
        int t, nx, ny, nz;
        if (sscanf(r.c_str(), "%d %d %d %d", &t, &nx, &ny, &nz) != 4)
          fail(CACG_EINVAL, "Invalid nae line in data file");
        if (t < 1 || t > net) fail(CACG_EINVAL, "Invalid type for nae set");
        if (nx < 2 || ny < 2 || nz < 2) fail(CACG_EINVAL, "Invalid naae values");
        nae[t][0] = nx;
        nae[t][1] = ny;
        nae[t][2] = nz;
      }
    } else if (keyword == "Numint") {
      next_lines(net, rows);
      for (auto &r : rows) {
        int t, n;
        if (sscanf(r.c_str(), "%d %d", &t, &n) != 2) fail(CACG_EINVAL, "Invalid numint line in data file");
        if (t < 1 || t > net) fail(CACG_EINVAL, "Invalid type for numint set");
        numint[t] = n;
        intp[t].assign(3 * (size_t) n, 0);
        weight[t].assign((size_t) n, 0.0);
      }
    } else if (keyword == "Intp") {
      long long tot = 0;
      for (int t = 1; t <= net; t++) tot += numint[t];
      next_lines(tot, rows);
      for (auto &r : rows) {
        auto w = split_words(r);
        if (w.size() < 6) fail(CACG_EINVAL, "Invalid Intp line in data file");
        int t = atoi(w[0].c_str()), m = atoi(w[1].c_str()) - 1;
        if (t < 1 || t > net || m < 0 || m >= numint[t]) fail(CACG_EINVAL, "Invalid Intp index");
        intp[t][3 * m] = atoi(w[2].c_str());
        intp[t][3 * m + 1] = atoi(w[3].c_str());
        intp[t][3 * m + 2] = atoi(w[4].c_str());
        weight[t][m] = atof(w[5].c_str());
      }
    } else if (keyword == "Atoms") {
      next_lines(natoms, rows);
      for (auto &r : rows) {
        auto w = split_words(r);
        if (w.size() != 5 && w.size() != 8) fail(CACG_EINVAL, "Incorrect atom format in data file");
        double x[3] = {atof(w[2].c_str()), atof(w[3].c_str()), atof(w[4].c_str())};
        remap(x, lo, hi, prd, periodic);
        int t = atoi(w[1].c_str());
        if (t < 1 || t > nat) fail(CACG_EINVAL, "Invalid atom type in Atoms section of data file");
        bool inside = true;
        for (int d = 0; d < 3; d++) {
          double l = lo[d], h = hi[d];
          if (periodic[d]) {
            l -= prd[d] * 1.0e-6;
            h += prd[d] * 1.0e-6;
          }
          inside = inside && x[d] >= l && x[d] < h;
        }
        if (!inside) fail(CACG_EINVAL, "Did not assign all atoms correctly");
        h_tag.push_back(atoi(w[0].c_str()));
        h_type.push_back(t);
        for (int d = 0; d < 3; d++) {
          h_x.push_back(x[d]);
          h_v.push_back(0.0);
        }
      }
    } else if (keyword == "Elements") {
      next_lines(nelem, rows);
      for (auto &r : rows) {
        auto w = split_words(r);
        if (w.size() != 5 && w.size() != 8) fail(CACG_EINVAL, "Incorrect element format in data file");
        double x[3] = {atof(w[2].c_str()), atof(w[3].c_str()), atof(w[4].c_str())};
        remap(x, lo, hi, prd, periodic);
        int t = atoi(w[1].c_str());
        if (t < 1 || t > net) fail(CACG_EINVAL, "Invalid atom type in Elements section of data file");
        int id = atoi(w[0].c_str());
        if (id >= (int) eid_to_index.size()) eid_to_index.resize(id + 1, -1);
        eid_to_index[id] = (int) h_etype.size();
        h_etag.push_back(id);
        h_etype.push_back(t);
        for (int d = 0; d < 3; d++) h_ex.push_back(x[d]);
      }
      h_nodex.assign(24 * h_etype.size(), 0.0);
      h_nodev.assign(24 * h_etype.size(), 0.0);
    } else if (keyword == "Nodes") {
      next_lines(nelem * NPE, rows);
      for (auto &r : rows) {
        auto w = split_words(r);
        if (w.size() != 6 && w.size() != 9) fail(CACG_EINVAL, "Incorrect node format in data file");
        int id = atoi(w[0].c_str()), k = atoi(w[1].c_str()) - 1;
        if (id < 0 || id >= (int) eid_to_index.size() || eid_to_index[id] < 0 || k < 0 || k >= NPE)
          fail(CACG_EINVAL, "Invalid node line in data file");
        int e = eid_to_index[id];
        for (int d = 0; d < 3; d++) h_nodex[24 * e + 3 * k + d] = atof(w[2 + d].c_str());
        if (w.size() == 9)
          for (int d = 0; d < 3; d++) h_nodev[24 * e + 3 * k + d] = atof(w[5 + d].c_str());
      }
    } else {
      fail(CACG_EINVAL, "Unknown identifier in data file: %s", keyword.c_str());
    }
    keyword.clear();
    while (std::getline(in, line)) {
      if (!blank(line) && line.find_first_not_of(" \t") != std::string::npos &&
          line[line.find_first_not_of(" \t")] != '#') {
        keyword = trim(line.substr(0, line.find('#')));
        break;
      }
    }
  }
  if ((long long) h_type.size() != natoms) fail(CACG_EINVAL, "Did not assign all atoms correctly");
  if ((long long) h_etype.size() != nelem) fail(CACG_EINVAL, "Did not assign all elements correctly");
  nlocal = (int) h_type.size();
  enlocal = (int) h_etype.size();
  inited = setup_done = list_built = elists_built = false;
}

// PairEAM::read_file + file2array + array2spline (pair_eam.cpp:197-580)
// The reference's funcfl variant (PairEAM::read_file, pair_eam.cpp:197-248):
// comment, "Z mass", "Nrho drho Nr dr cut", F(rho), rho(r), r*phi(r).
// With setfl (the eam/alloy format; the reference has no reader for it):
// three comments, "N el1 ... elN", "Nrho drho Nr dr cut", then for each
// element "Z mass a lattice", F(rho), rho(r), then the r*phi(r) tables of the
// pairs (i >= j).  One species is on this path (the element kernels are
// type-1 only), so a setfl file supplies `element`'s F and rho and the
// element-element r*phi; the tables then take the funcfl path's regrid and
// splines unchanged.
void cacg_context::read_eam(const std::string &path, bool setfl, const std::string &element) {
  FILE *fp = fopen(path.c_str(), "r");
  if (!fp) fail(CACG_EIO, "Cannot open EAM potential file %s", path.c_str());
  char buf[4096];
  int tmp, nrho_f = 0, nr_f = 0;
  double mass = 0, drho_f = 0, dr_f = 0, cut = 0;
  auto line = [&]() {
    if (!fgets(buf, sizeof(buf), fp)) {
      fclose(fp);
      fail(CACG_EIO, "EAM file truncated");
    }
  };
  int nel = 1, iel = 0;
  if (setfl) {
    line();
    line();
    line();
    line();
    std::vector<std::string> w = split_words(buf);
    if (w.empty()) {
      fclose(fp);
      fail(CACG_EIO, "Invalid setfl element line");
    }
    nel = atoi(w[0].c_str());
    if (nel < 1 || (int) w.size() < nel + 1) {
      fclose(fp);
      fail(CACG_EIO, "Invalid setfl element line");
    }
    iel = -1;
    for (int k = 0; k < nel; k++)
      if (w[1 + k] == element) iel = k;
    if (iel < 0) {
      fclose(fp);
      fail(CACG_EINVAL, "No matching element %s in setfl file", element.c_str());
    }
    line();
    sscanf(buf, "%d %lg %d %lg %lg", &nrho_f, &drho_f, &nr_f, &dr_f, &cut);
  } else {
    line();
    line();
    sscanf(buf, "%d %lg", &tmp, &mass);
    line();
    sscanf(buf, "%d %lg %d %lg %lg", &nrho_f, &drho_f, &nr_f, &dr_f, &cut);
  }
  if (nrho_f < 5 || nr_f < 5) {
    fclose(fp);
    fail(CACG_EINVAL, "EAM tables too short");
  }
  auto grab = [&](int n, std::vector<double> &v) {
    v.assign((size_t) n + 1, 0.0);
    int i = 0;
    while (i < n) {
      if (!fgets(buf, sizeof(buf), fp)) return false;
      char *p = strtok(buf, " \t\n\r\f");
      if (!p) continue;
      v[1 + i++] = atof(p);
      while ((p = strtok(nullptr, " \t\n\r\f")) && i < n) v[1 + i++] = atof(p);
    }
    return true;
  };
  std::vector<double> F, R, Z;
  bool ok = true;
  if (setfl) {
    std::vector<double> f2, r2;
    for (int k = 0; k < nel && ok; k++) {
      if (!fgets(buf, sizeof(buf), fp)) {
        ok = false;
        break;
      }
      double zz = 0, mk = 0;
      sscanf(buf, "%lg %lg", &zz, &mk);
      ok = grab(nrho_f, f2) && grab(nr_f, r2);
      if (k == iel) {
        mass = mk;
        F = f2;
        R = r2;
      }
    }
    // pair tables in the order (i, j), i >= j
    for (int i = 0; i < nel && ok; i++)
      for (int j = 0; j <= i && ok; j++) {
        ok = grab(nr_f, r2);
        if (i == iel && j == iel) Z = r2;
      }
  } else {
    ok = grab(nrho_f, F) && grab(nr_f, R) && grab(nr_f, Z);
  }
  fclose(fp);
  if (!ok) fail(CACG_EIO, "EAM file truncated");
  eam_mass = mass;
  eam_cut = cut;
  dr = dr_f;
  drho = drho_f;
  double rmax = (nr_f - 1) * dr_f, rhomax = (nrho_f - 1) * drho_f;
  nr = (int) (rmax / dr + 0.5);
  nrho = (int) (rhomax / drho + 0.5);
  const double sixth = 1.0 / 6.0;
  auto regrid = [&](int n, double delta, int nfile, double dfile, const std::vector<double> &src) {
    std::vector<double> dst((size_t) n + 1, 0.0);
    for (int m = 1; m <= n; m++) {
      double r = (m - 1) * delta;
      double p = r / dfile + 1.0;
      int k = (int) p;
      k = std::min(k, nfile - 2);
      k = std::max(k, 2);
      p -= k;
      p = std::min(p, 2.0);
      double cof1 = -sixth * p * (p - 1.0) * (p - 2.0);
      double cof2 = 0.5 * (p * p - 1.0) * (p - 2.0);
      double cof3 = -0.5 * p * (p + 1.0) * (p - 2.0);
      double cof4 = sixth * p * (p * p - 1.0);
      dst[m] = cof1 * src[k - 1] + cof2 * src[k] + cof3 * src[k + 1] + cof4 * src[k + 2];
    }
    return dst;
  };
  auto interpolate = [](int n, double delta, const std::vector<double> &f) {
    std::vector<double> sp((size_t) (n + 1) * 7, 0.0);
    auto S = [&](int m, int k) -> double & { return sp[(size_t) m * 7 + k]; };
    for (int m = 1; m <= n; m++) S(m, 6) = f[m];
    S(1, 5) = S(2, 6) - S(1, 6);
    S(2, 5) = 0.5 * (S(3, 6) - S(1, 6));
    S(n - 1, 5) = 0.5 * (S(n, 6) - S(n - 2, 6));
    S(n, 5) = S(n, 6) - S(n - 1, 6);
    for (int m = 3; m <= n - 2; m++)
      S(m, 5) = ((S(m - 2, 6) - S(m + 2, 6)) + 8.0 * (S(m + 1, 6) - S(m - 1, 6))) / 12.0;
    for (int m = 1; m <= n - 1; m++) {
      S(m, 4) = 3.0 * (S(m + 1, 6) - S(m, 6)) - 2.0 * S(m, 5) - S(m + 1, 5);
      S(m, 3) = S(m, 5) + S(m + 1, 5) - 2.0 * (S(m + 1, 6) - S(m, 6));
    }
    S(n, 4) = 0.0;
    S(n, 3) = 0.0;
    for (int m = 1; m <= n; m++) {
      S(m, 2) = S(m, 5) / delta;
      S(m, 1) = 2.0 * S(m, 4) / delta;
      S(m, 0) = 3.0 * S(m, 3) / delta;
    }
    return sp;
  };
  auto frho = regrid(nrho, drho, nrho_f, drho_f, F);
  auto rhor = regrid(nr, dr, nr_f, dr_f, R);
  auto z2r = regrid(nr, dr, nr_f, dr_f, Z);
  rdr = 1.0 / dr;
  rdrho = 1.0 / drho;
  frho_sp = interpolate(nrho, drho, frho);
  rhor_sp = interpolate(nr, dr, rhor);
  z2r_sp = interpolate(nr, dr, z2r);
  cutforcesq = cut * cut;
}

// ------------------------------------------------------------------ init

// Element tables: inter_ele/shape_array_inter_ele (element.cpp:1361-1423),
// intp_pcoord/shape_array_int (1170-1191, 1326-1354), sub-elements (725-906),
// find_node_list (1296-1319).
void cacg_context::element_tables() {
  int_off.assign(MAXT + 1, 0);
  inter_off.assign(MAXT + 1, 0);
  inter_num.assign(MAXT + 1, 0);
  numint_v.assign(MAXT + 1, 0);
  node_list.assign((MAXT + 1) * NPE, 0);
  spa_int.clear();
  w_all.clear();
  spa_inter.clear();
  int ioff = 0, roff = 0;
  std::vector<std::vector<double>> pcs(MAXT + 1);
  for (int t = 1; t <= netypes; t++) {
    int nx = nae[t][0], ny = nae[t][1], nz = nae[t][2];
    inter_num[t] = nx * ny * nz;
    inter_off[t] = roff;
    double inx = 2 / ((double) nx - 1), iny = 2 / ((double) ny - 1), inz = 2 / ((double) nz - 1);
    double N[8];
    for (int ii = 0; ii < nx; ii++)
      for (int jj = 0; jj < ny; jj++)
        for (int kk = 0; kk < nz; kk++) {
          double px = inx * (double) ii - 1, py = iny * (double) jj - 1, pz = inz * (double) kk - 1;
          pcs[t].push_back(px);
          pcs[t].push_back(py);
          pcs[t].push_back(pz);
          shape8(px, py, pz, N);
          spa_inter.insert(spa_inter.end(), N, N + 8);
        }
    roff += inter_num[t];
    numint_v[t] = numint[t];
    int_off[t] = ioff;
    double dx = 2 / ((double) nx - 1), dy = 2 / ((double) ny - 1), dz = 2 / ((double) nz - 1);
    for (int m = 0; m < numint[t]; m++) {
      double px = dx * ((double) intp[t][3 * m]) - 1;
      double py = dy * ((double) intp[t][3 * m + 1]) - 1;
      double pz = dz * ((double) intp[t][3 * m + 2]) - 1;
      shape8(px, py, pz, N);
      spa_int.insert(spa_int.end(), N, N + 8);
      w_all.push_back(weight[t][m]);
    }
    ioff += numint[t];
    if (pair_style == 2) {
      for (int q = 0; q < NPE; q++) {
        int kk;
        for (kk = 0; kk < numint[t]; kk++)
          if (std::fabs(spa_int[(size_t) (int_off[t] + kk) * NPE + q] - 1.0) < 0.01) {
            node_list[t * NPE + q] = kk;
            break;
          }
        if (kk == numint[t]) fail(CACG_EINVAL, "didn't contain all node integration point");
      }
    }
  }
  // sub-elements: type-1 geometry (element.cpp:786-787, 835-836)
  int ns = nsplit;
  nsub = ns * ns * ns;
  double ls = 2.0 / ns;
  std::vector<double> pc((size_t) nsub * NPE * 3);
  auto PC = [&](int i, int l, int d) -> double & { return pc[((size_t) i * NPE + l) * 3 + d]; };
  const double c0[8][3] = {{-1.0, -1.0, -1.0}, {ls - 1.0, -1.0, -1.0}, {ls - 1.0, ls - 1.0, -1.0},
                           {-1.0, ls - 1.0, -1.0}, {-1.0, -1.0, ls - 1.0}, {ls - 1.0, -1.0, ls - 1.0},
                           {ls - 1.0, ls - 1.0, ls - 1.0}, {-1.0, ls - 1.0, ls - 1.0}};
  for (int l = 0; l < NPE; l++)
    for (int d = 0; d < 3; d++) PC(0, l, d) = c0[l][d];
  int in = 0;
  for (int ii = 0; ii < ns; ii++)
    for (int jj = 0; jj < ns; jj++)
      for (int kk = 0; kk < ns; kk++) {
        if (ii == 0 && jj == 0 && kk == 0) continue;
        in++;
        for (int l = 0; l < NPE; l++) {
          PC(in, l, 0) = PC(0, l, 0) + ii * ls;
          PC(in, l, 1) = PC(0, l, 1) + jj * ls;
          PC(in, l, 2) = PC(0, l, 2) + kk * ls;
        }
      }
  spa_csub.assign((size_t) nsub * NPE, 0.0);
  sub_first.assign((size_t) nsub + 1, 0);
  list_isub.clear();
  spa_isub.clear();
  const std::vector<double> &pinter = pcs[1];
  int ninter = inter_num[1];
  for (int i = 0; i < nsub; i++) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int l = 0; l < NPE; l++)
      for (int d = 0; d < 3; d++) c[d] += PC(i, l, d);
    for (int d = 0; d < 3; d++) c[d] = c[d] / NPE;
    shape8(c[0], c[1], c[2], &spa_csub[(size_t) i * NPE]);
    double blo[3] = {PC(i, 0, 0), PC(i, 0, 1), PC(i, 0, 2)};
    double bhi[3] = {PC(i, 1, 0), PC(i, 3, 1), PC(i, 4, 2)};
    for (int d = 0; d < 3; d++) {
      if (blo[d] < -0.99) blo[d] = -1.01;
      if (bhi[d] > 0.99) bhi[d] = 1.01;
    }
    sub_first[i] = (int) list_isub.size();
    double N[8];
    for (int j = 0; j < ninter; j++) {
      const double *p = &pinter[3 * (size_t) j];
      if (p[0] > blo[0] && p[0] <= bhi[0] && p[1] > blo[1] && p[1] <= bhi[1] && p[2] > blo[2] &&
          p[2] <= bhi[2]) {
        shape8(p[0], p[1], p[2], N);
        spa_isub.insert(spa_isub.end(), N, N + 8);
        list_isub.push_back(j);
      }
    }
  }
  sub_first[nsub] = (int) list_isub.size();
  if ((int) list_isub.size() != ninter)
    fail(CACG_EINVAL, "sub atom total donot match total atom number");
  cudaStream_t s = stream;
  upload(d_spa_int, spa_int, s);
  upload(d_weight, w_all, s);
  upload(d_spa_inter, spa_inter, s);
  upload(d_spa_csub, spa_csub, s);
  upload(d_spa_isub, spa_isub, s);
  upload(d_int_off, int_off, s);
  upload(d_inter_off, inter_off, s);
  upload(d_numint, numint_v, s);
  upload(d_inter_num, inter_num, s);
  upload(d_node_list, node_list, s);
  upload(d_list_isub, list_isub, s);
  upload(d_sub_first, sub_first, s);
  // lattice sizes per type for the mixed site kernels
  std::vector<int> nae3(3 * (MAXT + 1), 2);
  maxlines = max_nax = max_naz = 0;
  for (int t = 1; t <= netypes; t++) {
    for (int d = 0; d < 3; d++) nae3[3 * t + d] = nae[t][d];
    maxlines = std::max(maxlines, nae[t][0] * nae[t][1]);
    max_nax = std::max(max_nax, nae[t][0]);
    max_naz = std::max(max_naz, nae[t][2]);
  }
  upload(d_nae, nae3, s);
  // per type 1 / (n_a - 1), 1 / (n_b - 1), 1 / (n_c - 1), 1 / n_b for the fused
  // element passes (FP32 division, correctly rounded, as the kernels would do it)
  std::vector<float4> rec(MAXT + 1, make_float4(0.f, 0.f, 0.f, 0.f));
  for (int t = 0; t <= MAXT; t++) {
    const int na = nae3[3 * t], nb = nae3[3 * t + 1], nc = nae3[3 * t + 2];
    rec[t] = make_float4(na > 1 ? 1.0f / (float) (na - 1) : 0.f, nb > 1 ? 1.0f / (float) (nb - 1) : 0.f,
                         nc > 1 ? 1.0f / (float) (nc - 1) : 0.f, 1.0f / (float) nb);
  }
  upload(d_lat_rec, rec, s);
  // the fractions k / (n - 1) of each lattice axis as double-single floats
  fstride = 1;
  for (int t = 1; t <= netypes; t++)
    for (int d = 0; d < 3; d++) fstride = std::max(fstride, nae[t][d]);
  std::vector<float2> frac((size_t) (MAXT + 1) * 3 * fstride, make_float2(0.f, 0.f));
  for (int t = 1; t <= netypes; t++)
    for (int d = 0; d < 3; d++)
      for (int k = 0; k < nae[t][d]; k++) {
        const double v = nae[t][d] > 1 ? (double) k / (double) (nae[t][d] - 1) : 0.0;
        const float h = (float) v;
        frac[(size_t) (t * 3 + d) * fstride + k] = make_float2(h, (float) (v - (double) h));
      }
  upload(d_frac, frac, s);
  // weight x shape function of every row and node, FP32 (the mixed nodal gather)
  std::vector<float> wn(spa_int.size());
  for (size_t r = 0; r < w_all.size(); r++)
    for (int q = 0; q < NPE; q++) wn[r * NPE + q] = (float) (w_all[r] * spa_int[r * NPE + q]);
  upload(d_wn, wn, s);
  // per type, the rows of nonzero weight in ascending order (the fused passes)
  std::vector<int> fjj, fjj_off(MAXT + 2, 0);
  fused_types_ok = true;
  for (int t = 0; t <= MAXT; t++) {
    fjj_off[t] = (int) fjj.size();
    if (t < 1 || t > netypes) continue;
    int nf = 0;
    for (int jj = 0; jj < numint[t]; jj++)
      if (w_all[int_off[t] + jj] != 0.0) {
        fjj.push_back(jj);
        nf++;
      }
    if (nf > 32) fused_types_ok = false;
  }
  fjj_off[MAXT + 1] = (int) fjj.size();
  // their weight x shape function products in the same order (the fused
  // nodal gather reads them without the row indirection)
  std::vector<float> wnf(std::max<size_t>(fjj.size(), 1) * NPE, 0.f);
  for (int t = 1; t <= netypes; t++)
    for (int j = fjj_off[t]; j < fjj_off[t + 1]; j++)
      for (int q = 0; q < NPE; q++) wnf[(size_t) j * NPE + q] = wn[((size_t) int_off[t] + fjj[j]) * NPE + q];
  upload(d_wnf, wnf, s);
  if (fjj.empty()) fjj.push_back(0);
  upload(d_fjj, fjj, s);
  upload(d_fjj_off, fjj_off, s);
  std::vector<int4> ip4;
  for (int t = 1; t <= netypes; t++)
    for (int m = 0; m < numint[t]; m++)
      ip4.push_back(make_int4(intp[t][3 * m], intp[t][3 * m + 1], intp[t][3 * m + 2], 0));
  if (ip4.empty()) ip4.push_back(make_int4(0, 0, 0, 0));
  upload(d_intp4, ip4, s);
  std::vector<float2> sihl(spa_int.size());
  for (size_t k = 0; k < spa_int.size(); k++)
    sihl[k] = make_float2((float) spa_int[k], (float) (spa_int[k] - (double) (float) spa_int[k]));
  upload(d_spa_int_hl, sihl, s);
}

// FP32 copies of the tables the mixed-precision kernels read from shared memory
void cacg_context::mixed_tables() {
  const int T = (MAXT + 1) * (MAXT + 1);
  if (pair_style == 1) {
    std::vector<float> lf(3 * T, 0.f);
    std::vector<double> c64(T, 0.0);
    for (int k = 0; k < T; k++) {
      lf[k] = (float) ljtab.lj1[k];
      lf[T + k] = (float) ljtab.lj2[k];
      lf[2 * T + k] = (float) ljtab.cutsq[k];
      c64[k] = ljtab.cutsq[k];
    }
    upload(d_ljf, lf, stream);
    upload(d_cutsq64, c64, stream);
  } else if (pair_style == 2) {
    std::vector<float4> val(nr + 1), ft(mixed::FTAB_W * (size_t) (nr + 1));
    for (int m = 0; m <= nr; m++) {
      const double *c = &rhor_sp[(size_t) m * 7];
      const double *z = &z2r_sp[(size_t) m * 7];
      val[m] = make_float4((float) c[3], (float) c[4], (float) c[5], (float) c[6]);
      ft[2 * m] = make_float4((float) c[0], (float) c[1], (float) c[2], (float) z[3]);
      ft[2 * m + 1] = make_float4((float) z[4], (float) z[5], (float) z[6], 0.f);
    }
    std::vector<float4> f4(nrho + 1);
    std::vector<float2> fds(3 * (size_t) (nrho + 1));
    for (int m = 0; m <= nrho; m++) {
      const double *c = &frho_sp[(size_t) m * 7];
      f4[m] = make_float4((float) c[0], (float) c[1], (float) c[2], 0.f);
      for (int k = 0; k < 3; k++) {  // the F' coefficients as double-single pairs
        const float h = (float) c[k];
        fds[3 * (size_t) m + k] = make_float2(h, (float) (c[k] - (double) h));
      }
    }
    upload(d_frho_ds, fds, stream);
    upload(d_rhor_val4, val, stream);
    upload(d_ftab, ft, stream);
    upload(d_fp4, f4, stream);
  }
}

// Element::element_size (element.cpp:567-625): running maximum of the body
// diagonals over local elements, per type the value reached at its last
// element, max_size never decreases.
void cacg_context::element_size() {
  if (enlocal == 0) return;
  d_diag.ensure(enlocal, stream);
  d_misc.ensure(32, stream);
  check(cudaMemsetAsync(d_misc.p + 8, 0, sizeof(int), stream), "memset");
  launch_elem_diag(d_nodex.p, d_ex.p, enlocal, d_diag.p, d_misc.p + 8, stream);
  launches++;
  std::vector<double> diag(enlocal);
  check(cudaMemcpyAsync(diag.data(), d_diag.p, sizeof(double) * enlocal, cudaMemcpyDeviceToHost, stream), "diag");
  check(cudaMemcpyAsync(h_pin + 8, d_misc.p + 8, sizeof(int), cudaMemcpyDeviceToHost, stream), "bad");
  std::vector<int> et(enlocal);
  check(cudaMemcpyAsync(et.data(), d_etype.p, sizeof(int) * enlocal, cudaMemcpyDeviceToHost, stream), "etype");
  sync();
  double mx[MAXT + 1] = {};
  double length = 0.0;
  for (int i = 0; i < enlocal; i++) {
    length = std::max(length, diag[i]);
    mx[et[i]] = length;
  }
  for (int t = 1; t <= netypes; t++) {
    esize[t] = mx[t];
    max_size = std::max(max_size, esize[t]);
  }
  if (h_pin[8]) fail(CACG_EINVAL, "element data has error");
}

void cacg_context::setup_cut() {
  // Neighbor::setup_cut, neighbor.cpp:284-293
  cut_all = cutneighmax + max_size;
  cut_allsq = cut_all * cut_all;
  cut_ele = cutneighmax + max_size / 2;
  cut_elesq = cut_ele * cut_ele;
  cut_subele = cutneighmax + max_size / (2 * nsplit);
  cut_subelesq = cut_subele * cut_subele;
}

// CommBrick::setup for one sub-domain spanning the box (comm_brick.cpp:182-367)
void cacg_context::comm_setup() {
  double cut = cutneighmax;
  for (int d = 0; d < 3; d++) cutghost[d] = cut_all;
  for (int t = 1; t <= netypes; t++) cutghostmulti[t] = cut + esize[t];
  int maxneed[3];
  for (int d = 0; d < 3; d++) {
    maxneed[d] = (int) (cutghost[d] * 1 / prd[d]) + 1;
    if (!periodic[d]) maxneed[d] = std::min(maxneed[d], 0);
  }
  swaps.clear();
  for (int dim = 0; dim < 3; dim++)
    for (int ineed = 0; ineed < 2 * maxneed[dim]; ineed++) {
      SwapDef w;
      w.dim = dim;
      double sublo = lo[dim], subhi = hi[dim];
      if (ineed % 2 == 0) {
        w.lo = ineed < 2 ? -1.0e20 : 0.5 * (sublo + subhi);
        w.hi = sublo + cutghost[dim];
        for (int t = 1; t <= netypes; t++) {
          w.mlo[t] = ineed < 2 ? -1.0e20 : 0.5 * (sublo + subhi);
          w.mhi[t] = sublo + cutghostmulti[t];
        }
        w.pbc = 1;
      } else {
        w.lo = subhi - cutghost[dim];
        w.hi = ineed < 2 ? 1.0e20 : 0.5 * (sublo + subhi);
        for (int t = 1; t <= netypes; t++) {
          w.mlo[t] = subhi - cutghostmulti[t];
          w.mhi[t] = ineed < 2 ? 1.0e20 : 0.5 * (sublo + subhi);
        }
        w.pbc = -1;
      }
      // AtomVecAtomic::pack_border / pack_comm: dx = pbc[d]*prd[d]
      for (int d = 0; d < 3; d++) w.d[d] = (d == dim ? w.pbc : 0) * prd[d];
      swaps.push_back(w);
    }
}

// Neighbor::setup_bins + stencil_half_bin_3d_no_newton (neighbor.cpp:768-976)
void cacg_context::setup_bins() {
  double bsublo[3], bsubhi[3], bbox[3];
  for (int d = 0; d < 3; d++) {
    bsublo[d] = lo[d] - cutghost[d] - max_size / 2.0;
    bsubhi[d] = hi[d] + cutghost[d] + max_size / 2.0;
    bbox[d] = hi[d] - lo[d];
  }
  double binsize_optimal = binsize_user > 0.0 ? binsize_user : 0.5 * cutneighmax;
  if (binsize_optimal == 0.0) binsize_optimal = bbox[0];
  double binsizeinv = 1.0 / binsize_optimal;
  for (int d = 0; d < 3; d++)
    if (bbox[d] * binsizeinv > 2147483647.0) fail(CACG_EINVAL, "Domain too large for neighbor bins");
  double binsize[3];
  for (int d = 0; d < 3; d++) {
    bins.nbin[d] = (int) (bbox[d] * binsizeinv);
    if (bins.nbin[d] == 0) bins.nbin[d] = 1;
    binsize[d] = bbox[d] / bins.nbin[d];
    bins.bininv[d] = 1.0 / binsize[d];
    bins.lo[d] = lo[d];
    bins.hi[d] = hi[d];
  }
  for (int d = 0; d < 3; d++)
    if (binsize_optimal * bins.bininv[d] > 100)
      fail(CACG_EINVAL, "Cannot use neighbor bins - box size << cutoff");
  for (int d = 0; d < 3; d++) {
    double coord = bsublo[d] - 1.0e-6 * bbox[d];
    int mlo_ = (int) ((coord - lo[d]) * bins.bininv[d]);
    if (coord < lo[d]) mlo_ = mlo_ - 1;
    coord = bsubhi[d] + 1.0e-6 * bbox[d];
    int mhi_ = (int) ((coord - lo[d]) * bins.bininv[d]);
    mlo_ -= 1;
    mhi_ += 1;
    bins.mlo[d] = mlo_;
    bins.mbin[d] = mhi_ - mlo_ + 1;
  }
  long long bb = (long long) bins.mbin[0] * bins.mbin[1] * bins.mbin[2];
  if (bb > 2147483647LL) fail(CACG_EINVAL, "Too many neighbor bins");
  bins.mbins = (int) bb;
  int sx = (int) (cutneighmax * bins.bininv[0]);
  if (sx * binsize[0] < cutneighmax) sx++;
  int sy = (int) (cutneighmax * bins.bininv[1]);
  if (sy * binsize[1] < cutneighmax) sy++;
  int sz = (int) (cutneighmax * bins.bininv[2]);
  if (sz * binsize[2] < cutneighmax) sz++;
  auto bin_distance = [&](int i, int j, int k) {
    double dx, dy, dz;
    if (i > 0) dx = (i - 1) * binsize[0];
    else if (i == 0) dx = 0.0;
    else dx = (i + 1) * binsize[0];
    if (j > 0) dy = (j - 1) * binsize[1];
    else if (j == 0) dy = 0.0;
    else dy = (j + 1) * binsize[1];
    if (k > 0) dz = (k - 1) * binsize[2];
    else if (k == 0) dz = 0.0;
    else dz = (k + 1) * binsize[2];
    return dx * dx + dy * dy + dz * dz;
  };
  stencil.clear();
  for (int k = -sz; k <= sz; k++)
    for (int j = -sy; j <= sy; j++)
      for (int i = -sx; i <= sx; i++)
        if (bin_distance(i, j, k) < cutneighmaxsq)
          stencil.push_back(k * bins.mbin[1] * bins.mbin[0] + j * bins.mbin[0] + i);
  upload(d_stencil, stencil, stream);
}

void cacg_context::init() {
  if (!box_set) fail(CACG_ESTATE, "Init before the box is defined (read_data or cacg_set_box)");
  ran = false;
  if (pair_style == 0) fail(CACG_ESTATE, "No pair style defined");
  int nt = std::max(ntypes, 1);
  for (int i = 1; i <= nt; i++)
    if (!setflag[i][i]) fail(CACG_EINVAL, "All pair coeffs are not set");
  if (netypes > 1 && enlocal > 0)
    fail(CACG_EINVAL, "Element forces use type-1 tables only (pair_lj_cut.cpp:327-331); one element type");
  for (int i = 1; i <= nt; i++)
    if (amass[i] <= 0.0) fail(CACG_EINVAL, "Not all atom masses are set");
  if (!h_pin) check(cudaMallocHost(&h_pin, 64 * sizeof(int)), "pinned");

  // Neighbor::init cutoffs (neighbor.cpp:335-374): per-type cutoff is 0, so the
  // list cutoff is the neighbor command's value
  cutneighmax = skin;
  cutneighmaxsq = cutneighmax * cutneighmax;
  triggersq = 0.25 * skin * skin;

  // Pair::init -> init_one (pair.cpp:102-155, pair_lj_cut.cpp:140-198)
  if (pair_style == 1 && lj_raw) {
    // tables as the caller's PairLJCut::init_one made them; lj3 = lj1 / 12
    // and lj4 = lj2 / 6 (4 eps sigma^12 and 4 eps sigma^6) for the energies
    memset(&ljtab, 0, sizeof(ljtab));
    const int T = (MAXT + 1) * (MAXT + 1);
    std::vector<double> lj5(5 * T, 0.0);
    for (int i = 1; i <= nt; i++)
      for (int j = 1; j <= nt; j++) {
        const int a = i * (MAXT + 1) + j, r = i * (nt + 1) + j;
        ljtab.lj1[a] = raw_lj1[r];
        ljtab.lj2[a] = raw_lj2[r];
        ljtab.cutsq[a] = raw_cutsq[r];
        lj5[a] = raw_lj1[r];
        lj5[T + a] = raw_lj2[r];
        lj5[2 * T + a] = raw_lj1[r] / 12.0;
        lj5[3 * T + a] = raw_lj2[r] / 6.0;
        lj5[4 * T + a] = raw_cutsq[r];
      }
    d_ljtab.ensure(1, stream);
    check(cudaMemcpyAsync(d_ljtab.p, &ljtab, sizeof(ljtab), cudaMemcpyHostToDevice, stream), "ljtab");
    upload(d_lj5, lj5, stream);
    h_lj5 = lj5;
  } else if (pair_style == 1) {
    memset(&ljtab, 0, sizeof(ljtab));
    for (int i = 1; i <= nt; i++)
      for (int j = i; j <= nt; j++) {
        double e = eps[i][j], s = sig[i][j], c = cutp[i][j];
        if (!setflag[i][j]) {
          e = std::sqrt(eps[i][i] * eps[j][j]);  // geometric mixing (pair.cpp:174-199)
          s = std::sqrt(sig[i][i] * sig[j][j]);
          c = std::sqrt(cutp[i][i] * cutp[j][j]);
        }
        double l1 = 48.0 * e * std::pow(s, 12.0), l2 = 24.0 * e * std::pow(s, 6.0);
        int a = i * (MAXT + 1) + j, b = j * (MAXT + 1) + i;
        ljtab.lj1[a] = ljtab.lj1[b] = l1;
        ljtab.lj2[a] = ljtab.lj2[b] = l2;
        ljtab.cutsq[a] = ljtab.cutsq[b] = c * c;
      }
    d_ljtab.ensure(1, stream);
    check(cudaMemcpyAsync(d_ljtab.p, &ljtab, sizeof(ljtab), cudaMemcpyHostToDevice, stream), "ljtab");
    // energy coefficients lj3 = 4 eps sigma^12, lj4 = 4 eps sigma^6 (pair_lj_cut.cpp:151-152)
    const int T = (MAXT + 1) * (MAXT + 1);
    std::vector<double> lj5(5 * T, 0.0);
    for (int i = 1; i <= nt; i++)
      for (int j = 1; j <= nt; j++) {
        double e = eps[std::min(i, j)][std::max(i, j)], sg = sig[std::min(i, j)][std::max(i, j)];
        if (!setflag[std::min(i, j)][std::max(i, j)]) {
          e = std::sqrt(eps[i][i] * eps[j][j]);
          sg = std::sqrt(sig[i][i] * sig[j][j]);
        }
        int k = i * (MAXT + 1) + j;
        lj5[k] = ljtab.lj1[k];
        lj5[T + k] = ljtab.lj2[k];
        lj5[2 * T + k] = 4.0 * e * std::pow(sg, 12.0);
        lj5[3 * T + k] = 4.0 * e * std::pow(sg, 6.0);
        lj5[4 * T + k] = ljtab.cutsq[k];
      }
    upload(d_lj5, lj5, stream);
    h_lj5 = lj5;
  } else {
    upload(d_frho, frho_sp, stream);
    upload(d_rhor, rhor_sp, stream);
    upload(d_z2r, z2r_sp, stream);
  }
  mixed_tables();
  // element masses: NAAE gives nae^3 * m(type 1) (element.cpp:1104) and
  // pair_coeff eam resets it from the potential file (element.cpp:1117-1123)
  for (int t = 1; t <= netypes; t++)
    emass[t] = nae[t][0] * nae[t][1] * nae[t][2] * (pair_style == 2 ? eam_mass : amass[1]);

  // upload per-particle state (owned particles only; ghosts come from borders)
  cudaStream_t s = stream;
  int na = std::max(nlocal, 1);
  d_x.ensure(na, s);
  d_v.ensure(3 * (size_t) na, s);
  d_f.ensure(3 * (size_t) na, s);
  d_xhold.ensure(3 * (size_t) na, s);
  d_type.ensure(na, s);
  d_tag.ensure(na, s);
  d_root.ensure(na, s);
  if (nlocal) {
    std::vector<double4> x4(nlocal);
    for (int i = 0; i < nlocal; i++) x4[i] = make_double4(h_x[3 * i], h_x[3 * i + 1], h_x[3 * i + 2], 0.0);
    std::vector<int> root(nlocal);
    for (int i = 0; i < nlocal; i++) root[i] = i;
    check(cudaMemcpyAsync(d_x.p, x4.data(), sizeof(double4) * nlocal, cudaMemcpyHostToDevice, s), "x");
    check(cudaMemcpyAsync(d_v.p, h_v.data(), sizeof(double) * 3 * nlocal, cudaMemcpyHostToDevice, s), "v");
    check(cudaMemsetAsync(d_f.p, 0, sizeof(double) * 3 * nlocal, s), "f");
    check(cudaMemcpyAsync(d_type.p, h_type.data(), sizeof(int) * nlocal, cudaMemcpyHostToDevice, s), "type");
    check(cudaMemcpyAsync(d_tag.p, h_tag.data(), sizeof(int) * nlocal, cudaMemcpyHostToDevice, s), "tag");
    check(cudaMemcpyAsync(d_root.p, root.data(), sizeof(int) * nlocal, cudaMemcpyHostToDevice, s), "root");
  }
  std::vector<double> massv(MAXT + 1, 0.0), emassv(MAXT + 1, 0.0);
  for (int t = 0; t <= MAXT; t++) {
    massv[t] = amass[t];
    emassv[t] = emass[t];
  }
  upload(d_mass, massv, s);
  upload(d_emass, emassv, s);
  for (int t = 0; t <= MAXT; t++) {
    up_mass[t] = massv[t];
    up_emass[t] = emassv[t];
  }
  nghost = 0;
  int ne = std::max(enlocal, 1);
  d_ex.ensure(3 * (size_t) ne, s);
  d_nodex.ensure(24 * (size_t) ne, s);
  d_nodev.ensure(24 * (size_t) ne, s);
  d_nodef.ensure(24 * (size_t) ne, s);
  d_nodexhold.ensure(24 * (size_t) ne, s);
  d_etype.ensure(ne, s);
  d_etag.ensure(ne, s);
  d_eroot.ensure(ne, s);
  if (enlocal) {
    std::vector<int> root(enlocal);
    for (int i = 0; i < enlocal; i++) root[i] = i;
    check(cudaMemcpyAsync(d_ex.p, h_ex.data(), sizeof(double) * 3 * enlocal, cudaMemcpyHostToDevice, s), "ex");
    check(cudaMemcpyAsync(d_nodex.p, h_nodex.data(), sizeof(double) * 24 * enlocal, cudaMemcpyHostToDevice, s), "nodex");
    check(cudaMemcpyAsync(d_nodev.p, h_nodev.data(), sizeof(double) * 24 * enlocal, cudaMemcpyHostToDevice, s), "nodev");
    check(cudaMemsetAsync(d_nodef.p, 0, sizeof(double) * 24 * enlocal, s), "nodef");
    check(cudaMemcpyAsync(d_etype.p, h_etype.data(), sizeof(int) * enlocal, cudaMemcpyHostToDevice, s), "etype");
    check(cudaMemcpyAsync(d_etag.p, h_etag.data(), sizeof(int) * enlocal, cudaMemcpyHostToDevice, s), "etag");
    check(cudaMemcpyAsync(d_eroot.p, root.data(), sizeof(int) * enlocal, cudaMemcpyHostToDevice, s), "eroot");
    element_tables();
    // integration-point rows of the owned elements (NodeNeighList rows, node_neigh_list.h:23-27)
    h_row_first.assign(enlocal + 1, 0);
    std::vector<int> re, rj;
    for (int e = 0; e < enlocal; e++) {
      h_row_first[e] = (int) re.size();
      for (int jj = 0; jj < numint[h_etype[e]]; jj++) {
        re.push_back(e);
        rj.push_back(jj);
      }
    }
    h_row_first[enlocal] = (int) re.size();
    nrows = (int) re.size();
    upload(d_row_elem, re, s);
    upload(d_row_jj, rj, s);
    upload(d_row_first, h_row_first, s);
    // rows of nonzero weight: the only ones whose force reaches the nodes
    std::vector<int> fr;
    for (int r = 0; r < nrows; r++)
      if (weight[h_etype[re[r]]][rj[r]] != 0.0) fr.push_back(r);
    nforce = (int) fr.size();
    upload(d_force_rows, fr, s);
    std::vector<unsigned char> isf(std::max(nrows, 1), 0);
    for (int r : fr) isf[r] = 1;
    upload(d_row_isforce, isf, s);
    element_size();
  } else {
    nrows = 0;
  }
  enghost = 0;
  cut_all = cutneighmax + max_size;
  cut_ele = cutneighmax + max_size / 2;
  cut_allsq = cut_all * cut_all;
  cut_elesq = cut_ele * cut_ele;
  inited = true;
  setup_done = list_built = elists_built = false;
}

// ------------------------------------------------------------------ ghosts

// CommBrick::borders (comm_brick.cpp:641-914): atoms, then elements
void cacg_context::borders() {
  borders_atoms();
  borders_elems();
}

// ghost atoms, swap by swap (comm_brick.cpp:657-801)
void cacg_context::borders_atoms() {
  cudaStream_t s = stream;
  d_misc.ensure(32, s);
  nghost = 0;
  size_t send_total = 0;
  int nfirst = 0, nlast = 0;
  for (size_t iw = 0; iw < swaps.size(); iw++) {
    SwapDef &w = swaps[iw];
    if (iw == 0 || swaps[iw - 1].dim != w.dim) nlast = 0;
    if (w.pbc == 1) {
      nfirst = nlast;
      nlast = nlocal + nghost;
    }
    int n = nlast - nfirst;
    d_flags.ensure(std::max(n, 1), s);
    d_pos.ensure(std::max(n, 1), s);
    launch_border_flags_atoms(d_x.p, nfirst, nlast, w.dim, w.lo, w.hi, d_flags.p, s);
    scan_exclusive(d_flags.p, d_pos.p, n, d_misc.p, d_scan, s);
    launches += 2;
    check(cudaMemcpyAsync(h_pin, d_misc.p, sizeof(int), cudaMemcpyDeviceToHost, s), "count");
    sync();
    int cnt = n > 0 ? h_pin[0] : 0;
    int n0 = nlocal + nghost;
    d_x.ensure((size_t) n0 + cnt, s, true);
    d_type.ensure((size_t) n0 + cnt, s, true);
    d_tag.ensure((size_t) n0 + cnt, s, true);
    d_root.ensure((size_t) n0 + cnt, s, true);
    d_send.ensure(send_total + cnt + 1, s, true);
    launch_border_scatter_atoms(d_x.p, d_type.p, d_tag.p, d_root.p, d_send.p + send_total,
                                d_flags.p, d_pos.p, nfirst, nlast, n0, w.d[0], w.d[1], w.d[2], s);
    launches++;
    w.nsend = cnt;
    w.firstrecv = n0;
    w.send_off = (int) send_total;
    send_total += cnt;
    nghost += cnt;
  }
}

// ghost elements, swap by swap (comm_brick.cpp:804-905), and the per-element
// offsets of their interpolated sites
void cacg_context::borders_elems() {
  cudaStream_t s = stream;
  d_misc.ensure(32, s);
  enghost = 0;
  size_t send_total = 0;
  int nfirst = 0, nlast = 0;
  for (size_t iw = 0; iw < swaps.size(); iw++) {
    SwapDef &w = swaps[iw];
    if (iw == 0 || swaps[iw - 1].dim != w.dim) nlast = 0;
    if (w.pbc == 1) {
      nfirst = nlast;
      nlast = enlocal + enghost;
    }
    int n = nlast - nfirst;
    if (enlocal == 0) {
      w.ensend = 0;
      w.efirstrecv = enlocal + enghost;
      w.esend_off = 0;
      continue;
    }
    d_flags.ensure(std::max(n, 1), s);
    d_pos.ensure(std::max(n, 1), s);
    launch_border_flags_elems(d_ex.p, d_etype.p, nfirst, nlast, w.dim, w.mlo, w.mhi, d_flags.p, s);
    scan_exclusive(d_flags.p, d_pos.p, n, d_misc.p, d_scan, s);
    launches += 2;
    check(cudaMemcpyAsync(h_pin, d_misc.p, sizeof(int), cudaMemcpyDeviceToHost, s), "count");
    sync();
    int cnt = n > 0 ? h_pin[0] : 0;
    int n0 = enlocal + enghost;
    d_ex.ensure(3 * ((size_t) n0 + cnt), s, true);
    d_nodex.ensure(24 * ((size_t) n0 + cnt), s, true);
    d_etype.ensure((size_t) n0 + cnt, s, true);
    d_etag.ensure((size_t) n0 + cnt, s, true);
    d_eroot.ensure((size_t) n0 + cnt, s, true);
    d_esend.ensure(send_total + cnt + 1, s, true);
    launch_border_scatter_elems(d_ex.p, d_nodex.p, d_etype.p, d_etag.p, d_eroot.p,
                                d_esend.p + send_total, d_flags.p, d_pos.p, nfirst, nlast, n0,
                                w.d[0], w.d[1], w.d[2], s);
    launches++;
    w.ensend = cnt;
    w.efirstrecv = n0;
    w.esend_off = (int) send_total;
    send_total += cnt;
    enghost += cnt;
  }
  // per-element site offsets (types of ghosts from their roots)
  int nall_e = enlocal + enghost;
  if (enlocal) {
    h_eroot.resize(nall_e);
    check(cudaMemcpyAsync(h_eroot.data(), d_eroot.p, sizeof(int) * nall_e, cudaMemcpyDeviceToHost, s), "eroot");
    sync();
    h_site_base.assign(nall_e + 1, 0);
    int acc = 0;
    for (int e = 0; e < nall_e; e++) {
      h_site_base[e] = acc;
      acc += inter_num[h_etype[h_eroot[e]]];
    }
    h_site_base[nall_e] = acc;
    nsites = acc;
    upload(d_site_base, h_site_base, s);
  } else {
    nsites = 0;
  }
}

// CommBrick::forward_comm / eforward_comm: ghost positions from their sources,
// swap by swap (comm_brick.cpp:1017-1112)
void cacg_context::forward_comm(int which) {
  if (!swaps.empty() && swaps.size() <= (size_t) MAX_SWAPS) {
    SwapChain ca{}, ce{};
    ca.n = ce.n = (int) swaps.size();
    for (size_t k = 0; k < swaps.size(); k++) {
      ca.first[k] = swaps[k].firstrecv;
      ce.first[k] = swaps[k].efirstrecv;
      for (int d = 0; d < 3; d++) ca.d[k][d] = ce.d[k][d] = swaps[k].d[d];
    }
    if ((which & 1) && nlocal && nghost) {
      launch_forward_atoms_all(d_x.p, d_send.p, nlocal, nghost, ca, stream);
      launches++;
    }
    if ((which & 2) && enlocal && enghost) {
      launch_forward_elems_all(d_nodex.p, d_esend.p, enlocal, enghost, ce, stream);
      launches++;
    }
    return;
  }
  for (auto &w : swaps) {
    if ((which & 1) && nlocal && w.nsend) {
      launch_forward_atoms(d_x.p, d_send.p + w.send_off, w.nsend, w.firstrecv, w.d[0], w.d[1], w.d[2], stream);
      launches++;
    }
    if ((which & 2) && enlocal && w.ensend) {
      launch_forward_elems(d_nodex.p, d_esend.p + w.esend_off, w.ensend, w.efirstrecv, w.d[0], w.d[1], w.d[2], stream);
      launches++;
    }
  }
}

void cacg_context::pbc() {
  launch_pbc_atoms(d_x.p, nlocal, lo, hi, prd, periodic, stream);
  launch_pbc_elems(d_ex.p, d_nodex.p, enlocal, lo, hi, prd, periodic, stream);
  launches += 2;
}

// ------------------------------------------------------------------ lists

void cacg_context::neighbor_build() {
  list_builds++;
  cudaStream_t s = stream;
  int nall = nlocal + nghost;
  if (nlocal == 0) {
    list_built = true;
    return;
  }
  d_misc.ensure(32, s);
  d_abin.ensure(nall, s);
  check(cudaMemsetAsync(d_misc.p + 1, 0, sizeof(int) * 2, s), "memset");
  launch_coord2bin_atoms(d_x.p, nall, bins, d_abin.p, d_misc.p + 1, s);
  build_bins(d_abin.p, nall, bins.mbins, d_bcount, d_bstart, d_bmem, d_scan, s);
  d_bx.ensure(nall, s);
  launch_gather_bin_x_atoms(d_bmem.p, d_x.p, d_bx.p, nall, s);
  launches += 7;
  stride = (nlocal + 31) / 32 * 32;
  d_num.ensure(nlocal, s);
  for (int attempt = 0; attempt < 3; attempt++) {
    d_list.ensure((size_t) maxneigh * stride, s);
    check(cudaMemsetAsync(d_misc.p + 2, 0, sizeof(int), s), "memset");
    launch_atom_list(d_x.p, d_abin.p, d_bstart.p, d_bmem.p, d_bx.p, d_stencil.p,
                     (int) stencil.size(), bins.mbins, nlocal, cutneighmaxsq, maxneigh, stride,
                     d_num.p, d_list.p, d_misc.p + 2, s);
    launches++;
    check(cudaMemcpyAsync(h_pin + 1, d_misc.p + 1, sizeof(int) * 2, cudaMemcpyDeviceToHost, s), "ovf");
    sync();
    if (h_pin[1]) fail(CACG_EINVAL, "%d atoms outside the bin grid (lost atoms)", h_pin[1]);
    if (h_pin[2] == 0) break;
    if (h_pin[2] > oneatom || attempt == 2)
      fail(CACG_EOVERFLOW, "Neighbor list overflow, boost neigh_modify one");
    maxneigh = (h_pin[2] + 8 + 7) / 8 * 8;
  }
  launch_hold_atoms(d_x.p, d_xhold.p, nlocal, s);
  launches++;
  list_built = true;
}

void cacg_context::neighbor_ebuild() {
  cudaStream_t s = stream;
  setup_cut();
  if (enlocal == 0) {
    elists_built = true;
    return;
  }
  int nall = enlocal + enghost;
  if (dist_check)
    check(cudaMemcpyAsync(d_nodexhold.p, d_nodex.p, sizeof(double) * 24 * enlocal, cudaMemcpyDeviceToDevice, s), "hold");
  d_ebin.ensure(nall, s);
  check(cudaMemsetAsync(d_misc.p + 3, 0, sizeof(int) * 2, s), "memset");
  launch_coord2bin_elems(d_ex.p, nall, bins, d_ebin.p, d_misc.p + 3, s);
  build_bins(d_ebin.p, nall, bins.mbins, d_ebcount, d_ebstart, d_ebmem, d_scan, s);
  d_ebx.ensure(nall, s);
  launch_gather_bin_x_elems(d_ebmem.p, d_ex.p, d_ebx.p, nall, s);
  launches += 7;
  estride = (enlocal + 31) / 32 * 32;
  d_enum.ensure(enlocal, s);
  for (int attempt = 0; attempt < 3; attempt++) {
    d_elist.ensure((size_t) maxeneigh * estride, s);
    check(cudaMemsetAsync(d_misc.p + 4, 0, sizeof(int), s), "memset");
    launch_elem_list(d_ex.p, d_ebin.p, d_ebstart.p, d_ebmem.p, d_ebx.p, d_stencil.p,
                     (int) stencil.size(), bins.mbins, enlocal, cut_allsq, maxeneigh, estride,
                     d_enum.p, d_elist.p, d_misc.p + 4, s);
    launches++;
    check(cudaMemcpyAsync(h_pin + 3, d_misc.p + 3, sizeof(int) * 2, cudaMemcpyDeviceToHost, s), "ovf");
    sync();
    if (h_pin[3]) fail(CACG_EINVAL, "%d elements outside the bin grid (lost elements)", h_pin[3]);
    if (h_pin[4] == 0) break;
    if (h_pin[4] > oneatom || attempt == 2)
      fail(CACG_EOVERFLOW, "Neighbor list overflow, boost neigh_modify one");
    maxeneigh = (h_pin[4] + 8 + 7) / 8 * 8;
  }
  elists_built = false;
}

void cacg_context::neighbor_nbuild() {
  cudaStream_t s = stream;
  if (enlocal == 0) {
    elists_built = true;
    return;
  }
  int nall = enlocal + enghost;
  ElemTables t = etab();
  d_site_x.ensure(std::max(nsites, 1), s);
  launch_sites(d_nodex.p, d_etype.p, d_site_base.p, nall, t, d_site_x.p, nullptr, s);
  d_subc.ensure((size_t) nall * nsub, s);
  launch_sub_centres(d_nodex.p, nall, t, d_subc.p, s);
  launches += 2;
  rowstride = (nrows + 31) / 32 * 32;
  d_ipnum.ensure(std::max(nrows, 1), s);
  for (int attempt = 0; attempt < 3; attempt++) {
    d_ipent.ensure((size_t) maxip * rowstride, s);
    check(cudaMemsetAsync(d_misc.p + 5, 0, sizeof(int), s), "memset");
    launch_ip_list(d_nodex.p, d_ex.p, d_etype.p, d_row_elem.p, d_row_jj.p, nrows, d_enum.p,
                   d_elist.p, estride, d_subc.p, d_site_x.p, d_site_base.p, t, cut_elesq,
                   cut_subelesq, cutneighmaxsq, maxip, rowstride, d_ipnum.p, d_ipent.p,
                   d_misc.p + 5, s);
    launches++;
    check(cudaMemcpyAsync(h_pin + 5, d_misc.p + 5, sizeof(int), cudaMemcpyDeviceToHost, s), "ovf");
    sync();
    if (h_pin[5] == 0) break;
    if (h_pin[5] > oneatom || attempt == 2)
      fail(CACG_EOVERFLOW, "Neighbor list overflow, boost neigh_modify one");
    maxip = (h_pin[5] + 8 + 7) / 8 * 8;
  }
  d_fip.ensure(3 * (size_t) std::max(nrows, 1), s);
  check(cudaMemsetAsync(d_fip.p, 0, sizeof(double) * 3 * std::max(nrows, 1), s), "fip");
  d_fipf.ensure(3 * (size_t) std::max(nrows, 1), s);
  check(cudaMemsetAsync(d_fipf.p, 0, sizeof(float2) * 3 * std::max(nrows, 1), s), "fipf");
  // the sites any list references: the per-step site kernels compute only these
  d_site_flag.ensure(std::max(nsites, 1), s);
  d_site_pos.ensure(std::max(nsites, 1), s);
  check(cudaMemsetAsync(d_site_flag.p, 0, sizeof(int) * std::max(nsites, 1), s), "flag");
  fp64_fma::mark_sites(d_ipnum.p, d_ipent.p, nrows, rowstride, d_site_flag.p, s);
  scan_exclusive(d_site_flag.p, d_site_pos.p, nsites, d_misc.p + 7, d_scan, s);
  check(cudaMemcpyAsync(h_pin + 7, d_misc.p + 7, sizeof(int), cudaMemcpyDeviceToHost, s), "nneed");
  // the lists row-major for the mixed passes: row_start[nrows] = all entries
  d_row_start.ensure((size_t) nrows + 1, s);
  scan_exclusive(d_ipnum.p, d_row_start.p, nrows, d_row_start.p + nrows, d_scan, s);
  check(cudaMemcpyAsync(h_pin + 10, d_row_start.p + nrows, sizeof(int), cudaMemcpyDeviceToHost, s),
        "entries");
  sync();
  nneed = h_pin[7];
  d_ent.ensure(std::max(h_pin[10], 1), s);
  mixed::ip_csr(d_ipnum.p, d_ipent.p, nrows, rowstride, d_row_start.p, d_ent.p, s);
  d_need.ensure(std::max(nneed, 1), s);
  d_need_elem.ensure(std::max(nneed, 1), s);
  fp64_fma::need_compact(d_site_flag.p, d_site_pos.p, nsites, d_site_base.p, nall, d_need.p,
                         d_need_elem.p, s);
  launches += 4;
  // for the mixed passes: the row-major lists as line codes
  // (element * maxlines + line) << 6 | kk, and the lines every row's entries
  // (every force row's) reference, a bit per site
  code_kb = 1;
  while ((1 << code_kb) < max_naz) code_kb++;
  codes_ok = max_naz <= 64 && (long long) nall * std::max(maxlines, 1) < (1LL << (31 - code_kb));
  if (codes_ok) {
    const long long nmask = (long long) std::max(nall, 1) * std::max(maxlines, 1);
    mixed::Lattice lat{d_nae.p, d_frac.p, fstride, code_kb};
    mixed::ent_codes(d_ent.p, h_pin[10], d_site_base.p, nall, d_etype.p, d_nae.p, maxlines, code_kb,
                     s);
    d_line_mask.ensure(nmask, s);
    d_line_mask_f.ensure(nmask, s);
    mixed::line_masks(d_row_start.p, d_ent.p, nullptr, nrows, lat, d_row_isforce.p, d_line_mask.p,
                      d_line_mask_f.p, nmask, nullptr, s);
    d_nlines.ensure(2, s);
    self_contained = mixed::self_check(d_row_start.p, d_ent.p, d_row_elem.p, nrows, lat, maxlines,
                                       d_nlines.p, s) == 0;
    mixed::count_lines(d_line_mask.p, d_line_mask_f.p, nmask, d_nlines.p, s);
    check(cudaMemcpyAsync(h_nlines, d_nlines.p, sizeof(h_nlines), cudaMemcpyDeviceToHost, s), "nlines");
    sync();
    launches += 4;
  }
  elist_builds++;
  elists_built = true;
}

// ------------------------------------------------------------------ forces

void cacg_context::pair_compute() {
  pair_compute_pass(1);
  pair_compute_pass(2);
}

// pass 1: LJ forces, or EAM densities + F'(rho) + ghost copy; pass 2: EAM forces
void cacg_context::pair_compute_pass(int pass) {
  if (nlocal == 0) return;
  if (!list_built) fail(CACG_ESTATE, "Pair::compute before the atom neighbor list is built");
  cudaStream_t s = stream;
  bool exact = !fast();
  int nall = nlocal + nghost;
  if (mode == CACG_MIXED) {
    pair_compute_mixed(pass);
    return;
  }
  const float cp = atom_cut_pass();
  if (pass == 1) {
    // float copies and the short list of this step (both FP64 modes)
    d_xh.ensure(nall, s);
    launch_split_hi(d_x.p, d_xh.p, nall, s);
    d_snum.ensure(nlocal, s);
    d_slist.ensure((size_t) maxneigh * stride, s);
    fp64_fma::filter_atoms(d_xh.p, d_num.p, d_list.p, stride, nlocal, cp, d_snum.p, d_slist.p, s);
    launches += 2;
  }
  const int *num = d_snum.p, *lst = d_slist.p;
  if (pair_style == 1) {
    if (pass != 1) return;
    kmark(KT_ATOM1, 0);
    if (exact) fp64_exact::lj_atoms(d_x.p, d_type.p, num, lst, stride, nlocal, d_ljtab.p, d_f.p, s);
    else fp64_fma::lj_atoms(d_x.p, d_xh.p, d_type.p, num, lst, stride, nlocal, d_ljtab.p, cp, d_f.p, s);
    kmark(KT_ATOM1, 1);
    launches++;
    return;
  }
  EamTables e = eamtab();
  if (pass == 1) {
    d_rho.ensure(nall, s);
    d_fp.ensure(nall, s);
    kmark(KT_ATOM1, 0);
    if (exact) fp64_exact::eam_rho_atoms(d_x.p, num, lst, stride, nlocal, e, d_rho.p, d_fp.p, s);
    else fp64_fma::eam_rho_atoms(d_x.p, d_xh.p, num, lst, stride, nlocal, e, cp, d_rho.p, d_fp.p, s);
    kmark(KT_ATOM1, 1);
    // forward_comm_pair: ghost fp = owner fp (comm_brick.cpp:941-971)
    launch_copy_root(d_fp.p, 1, d_root.p, nlocal, nghost, s);
    launches += 2;
  } else {
    kmark(KT_ATOM2, 0);
    if (exact) fp64_exact::eam_force_atoms(d_x.p, num, lst, stride, nlocal, e, d_fp.p, d_f.p, s);
    else fp64_fma::eam_force_atoms(d_x.p, d_xh.p, num, lst, stride, nlocal, e, cp, d_fp.p, d_f.p, s);
    kmark(KT_ATOM2, 1);
    launches++;
  }
}

// Mixed precision, atoms: double-single coordinates, FP32 pair terms, FP64 sums
void cacg_context::pair_compute_mixed(int pass) {
  cudaStream_t s = stream;
  int nall = nlocal + nghost;
  const float eps = band_eps;
  mixed::MixedAtoms m{};
  m.block = mixed_block;
  m.fprime64 = fprime64;
  m.frho_ds = d_frho_ds.p;
  m.x = d_x.p;
  m.num = d_num.p;
  m.list = d_list.p;
  m.stride = stride;
  m.nlocal = nlocal;
  double l0[3], g;
  pack_grid(l0, g);
  if (pass == 1) {
    d_xh.ensure(nall, s);
    d_misc.ensure(32, s);
    if (!oob_zeroed) {
      check(cudaMemsetAsync(d_misc.p + 9, 0, sizeof(int), s), "oob");
      oob_zeroed = true;
    }
    // the displacement since the list reorder (slot 11, float bits), measured
    // against the reorder's packed coordinates when the lists and the grid are
    // unchanged, else set huge so that the lists are reordered in this pass;
    // slot 12: reordered in this pass
    const bool same = part_of == list_builds && ref_g == g && ref_l0[0] == l0[0] &&
                      ref_l0[1] == l0[1] && ref_l0[2] == l0[2];
    check(cudaMemsetAsync(d_misc.p + 11, same ? 0 : 0x7F, sizeof(int), s), "dmax");
    check(cudaMemsetAsync(d_misc.p + 12, 0, sizeof(int), s), "reordered");
    mixed::pack_rel(d_x.p, nall, mixed::make_pack_grid(l0, g, d_misc.p + 9), d_xh.p,
                    same ? d_xq_ref.p : nullptr, nlocal,
                    reinterpret_cast<unsigned *>(d_misc.p + 11), s);
    launches++;
  }
  m.xq = d_xh.p;
  m.qg = (float) g;
  d_snum.ensure(std::max(nlocal, 1), s);
  d_slist.ensure((size_t) maxneigh * stride, s);
  m.snum = d_snum.p;
  m.slist = d_slist.p;
  if (pair_style == 1) {
    if (pass != 1) return;
    m.cutsq_f = 0.f;
    m.band_lo = 1.0f - eps;
    m.band_hi = 1.0f + eps;
    const int T = (MAXT + 1) * (MAXT + 1);
    mixed::lj_atoms(m, d_type.p, d_ljf.p, d_ljf.p + T, d_ljf.p + 2 * T, d_cutsq64.p, d_f.p, s);
    launches++;
    return;
  }
  EamTables e = eamtab();
  m.cutsq = cutforcesq;
  m.cutsq_f = (float) cutforcesq;
  m.band_lo = m.cutsq_f * (1.0f - eps);
  m.band_hi = m.cutsq_f * (1.0f + eps);
  if (mixed_union && pass == 1 && union_of != list_builds) {
    // the groups' neighbor unions, once per atom list build
    const int ngroups = (nlocal + 31) / 32;
    d_union_j.ensure((size_t) std::max(ngroups, 1) * mixed::union_max(), s);
    d_union_n.ensure(std::max(ngroups, 1), s);
    d_slot.ensure((size_t) maxneigh * stride, s);
    d_sslot.ensure((size_t) maxneigh * stride, s);
    mixed::union_build(d_num.p, d_list.p, stride, nlocal, d_union_j.p, d_union_n.p, d_slot.p, s);
    launches++;
    union_of = list_builds;
  }
  if (!mixed_union) {
    if (pass == 1) {
      d_mlist.ensure((size_t) maxneigh * stride, s);
      d_nnear.ensure(std::max(nlocal, 1), s);
      d_xq_ref.ensure(std::max(nlocal, 1), s);
      if (!areorders_zeroed) {
        check(cudaMemsetAsync(d_misc.p + 16, 0, sizeof(int), s), "areorders");
        areorders_zeroed = true;
      }
      kmark(KT_APART, 0);
      mixed::list_partition(d_xh.p, m.qg, d_num.p, d_list.p, stride, nlocal, m.band_hi,
                            (float) std::sqrt(cutforcesq), d_mlist.p, d_nnear.p, d_xq_ref.p,
                            reinterpret_cast<unsigned *>(d_misc.p + 11),
                            reinterpret_cast<unsigned *>(d_misc.p + 16), s);
      kmark(KT_APART, 1);
      for (int d = 0; d < 3; d++) ref_l0[d] = l0[d];
      ref_g = g;
      launches++;
      part_of = list_builds;
    }
    m.list = d_mlist.p;
    m.nnear = mixed_cull ? d_nnear.p : nullptr;
    m.dmax2 = reinterpret_cast<const unsigned *>(d_misc.p + 11);
  }
  if (pass == 1) {
    d_rho.ensure(nall, s);
    d_fpf.ensure(nall, s);
    if (mixed_union)
      mixed::eam_rho_union(m, d_union_j.p, d_union_n.p, d_slot.p, d_sslot.p, d_rhor_val4.p, e,
                           d_fp4.p, d_rho.p, d_fpf.p, s);
    else {
      kmark(KT_ATOM1, 0);
      mixed::eam_rho_atoms(m, d_rhor_val4.p, e, d_fp4.p, d_rho.p, d_fpf.p, s);
      kmark(KT_ATOM1, 1);
    }
    launch_copy_root(d_fpf.p, 1, d_root.p, nlocal, nghost, s);
    launches += 2;
  } else {
    if (mixed_union)
      mixed::eam_force_union(m, d_union_j.p, d_union_n.p, d_sslot.p, d_ftab.p, e, d_fpf.p, d_f.p,
                             s);
    else {
      kmark(KT_ATOM2, 0);
      mixed::eam_force_atoms(m, d_ftab.p, e, d_fpf.p, d_f.p, s);
      kmark(KT_ATOM2, 1);
    }
    launches++;
  }
}

// Mixed precision, elements: sites and integration points interpolated in
// double-single FP32 (hi/lo float pairs) and packed cell-relative, FP32 pair
// terms, FP64 sums and FP64 nodal gather
void cacg_context::pair_ecompute_mixed() {
  cudaStream_t s = stream;
  int nall = enlocal + enghost;
  if (!codes_ok)
    fail(CACG_EINVAL, "mixed element passes: at most 64 sites per lattice line and 2^(31 - bits of "
                      "the sites per line) lattice lines (element list build)");
  double l0[3], g;
  pack_grid(l0, g);
  d_misc.ensure(32, s);
  if (!oob_zeroed) {
    check(cudaMemsetAsync(d_misc.p + 9, 0, sizeof(int), s), "oob");
    oob_zeroed = true;
  }
  const mixed::PackGrid pg = mixed::make_pack_grid(l0, g, d_misc.p + 9);
  const long long nmask = (long long) std::max(nall, 1) * std::max(maxlines, 1);
  d_node_hl.ensure((size_t) 24 * nall, s);
  d_line_pos.ensure(3 * (size_t) nmask, s);
  // displacement culling of the integration-point lists: slot 13 holds the
  // largest squared node displacement since the last reorder (set huge after
  // an element list build, so that this pass reorders), slot 14 flags a
  // reorder in this pass.  The lists are kept reordered even with "tune cull
  // no", so that culling changes no bit: it only stops each row early.
  const bool cull_e = mixed_cull;
  unsigned *eflags = reinterpret_cast<unsigned *>(d_misc.p + 13);
  const bool same_e = epart_of == elist_builds;
  d_ent_near.ensure(std::max((size_t) 1, d_ent.cap), s);
  d_nnear_row.ensure(std::max(nrows, 1), s);
  d_node_ref.ensure((size_t) 24 * nall, s);
  d_line_mask_n.ensure(nmask, s);
  d_line_mask_nf.ensure(nmask, s);
  if (!ereorders_zeroed) {
    check(cudaMemsetAsync(d_misc.p + 15, 0, sizeof(int), s), "ereorders");
    ereorders_zeroed = true;
  }
  check(cudaMemsetAsync(d_misc.p + 13, same_e ? 0 : 0x7F, sizeof(int), s), "edmax");
  check(cudaMemsetAsync(d_misc.p + 14, 0, sizeof(int), s), "ereordered");
  const EamTables et = pair_style == 2 ? eamtab() : EamTables{};
  const bool fused = fused_on && self_contained && fused_types_ok &&
                     mixed::fused_fits(pair_style == 2 ? et.nr : 0, pair_style == 2 ? et.nrho : 0);
  // the fused passes need the line data and row points only to reorder the lists
  const unsigned *gate = fused ? eflags : nullptr;
  fused_used = fused;
  kmark(KT_SITES, 0);
  mixed::node_split(d_nodex.p, nall, d_node_hl.p, same_e ? d_node_ref.p : nullptr, eflags, s);
  const mixed::Lattice lat{d_nae.p, d_frac.p, fstride, code_kb};
  // the lattice lines that the scanned entries reference (all referenced
  // lines in a step that reorders)
  mixed::lines(d_node_hl.p, d_etype.p, lat, max_nax, d_line_mask.p,
               cull_e ? d_line_mask_n.p : nullptr, eflags, maxlines, pg, nall, d_line_pos.p, s,
               gate);
  kmark(KT_SITES, 1);
  d_ip_q.ensure(std::max(nrows, 1), s);
  d_ip_h.ensure(std::max(nrows, 1), s);
  d_ip_l.ensure(std::max(nrows, 1), s);
  kmark(KT_EPREP, 0);
  mixed::row_q(d_row_elem.p, d_row_jj.p, d_etype.p, d_int_off.p, d_spa_int_hl.p, d_node_hl.p, nrows,
               pg, d_ip_q.p, d_ip_h.p, d_ip_l.p, s, gate);
  const double csq_e = pair_style == 1 ? ljtab.cutsq[1 * (MAXT + 1) + 1] : cutforcesq;
  mixed::ip_reorder(d_row_start.p, d_ent.p, nrows, d_ip_q.p, d_line_pos.p, lat, pg,
                    (float) std::sqrt(csq_e), d_ent_near.p, d_nnear_row.p, d_node_hl.p, nall,
                    d_node_ref.p, eflags, s);
  mixed::line_masks(d_row_start.p, d_ent_near.p, d_nnear_row.p, nrows, lat, d_row_isforce.p,
                    d_line_mask_n.p, d_line_mask_nf.p, nmask, eflags, s);
  kmark(KT_EPREP, 1);
  launches += 6;
  epart_of = elist_builds;
  const bool use_sur = sur && nfar > 0;
  const float eps = band_eps;
  mixed::MixedElems m{};
  m.block = mixed_block;
  if (mixed_ip_group) {
    m.group = mixed_ip_group;
  } else {
    int dev = 0, nsm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    const long long want = (long long) nsm * 2048;
    m.group = (long long) nforce * 4 >= want ? 4 : (long long) nforce * 8 >= want ? 8 : 16;
  }
  m.line_pos = d_line_pos.p;
  m.ip_q = d_ip_q.p;
  m.ip_h = d_ip_h.p;
  m.ip_l = d_ip_l.p;
  m.etype = d_etype.p;
  m.row_elem = d_row_elem.p;
  m.row_first = d_row_first.p;
  m.node_list = d_node_list.p;
  m.row_start = d_row_start.p;
  m.ent = d_ent_near.p;
  m.nnear_row = cull_e ? d_nnear_row.p : nullptr;
  m.eflags = eflags;
  m.nlocal_e = enlocal;
  m.rows = d_force_rows.p;
  m.nforce = nforce;
  m.lat = lat;
  m.pg = pg;
  if (use_sur) m.skip = d_skip.p;
  if (fused) {
    if (d_band.cap < 3 + (size_t) enlocal) {  // outside captures: the eager step allocates
      d_band.ensure(3 + (size_t) enlocal, s);
      check(cudaMemsetAsync(d_band.p, 0, 3 * sizeof(int), s), "band list");
    }
    mixed::FusedTables ft{d_node_hl.p, d_nodex.p, d_int_off.p, d_inter_off.p, d_intp4.p,
                          d_spa_int.p, d_spa_inter.p, d_fjj.p, d_fjj_off.p, d_wn.p, maxlines,
                          fused_variant, d_spa_int_hl.p, d_frho_ds.p, d_wnf.p, d_band.p,
                          d_lat_rec.p};
    // the surrogate's nodal forces go in before the force pass, which skips
    // (writes nothing for) the elements the surrogate evaluates
    auto sur_write = [&] {
      surrogate::write_forces(d_smean.p, d_far.p, d_sdue.p, d_sdue_n.p, nfar, d_skip.p, d_nodef.p, s);
      launches++;
    };
    // the force pass, in parts when run_host copies the node velocities out
    // part by part (each part's velocities integrated while the next part's
    // forces run); the caller integrates the last part
    auto force_parts = [&](auto pass) {
      const int want = out_parts ? out_parts : enlocal >= 65536 ? 4 : 1;
      const int parts = out_split ? std::max(1, std::min(want, enlocal)) : 1;
      part_bounds.assign(parts + 1, enlocal);
      for (int p = 0; p < parts; p++) part_bounds[p] = (int) ((long long) enlocal * p / parts);
      for (int p = 0; p < parts; p++) {
        pass(part_bounds[p], part_bounds[p + 1]);
        launches += 2;  // the pass and its guard-band exact pass
        if (p + 1 < parts) {
          nve_nodes_final_range(part_bounds[p], part_bounds[p + 1]);
          check(cudaEventRecord(ev_nvpart[p], s), "nodev part final");
        }
      }
      parts_done = parts;
    };
    if (pair_style == 1) {
      int a = 1 * (MAXT + 1) + 1;
      m.cutsq = ljtab.cutsq[a];
      m.cutsq_f = (float) m.cutsq;
      m.band_lo = m.cutsq_f * (1.0f - eps);
      m.band_hi = m.cutsq_f * (1.0f + eps);
      if (use_sur) {
        kmark(KT_SUR, 0);
        surrogate_predict(et);
        kmark(KT_SUR, 1);
        sur_write();
      }
      kmark(KT_ELEM_FORCE, 0);
      force_parts([&](int b0, int b1) {
        mixed::elem_fused(m, ft, 0, nullptr, et, (float) ljtab.lj1[a], (float) ljtab.lj2[a],
                          nullptr, nullptr, d_nodef.p, s, b0, b1);
      });
      kmark(KT_ELEM_FORCE, 1);
    } else {
      m.cutsq = cutforcesq;
      m.cutsq_f = (float) cutforcesq;
      m.band_lo = m.cutsq_f * (1.0f - eps);
      m.band_hi = m.cutsq_f * (1.0f + eps);
      m.fp4 = d_fp4.p;
      m.nrho = nrho;
      m.rdrho = (float) rdrho;
      d_erho.ensure((size_t) NPE * nall, s);
      kmark(KT_ELEM_RHO, 0);
      mixed::elem_fused(m, ft, 1, d_rhor_val4.p, et, 0.f, 0.f, nullptr, d_erho.p, nullptr, s);
      kmark(KT_ELEM_RHO, 1);
      launches += 2;  // the pass and its guard-band exact pass
      if (use_sur) {
        kmark(KT_SUR, 0);
        surrogate_predict(et);
        kmark(KT_SUR, 1);
        sur_write();
      }
      kmark(KT_ELEM_FORCE, 0);
      force_parts([&](int b0, int b1) {
        mixed::elem_fused(m, ft, 2, d_ftab.p, et, 0.f, 0.f, d_erho.p, nullptr, d_nodef.p, s, b0,
                          b1);
      });
      kmark(KT_ELEM_FORCE, 1);
    }
    return;
  }
  if (pair_style == 1) {
    int a = 1 * (MAXT + 1) + 1;
    m.cutsq = ljtab.cutsq[a];
    m.cutsq_f = (float) m.cutsq;
    m.band_lo = m.cutsq_f * (1.0f - eps);
    m.band_hi = m.cutsq_f * (1.0f + eps);
    EamTables e{};
    if (use_sur) {
      kmark(KT_SUR, 0);
      surrogate_predict(eamtab());
      kmark(KT_SUR, 1);
    }
    kmark(KT_ELEM_FORCE, 0);
    mixed::ip_pass(m, 0, nullptr, e, (float) ljtab.lj1[a], (float) ljtab.lj2[a], nullptr,
                   d_fipf.p, s);
    kmark(KT_ELEM_FORCE, 1);
    launches++;
  } else {
    EamTables e = eamtab();
    m.cutsq = cutforcesq;
    m.cutsq_f = (float) cutforcesq;
    m.band_lo = m.cutsq_f * (1.0f - eps);
    m.band_hi = m.cutsq_f * (1.0f + eps);
    d_erho.ensure((size_t) NPE * nall, s);
    d_line_rho.ensure(nmask, s);
    kmark(KT_ELEM_RHO, 0);
    mixed::ip_pass(m, 1, d_rhor_val4.p, e, 0.f, 0.f, d_erho.p, nullptr, s);
    kmark(KT_ELEM_RHO, 1);
    launch_copy_root(d_erho.p, NPE, d_eroot.p, enlocal, enghost, s);
    kmark(KT_SITE_FP, 0);
    mixed::line_rho(d_erho.p, d_etype.p, lat, d_line_mask_f.p, cull_e ? d_line_mask_nf.p : nullptr,
                    eflags, maxlines, nall, d_line_rho.p, s);
    d_row_fpf.ensure(std::max(nrows, 1), s);
    mixed::row_fp(d_force_rows.p, nforce, d_row_elem.p, d_row_jj.p, d_etype.p, d_int_off.p,
                  d_spa_int.p, d_erho.p, e, d_row_fpf.p, s);
    kmark(KT_SITE_FP, 1);
    m.line_rho = d_line_rho.p;
    m.fp4 = d_fp4.p;
    m.nrho = nrho;
    m.rdrho = (float) rdrho;
    m.row_fp = d_row_fpf.p;
    if (use_sur) {
      kmark(KT_SUR, 0);
      surrogate_predict(e);
      kmark(KT_SUR, 1);
    }
    kmark(KT_ELEM_FORCE, 0);
    mixed::ip_pass(m, 2, d_ftab.p, e, 0.f, 0.f, nullptr, d_fipf.p, s);
    kmark(KT_ELEM_FORCE, 1);
    launches += 5;
  }
  mixed::gather_nodef(d_fipf.p, d_etype.p, d_row_first.p, d_numint.p, d_int_off.p, d_wn.p, enlocal,
                      d_nodef.p, s);
  launches++;
  if (use_sur) {
    surrogate::write_forces(d_smean.p, d_far.p, d_sdue.p, d_sdue_n.p, nfar, d_skip.p, d_nodef.p, s);
    launches++;
  }
}

// ------------------------------------------------------------------ analysis and output

// Output::centro_atom (output.cpp:352-447) over the atom list, in chunks of
// atoms so that the per-atom neighbor scratch stays bounded
void cacg_context::compute_centro(double *out) {
  if (!list_built) fail(CACG_ESTATE, "centro-symmetry before the atom neighbor list is built");
  cudaStream_t s = stream;
  DBuf<double> d_out, d_dsq;
  DBuf<int> d_near;
  const int chunk = std::max(1, std::min(nlocal, 65536));
  d_out.ensure(std::max(nlocal, 1), s);
  d_dsq.ensure((size_t) std::max(maxneigh, 1) * chunk, s);
  d_near.ensure((size_t) std::max(maxneigh, 1) * chunk, s);
  for (int i0 = 0; i0 < nlocal; i0 += chunk)
    analysis::centro(d_x.p, d_num.p, d_list.p, stride, i0, std::min(chunk, nlocal - i0),
                     cutneighmaxsq, d_dsq.p, d_near.p, chunk, d_out.p, s);
  launches += (nlocal + chunk - 1) / chunk;
  if (nlocal)
    check(cudaMemcpyAsync(out, d_out.p, sizeof(double) * nlocal, cudaMemcpyDeviceToHost, s), "centro");
  sync();
  d_out.release();
  d_dsq.release();
  d_near.release();
}

// DumpXyz (dump_xyz.cpp:36-140 with Dump::count, dump.cpp:352-365): the atoms
// with 1 < centro < 10, header "N\nXYZ\n", lines "Cu x y z centro" (%g)
void cacg_context::dump_xyz(const char *path) {
  std::vector<double> c(std::max(nlocal, 1));
  compute_centro(c.data());
  std::vector<double4> x4(std::max(nlocal, 1));
  if (nlocal)
    check(cudaMemcpyAsync(x4.data(), d_x.p, sizeof(double4) * nlocal, cudaMemcpyDeviceToHost, stream), "x");
  sync();
  FILE *fp = fopen(path, "w");
  if (!fp) fail(CACG_EIO, "Cannot open dump file %s", path);
  long long nd = 0;
  for (int i = 0; i < nlocal; i++) nd += c[i] > 1 && c[i] < 10;
  fprintf(fp, "%lld\nXYZ\n", nd);
  for (int i = 0; i < nlocal; i++)
    if (c[i] > 1 && c[i] < 10) fprintf(fp, "Cu %g %g %g %g\n", x4[i].x, x4[i].y, x4[i].z, c[i]);
  fclose(fp);
}

// DumpElement (dump_element.cpp:69-128): a Tecplot FE-brick zone of the local
// elements' nodes, one "x y z vx vy vz fx fy fz" (%g) line per node in
// element order, then each element's 8 node numbers (1-based, consecutive:
// the reference writes connectivity one element after another).  n counts
// the nodes written (the reference's header takes the atom count of its
// centro filter, dump.cpp:247, which does not describe the element zone).
void cacg_context::dump_elements(const char *path, int append) {
  if (!inited) fail(CACG_ESTATE, "no device state yet (cacg_init)");
  const int n = enlocal;
  std::vector<double> nx((size_t) 24 * n + 1), nv((size_t) 24 * n + 1), nf((size_t) 24 * n + 1);
  if (n) {
    check(cudaMemcpyAsync(nx.data(), d_nodex.p, sizeof(double) * 24 * n, cudaMemcpyDeviceToHost, stream), "nodex");
    check(cudaMemcpyAsync(nv.data(), d_nodev.p, sizeof(double) * 24 * n, cudaMemcpyDeviceToHost, stream), "nodev");
    check(cudaMemcpyAsync(nf.data(), d_nodef.p, sizeof(double) * 24 * n, cudaMemcpyDeviceToHost, stream), "nodef");
  }
  sync();
  FILE *fp = fopen(path, append ? "a" : "w");
  if (!fp) fail(CACG_EIO, "Cannot open dump file %s", path);
  const long long nn = (long long) NPE * n;
  fprintf(fp, "title=\"results for cac\"\n");
  fprintf(fp, "variables=\"x\", \"y\", \"z\", \"vx\", \"vy\", \"vz\", \"fx\", \"fy\", \"fz\"\n");
  fprintf(fp, "zone t=\"load step %lld\",", ntimestep);
  fprintf(fp, " n=  %lld e =  %d", nn, n);
  fprintf(fp, " datapacking=point, zonetype=febrick\n");
  for (long long k = 0; k < nn; k++)
    fprintf(fp, "%g %g %g %g %g %g %g %g %g\n", nx[3 * k], nx[3 * k + 1], nx[3 * k + 2], nv[3 * k],
            nv[3 * k + 1], nv[3 * k + 2], nf[3 * k], nf[3 * k + 1], nf[3 * k + 2]);
  for (int e = 0; e < n; e++) {
    long long b = (long long) NPE * e;
    fprintf(fp, "%lld %lld %lld %lld %lld %lld %lld %lld\n", b + 1, b + 2, b + 3, b + 4, b + 5,
            b + 6, b + 7, b + 8);
  }
  fclose(fp);
}

// ------------------------------------------------------------------ surrogate

void cacg_context::surrogate_reference(const double *nodex0) {
  if (!inited || enlocal == 0) fail(CACG_ESTATE, "no elements on the device yet");
  d_nodex0.ensure((size_t) 24 * enlocal, stream);
  if (nodex0)
    check(cudaMemcpyAsync(d_nodex0.p, nodex0, sizeof(double) * 24 * enlocal, cudaMemcpyHostToDevice, stream), "nodex0");
  else
    check(cudaMemcpyAsync(d_nodex0.p, d_nodex.p, sizeof(double) * 24 * enlocal, cudaMemcpyDeviceToDevice, stream), "nodex0");
  have_x0 = true;
}

// features (raw) and plain-quadrature nodal forces of every local element at
// the current state, in the handle's precision mode, the surrogate detached
void cacg_context::surrogate_samples(float *x, float *t) {
  if (!elists_built) fail(CACG_ESTATE, "samples before the node neighbor list is built");
  if (!have_x0) surrogate_reference(nullptr);
  cacg_mlp_t *keep = sur;
  sur = nullptr;
  try {
    forward_comm();  // ghosts follow nodes put since the last step
    pair_ecompute();
  } catch (...) {
    sur = keep;
    throw;
  }
  sur = keep;
  cudaStream_t s = stream;
  d_sraw.ensure((size_t) enlocal * (MLP_IN + MLP_OUT), s);
  surrogate::raw_features(d_nodex.p, d_nodex0.p, pair_style == 2 ? d_erho.p : nullptr, enlocal,
                          d_sraw.p, s);
  surrogate::to_float(d_nodef.p, (long long) enlocal * MLP_OUT, d_sraw.p + (size_t) enlocal * MLP_IN, s);
  check(cudaMemcpyAsync(x, d_sraw.p, sizeof(float) * enlocal * MLP_IN, cudaMemcpyDeviceToHost, s), "x");
  check(cudaMemcpyAsync(t, d_sraw.p + (size_t) enlocal * MLP_IN, sizeof(float) * enlocal * MLP_OUT,
                        cudaMemcpyDeviceToHost, s), "t");
  sync();
}

// Elements whose whole extent (centre +- the largest centre-node distance)
// lies farther than `dist` from every local atom use the surrogate; the rows
// lists of both kinds are fixed here.
void cacg_context::surrogate_attach(cacg_mlp_t *m, double tol, double dist) {
  invalidate_graph();
  sur = nullptr;
  nfar = 0;
  if (!m) return;
  if (mode != CACG_MIXED) fail(CACG_EINVAL, "the surrogate runs in the mixed-precision element pass");
  if (!elists_built || !setup_done) fail(CACG_ESTATE, "attach the surrogate after the lists are built");
  if (!(tol >= 0) || !(dist >= 0)) fail(CACG_EINVAL, "bad surrogate tolerance or distance");
  if (!have_x0) surrogate_reference(nullptr);
  cudaStream_t s = stream;
  std::vector<double> nx((size_t) 24 * enlocal), ax;
  check(cudaMemcpyAsync(nx.data(), d_nodex.p, sizeof(double) * nx.size(), cudaMemcpyDeviceToHost, s), "nodex");
  std::vector<double4> x4(nlocal);
  if (nlocal)
    check(cudaMemcpyAsync(x4.data(), d_x.p, sizeof(double4) * nlocal, cudaMemcpyDeviceToHost, s), "x");
  sync();
  std::vector<double> cx(3 * enlocal), rad(enlocal);
  double rmax = 0.0;
  for (int e = 0; e < enlocal; e++) {
    double c[3] = {0, 0, 0};
    for (int k = 0; k < NPE; k++)
      for (int d = 0; d < 3; d++) c[d] += nx[24 * e + 3 * k + d] / NPE;
    double r2 = 0.0;
    for (int k = 0; k < NPE; k++) {
      double q = 0.0;
      for (int d = 0; d < 3; d++) q += (nx[24 * e + 3 * k + d] - c[d]) * (nx[24 * e + 3 * k + d] - c[d]);
      r2 = std::max(r2, q);
    }
    for (int d = 0; d < 3; d++) cx[3 * e + d] = c[d];
    rad[e] = std::sqrt(r2);
    rmax = std::max(rmax, rad[e]);
  }
  // atoms binned in cubes of side >= dist + rmax
  const double side = std::max(dist + rmax, 1e-6);
  int nb[3];
  for (int d = 0; d < 3; d++) nb[d] = std::max(1, std::min(1024, (int) std::floor(prd[d] / side)));
  auto cell = [&](double v, int d) {
    int c = (int) std::floor((v - lo[d]) / prd[d] * nb[d]);
    return std::min(std::max(c, 0), nb[d] - 1);
  };
  std::vector<std::vector<int>> bins((size_t) nb[0] * nb[1] * nb[2]);
  for (int i = 0; i < nlocal; i++)
    bins[((size_t) cell(x4[i].x, 0) * nb[1] + cell(x4[i].y, 1)) * nb[2] + cell(x4[i].z, 2)].push_back(i);
  std::vector<int> far;
  for (int e = 0; e < enlocal; e++) {
    const double lim = dist + rad[e];
    const double *c = &cx[3 * e];
    int cc[3] = {cell(c[0], 0), cell(c[1], 1), cell(c[2], 2)};
    bool near_ = false;
    for (int dx = -1; dx <= 1 && !near_; dx++)
      for (int dy = -1; dy <= 1 && !near_; dy++)
        for (int dz = -1; dz <= 1 && !near_; dz++) {
          int q[3] = {cc[0] + dx, cc[1] + dy, cc[2] + dz};
          bool outside = false;
          for (int d = 0; d < 3; d++)
            if (q[d] < 0 || q[d] >= nb[d]) {
              if (periodic[d]) q[d] = (q[d] + nb[d]) % nb[d];
              else outside = true;
            }
          if (outside) continue;
          for (int i : bins[((size_t) q[0] * nb[1] + q[1]) * nb[2] + q[2]]) {
            double dd[3] = {x4[i].x - c[0], x4[i].y - c[1], x4[i].z - c[2]};
            double r2 = 0.0;
            for (int d = 0; d < 3; d++) {
              if (periodic[d]) dd[d] -= prd[d] * std::nearbyint(dd[d] / prd[d]);
              r2 += dd[d] * dd[d];
            }
            if (r2 < lim * lim) {
              near_ = true;
              break;
            }
          }
        }
    if (!near_) {
      far.push_back(e);
    }
  }
  nfar = (int) far.size();
  upload(d_far, far.empty() ? std::vector<int>{0} : far, s);
  d_skip.ensure(std::max(enlocal, 1), s);
  check(cudaMemsetAsync(d_skip.p, 0, std::max(enlocal, 1), s), "skip");
  d_swait.ensure(std::max(nfar, 1), s);
  d_sstreak.ensure(std::max(nfar, 1), s);
  check(cudaMemsetAsync(d_swait.p, 0, std::max(nfar, 1), s), "wait");
  check(cudaMemsetAsync(d_sstreak.p, 0, std::max(nfar, 1), s), "streak");
  d_sdue.ensure(std::max(nfar, 1), s);
  d_sdue_n.ensure(1, s);
  d_scount.ensure(2, s);
  check(cudaMemsetAsync(d_scount.p, 0, 2 * sizeof(unsigned long long), s), "scount");
  d_sfeat.ensure((size_t) 64 * std::max(nfar, 1), s);
  d_smean.ensure((size_t) MLP_OUT * std::max(nfar, 1), s);
  d_sspread.ensure(std::max(nfar, 1), s);
  sur_tol = tol;
  sur_dist = dist;
  sur = m;
  sync();
}

// The far elements due for a test this step are compacted on the device; their
// features, the ensemble and the acceptance run on that list (the launches
// cover every far element and stop at the device count).
void cacg_context::surrogate_predict(const EamTables &) {
  mlp::Net *net = mlp::net_of(sur);
  cudaStream_t s = stream;
  surrogate::due(nfar, d_far.p, d_swait.p, d_skip.p, d_sdue.p, d_sdue_n.p, s);
  d_sfar_due.ensure(std::max(nfar, 1), s);
  surrogate::gather_far(d_far.p, d_sdue.p, d_sdue_n.p, nfar, d_sfar_due.p, s);
  surrogate::features(d_nodex.p, d_nodex0.p, pair_style == 2 ? d_erho.p : nullptr, d_sfar_due.p,
                      nfar, d_sdue_n.p, mlp::norm_device(net), d_sfeat.p, s);
  mlp::predict(net, d_sfeat.p, nfar, d_smean.p, d_sspread.p, s, d_sdue_n.p);
  surrogate::accept(d_sspread.p, d_far.p, d_sdue.p, d_sdue_n.p, nfar,
                    (float) (sur_tol * mlp::force_scale(net)), d_skip.p, d_swait.p, d_sstreak.p,
                    d_scount.p, s);
  launches += 6;
}

void cacg_context::pair_ecompute() {
  if (enlocal == 0) return;
  if (!elists_built) fail(CACG_ESTATE, "Pair::ecompute before the node neighbor list is built");
  if (mode == CACG_MIXED) {
    pair_ecompute_mixed();
    return;
  }
  cudaStream_t s = stream;
  bool exact = !fast();
  int nall = enlocal + enghost;
  ElemTables t = etab();
  // sites of every local and ghost element at the current node positions,
  // with their float copies, then this step's short lists of the rows
  d_site_h.ensure(std::max(nsites, 1), s);
  // contraction-free in both modes: bit-identical to the all-sites kernel
  kmark(KT_SITES, 0);
  fp64_fma::sites_needed(d_nodex.p, d_etype.p, d_site_base.p, d_need.p, d_need_elem.p, nneed, t,
                         d_site_x.p, d_site_h.p, s);
  kmark(KT_SITES, 1);
  const double csq = pair_style == 1 ? ljtab.cutsq[1 * (MAXT + 1) + 1] : cutforcesq;
  const float cp = cut_pass(csq);
  d_sipnum.ensure(std::max(nrows, 1), s);
  d_sipent.ensure((size_t) maxip * rowstride, s);
  fp64_fma::filter_rows(d_nodex.p, d_etype.p, d_row_elem.p, d_row_jj.p, nrows, d_ipnum.p, d_ipent.p,
                        rowstride, d_site_h.p, t, cp, exact ? 0 : 1, d_sipnum.p, d_sipent.p, s);
  launches += 2;
  const int *ipn = d_sipnum.p, *ipe = d_sipent.p;
  if (pair_style == 1) {
    int a = 1 * (MAXT + 1) + 1;
    kmark(KT_ELEM_FORCE, 0);
    if (exact)
      fp64_exact::lj_ip(d_nodex.p, d_etype.p, d_row_elem.p, d_row_jj.p, nrows, ipn, ipe,
                        rowstride, d_site_x.p, t, ljtab.lj1[a], ljtab.lj2[a], ljtab.cutsq[a], d_fip.p, s);
    else
      fp64_fma::lj_ip(d_nodex.p, d_etype.p, d_row_elem.p, d_row_jj.p, nforce, ipn, ipe,
                      rowstride, d_site_x.p, d_site_h.p, t, ljtab.lj1[a], ljtab.lj2[a], ljtab.cutsq[a],
                      cp, d_force_rows.p, d_fip.p, s);
    kmark(KT_ELEM_FORCE, 1);
    launches++;
  } else {
    EamTables e = eamtab();
    d_erho.ensure((size_t) NPE * nall, s);
    d_site_fp.ensure(std::max(nsites, 1), s);
    kmark(KT_ELEM_RHO, 0);
    if (exact) {
      fp64_exact::eam_erho(d_nodex.p, d_etype.p, d_row_first.p, enlocal, ipn, ipe, rowstride, d_site_x.p, t, e, d_erho.p, s);
    } else {
      fp64_fma::eam_erho(d_nodex.p, d_etype.p, d_row_first.p, enlocal, ipn, ipe, rowstride, d_site_x.p, d_site_h.p, t, e, cp, d_erho.p, s);
    }
    kmark(KT_ELEM_RHO, 1);
    // eforward_comm_pair: ghost nodal densities from their owners (comm_brick.cpp:978-1010)
    launch_copy_root(d_erho.p, NPE, d_eroot.p, enlocal, enghost, s);
    if (exact) {
      kmark(KT_SITE_FP, 0);
      fp64_exact::eam_site_fp(d_erho.p, d_etype.p, d_site_base.p, nall, t, e, d_site_fp.p, s);
      kmark(KT_SITE_FP, 1);
      kmark(KT_ELEM_FORCE, 0);
      fp64_exact::eam_ip(d_nodex.p, d_erho.p, d_etype.p, d_row_elem.p, d_row_jj.p, nrows, ipn, ipe,
                         rowstride, d_site_x.p, d_site_fp.p, t, e, d_fip.p, s);
      kmark(KT_ELEM_FORCE, 1);
    } else {
      kmark(KT_SITE_FP, 0);
      fp64_fma::site_fp_needed(d_erho.p, d_etype.p, d_site_base.p, d_need.p, d_need_elem.p, nneed,
                               t, e, d_site_fp.p, s);
      kmark(KT_SITE_FP, 1);
      kmark(KT_ELEM_FORCE, 0);
      fp64_fma::eam_ip(d_nodex.p, d_erho.p, d_etype.p, d_row_elem.p, d_row_jj.p, nforce, ipn, ipe,
                       rowstride, d_site_x.p, d_site_h.p, d_site_fp.p, t, e, cp, d_force_rows.p,
                       d_fip.p, s);
      kmark(KT_ELEM_FORCE, 1);
    }
    launches += 4;
  }
  if (exact) fp64_exact::gather_nodef(d_fip.p, d_etype.p, d_row_first.p, enlocal, t, d_nodef.p, s);
  else fp64_fma::gather_nodef(d_fip.p, d_etype.p, d_row_first.p, enlocal, t, d_nodef.p, s);
  launches++;
}

// ------------------------------------------------------------------ thermo

void cacg_context::compute_thermo(double *out) {
  if (!setup_done || (nlocal && !list_built) || (enlocal && !elists_built))
    fail(CACG_ESTATE, "thermo before the neighbor lists are built");
  cudaStream_t s = stream;
  for (int k = 0; k < 17; k++) out[k] = 0.0;
  auto reduce = [&](int nblocks, double *acc) {
    std::vector<double> h((size_t) nblocks * 7);
    check(cudaMemcpyAsync(h.data(), d_part.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, s), "part");
    sync();
    for (int b = 0; b < nblocks; b++)
      for (int k = 0; k < 7; k++) acc[k] += h[(size_t) b * 7 + k];
  };
  const double mvv2e = metal ? 1.0364269e-4 : 1.0;  // force->mvv2e (update.cpp:90,110)
  double q[7];
  if (nlocal) {
    int nb = thermo::partial_blocks(nlocal);
    d_part.ensure((size_t) nb * 7, s);
    int nall = nlocal + nghost;
    if (pair_style == 1) {
      thermo::atoms_lj(d_x.p, d_type.p, d_num.p, d_list.p, stride, nlocal, d_lj5.p, d_part.p, s);
    } else {
      EamTables e = eamtab();
      d_rho.ensure(nall, s);
      d_fp.ensure(nall, s);
      fp64_exact::eam_rho_atoms(d_x.p, d_num.p, d_list.p, stride, nlocal, e, d_rho.p, d_fp.p, s);
      launch_copy_root(d_fp.p, 1, d_root.p, nlocal, nghost, s);
      thermo::atoms_eam(d_x.p, d_num.p, d_list.p, stride, nlocal, e, d_rho.p, d_fp.p, d_part.p, s);
    }
    for (double &v : q) v = 0.0;
    reduce(nb, q);
    out[0] = q[0];
    for (int k = 0; k < 6; k++) out[4 + k] += q[1 + k];
    nb = thermo::partial_blocks(nlocal);
    thermo::kinetic(d_v.p, d_type.p, d_mass.p, nlocal, 1, 1.0, d_part.p, s);
    for (double &v : q) v = 0.0;
    reduce(nb, q);
    out[2] = q[0] * mvv2e;
    for (int k = 0; k < 6; k++) out[10 + k] += q[1 + k] * mvv2e;
  }
  if (enlocal) {
    int nall = enlocal + enghost;
    ElemTables t = etab();
    EamTables e = eamtab();
    d_site_x.ensure(std::max(nsites, 1), s);
    d_site_h.ensure(std::max(nsites, 1), s);
    fp64_fma::sites_needed(d_nodex.p, d_etype.p, d_site_base.p, d_need.p, d_need_elem.p, nneed, t,
                           d_site_x.p, d_site_h.p, s);
    if (pair_style == 2) {
      d_erho.ensure((size_t) NPE * nall, s);
      d_site_fp.ensure(std::max(nsites, 1), s);
      fp64_exact::eam_erho(d_nodex.p, d_etype.p, d_row_first.p, enlocal, d_ipnum.p, d_ipent.p, rowstride,
                           d_site_x.p, t, e, d_erho.p, s);
      launch_copy_root(d_erho.p, NPE, d_eroot.p, enlocal, enghost, s);
      fp64_fma::site_fp_needed(d_erho.p, d_etype.p, d_site_base.p, d_need.p, d_need_elem.p, nneed, t,
                               e, d_site_fp.p, s);
    }
    int nb = thermo::partial_blocks(nforce);
    d_part.ensure((size_t) std::max(nb, thermo::partial_blocks((long long) enlocal * NPE)) * 7, s);
    // elements carry one species: the 1-1 pair coefficients (pair_lj_cut.cpp:295-330)
    const int T = (MAXT + 1) * (MAXT + 1), a = 1 * (MAXT + 1) + 1;
    double l5[5] = {0, 0, 0, 0, 0};
    if (pair_style == 1)
      for (int k = 0; k < 5; k++) l5[k] = h_lj5[(size_t) k * T + a];
    thermo::ip(d_nodex.p, d_erho.p, d_etype.p, d_row_elem.p, d_row_jj.p, d_force_rows.p, nforce,
               d_ipnum.p, d_ipent.p, rowstride, d_site_x.p, d_site_fp.p, t, e, pair_style == 2,
               l5[0], l5[1], l5[2], l5[3], l5[4], d_part.p, s);
    for (double &v : q) v = 0.0;
    reduce(nb, q);
    out[1] = q[0];
    for (int k = 0; k < 6; k++) out[4 + k] += q[1 + k];
    nb = thermo::partial_blocks((long long) enlocal * NPE);
    thermo::kinetic(d_nodev.p, d_etype.p, d_emass.p, enlocal * NPE, NPE, 1.0 / NPE, d_part.p, s);
    for (double &v : q) v = 0.0;
    reduce(nb, q);
    out[3] = q[0] * mvv2e;
    for (int k = 0; k < 6; k++) out[10 + k] += q[1 + k] * mvv2e;
  }
  out[16] = prd[0] * prd[1] * prd[2];
}

// ------------------------------------------------------------------ integrate

// FixNVE's dtfm = dtf / mass per atom type, and dtf / (M_e / 8) per element
// type (fix_nve.cpp:54-157), formed on the host: the same IEEE quotients
void cacg_context::nve_scales(TypeScale &a, TypeScale &e) const {
  const double dtf = 0.5 * dt * ftm2v;
  const double inv_npe = 1 / (double) NPE;
  for (int t = 0; t <= MAXT; t++) {
    a.v[t] = up_mass[t] != 0.0 ? dtf / up_mass[t] : 0.0;
    e.v[t] = up_emass[t] != 0.0 ? dtf / (inv_npe * up_emass[t]) : 0.0;
  }
}

void cacg_context::nve_initial(int which) {
  TypeScale a, e;
  nve_scales(a, e);
  if (which & 1) {
    launch_nve_atoms_initial(d_x.p, d_v.p, d_f.p, d_type.p, a, nlocal, dt, fast(), stream);
    launches++;
  }
  if (which & 2) {
    launch_nve_nodes_initial(d_ex.p, d_nodex.p, d_nodev.p, d_nodef.p, d_etype.p, e, enlocal, dt, fast(),
                             stream);
    launches++;
  }
}

// the nodes' second half-step of elements [b0, b1)
void cacg_context::nve_nodes_final_range(int b0, int b1) {
  TypeScale a, e;
  nve_scales(a, e);
  launch_nve_nodes_final(d_nodev.p + 24 * (size_t) b0, d_nodef.p + 24 * (size_t) b0,
                         d_etype.p + b0, e, b1 - b0, fast(), stream);
  launches++;
}

void cacg_context::nve_final(int which) {
  TypeScale a, e;
  nve_scales(a, e);
  if (which & 1) {
    launch_nve_atoms_final(d_v.p, d_f.p, d_type.p, a, nlocal, fast(), stream);
    launches++;
  }
  if (which & 2) {
    launch_nve_nodes_final(d_nodev.p, d_nodef.p, d_etype.p, e, enlocal, fast(), stream);
    launches++;
  }
}

// Neighbor::decide (neighbor.cpp:1150-1163); ago counts steps since setup and
// is not reset by a rebuild, as in the reference
int cacg_context::decide() {
  ago++;
  if (ago >= delay && ago % every == 0) {
    host_decisions++;
    if (dist_check == 0) return 1;
    d_misc.ensure(32, stream);
    check(cudaMemsetAsync(d_misc.p + 6, 0, sizeof(int), stream), "memset");
    BoxWrap box{};
    for (int d = 0; d < 3; d++) {
      box.lo[d] = lo[d];
      box.hi[d] = hi[d];
      box.periodic[d] = periodic[d];
    }
    launch_check_distance(d_x.p, d_xhold.p, nlocal, d_nodex.p, d_nodexhold.p, enlocal,
                          enlocal ? d_ex.p : nullptr, box, triggersq, d_misc.p + 6, stream);
    launches++;
    check(cudaMemcpyAsync(h_pin + 6, d_misc.p + 6, sizeof(int), cudaMemcpyDeviceToHost, stream), "flag");
    sync();
    // a wrap alone needs no rebuild (the reference's check tests distances only)
    return (h_pin[6] & 3) ? h_pin[6] : 0;
  }
  return 0;
}

// atoms that left the packed-coordinate range of the mixed atom passes
void cacg_context::check_packed_range() {
  if (mode != CACG_MIXED || !d_misc.p || !oob_zeroed) return;
  check(cudaMemcpyAsync(h_pin + 9, d_misc.p + 9, sizeof(int), cudaMemcpyDeviceToHost, stream), "oob");
  sync();
  if (h_pin[9]) {
    int n = h_pin[9];
    check(cudaMemsetAsync(d_misc.p + 9, 0, sizeof(int), stream), "oob reset");
    fail(CACG_EINVAL, "%d atoms or element sites outside the packed-coordinate range of the mixed passes", n);
  }
}

// A rebuild (Verlet::run's reneighbor branch, verlet.cpp:184-198).  flags are
// decide()'s bits: with the element lists lazy, a rebuild that atoms alone
// triggered (bit 1 without bits 2 and 4), in a fixed box, re-bins and re-lists
// the atoms and keeps the element lists, element ghosts and cutoffs.
void cacg_context::rebuild(int flags) {
  check_packed_range();
  nrebuild++;
  invalidate_graph();
  if (!rb_ev[0]) {
    check(cudaEventCreate(&rb_ev[0]), "event");
    check(cudaEventCreate(&rb_ev[1]), "event");
  }
  check(cudaEventRecord(rb_ev[0], stream), "event record");
  const bool atoms_only = lazy_elists && mode != CACG_FP64_EXACT && !deform_on && elists_built &&
                          enlocal > 0 && (flags & 6) == 0;
  if (atoms_only) {
    nrebuild_atoms++;
    launch_pbc_atoms(d_x.p, nlocal, lo, hi, prd, periodic, stream);
    launches++;
    borders_atoms();
    if (nlocal) neighbor_build();
  } else {
    pbc();
    if (enlocal) element_size();
    setup_cut();
    comm_setup();
    setup_bins();
    borders();
    if (nlocal) neighbor_build();
    if (enlocal) {
      neighbor_ebuild();
      neighbor_nbuild();
    }
  }
  check(cudaEventRecord(rb_ev[1], stream), "event record");
  check(cudaEventSynchronize(rb_ev[1]), "event sync");
  float ms = 0.f;
  check(cudaEventElapsedTime(&ms, rb_ev[0], rb_ev[1]), "elapsed");
  rebuild_ms_total += ms;
}

void cacg_context::setup() {
  require_init();
  invalidate_graph();
  // Verlet::setup wraps positions first (domain->pbc before comm->setup): a
  // set-up after steps finds atoms and elements back inside the periodic box
  if (ran) pbc();
  comm_setup();
  setup_bins();
  borders();
  ago = 0;
  setup_done = true;
  list_built = elists_built = false;
}

void cacg_context::run(int n) {
  if (n < 0) fail(CACG_EINVAL, "Illegal run command");
  if (!setup_done) setup();
  if (!list_built) neighbor_build();
  if (!elists_built && enlocal) {
    neighbor_ebuild();
    neighbor_nbuild();
  }
  if (!fix_nve) fail(CACG_ESTATE, "run without fix nve");
  ran = ran || n > 0;
  for (int k = 0; k < 8; k++) t_ms[k] = 0.0;
  for (int k = 0; k < KT_N; k++) t_kern[k] = 0.0;
  std::fill(pev_used.begin(), pev_used.end(), 0);
  for (auto &e : ev)
    if (!e) check(cudaEventCreate(&e), "event");
  check(cudaEventRecord(ev[0], stream), "ev");
  const size_t P = 6;  // phase marks per step
  std::fill(kev_used.begin(), kev_used.end(), 0);
  cur_step = 0;
  for (int step = 0; step < n; step++) {
    // the device loop runs the steps it can; it hands back a step that must
    // run here first (after set-up or a rebuild: first-call allocations and
    // read-backs stay outside the capture), and all steps once its capture
    // has failed
    if (loop_device && use_graphs && graph_ok && !deform_on) {
      const int k = run_loop(n - step);
      if (k > 0) {
        step += k - 1;
        continue;
      }
    }
    size_t b = (size_t) step * P;
    cur_step = (size_t) step;
    ntimestep++;
    // a step that reaches no rebuild decision (Neighbor::decide returns 0
    // without checking) replays the captured graph of the previous such step
    const bool plain = !(ago + 1 >= delay && (ago + 1) % every == 0);
    if (plain && use_graphs && graph_ok && !deform_on) {
      ago++;
      if (graph_valid && graph_epoch == dbuf_epoch()) {
        check(cudaGraphLaunch(gexec, stream), "graph launch");
        launches += graph_launches;
        graph_steps++;
        continue;
      }
      if (eager_since >= 1 && capture_plain_step()) {
        check(cudaGraphLaunch(gexec, stream), "graph launch");
        launches += graph_launches;
        graph_steps++;
        continue;
      }
      mark(b);
      if (fork_ok()) {
        const bool nodes_done = post_fixes.empty();
        forked(
            [&] {
              nve_initial(1);
              forward_comm(1);
              pair_compute_pass(1);
              pair_compute_pass(2);
            },
            [&] {
              nve_initial(2);
              forward_comm(2);
              pair_ecompute();
              if (nodes_done) nve_final(2);  // no fix acts on the forces in between
            });
        post_force();
        nve_final(nodes_done ? 1 : 3);
      } else {
        nve_initial();
        forward_comm();
        mark(b + 1);
        force_passes((long long) b);
        post_force();
        mark(b + 4);
        nve_final();
        mark(b + 5);
      }
      eager_since++;
      continue;
    }
    mark(b);
    nve_initial();
    int nflag = decide();
    if (nflag == 0) forward_comm();
    else rebuild(nflag);
    mark(b + 1);
    force_passes((long long) b);
    post_force();  // verlet.cpp:206
    mark(b + 4);
    nve_final();
    deform_step();
    mark(b + 5);
    if (nflag == 0) eager_since++;  // every pass of a plain step has run eagerly
  }
  // the packed-range counter is read back behind the last step, so that one
  // synchronisation serves both
  const bool oob_read = mode == CACG_MIXED && d_misc.p && oob_zeroed;
  if (oob_read)
    check(cudaMemcpyAsync(h_pin + 9, d_misc.p + 9, sizeof(int), cudaMemcpyDeviceToHost, stream), "oob");
  check(cudaEventRecord(ev[1], stream), "ev");
  check(cudaEventSynchronize(ev[1]), "ev sync");
  if (oob_read && h_pin[9]) {
    const int nout = h_pin[9];
    check(cudaMemsetAsync(d_misc.p + 9, 0, sizeof(int), stream), "oob reset");
    fail(CACG_EINVAL, "%d atoms or element sites outside the packed-coordinate range of the mixed passes", nout);
  }
  float ms = 0;
  cudaEventElapsedTime(&ms, ev[0], ev[1]);
  t_ms[0] = ms;
  if (timing && n > 0) {
    for (int step = 0; step < n; step++) {
      size_t b = (size_t) step * P;
      for (size_t k = 0; k < P - 1; k++) {
        float d = 0;
        if (b + k + 1 >= pev.size() || !pev_used[b + k] || !pev_used[b + k + 1]) continue;
        check(cudaEventElapsedTime(&d, pev[b + k], pev[b + k + 1]), "elapsed");
        t_ms[1 + k] += d;
      }
      // the main kernels alone; [6]: the atom pass-1 kernel
      for (int k = 0; k < KT_N; k++) {
        const size_t kb = 2 * ((size_t) step * KT_N + (size_t) k);
        float d = 0;
        if (kb + 1 < kev.size() && kev_used[kb] && kev_used[kb + 1]) {
          check(cudaEventElapsedTime(&d, kev[kb], kev[kb + 1]), "elapsed");
          t_kern[k] += d;
        }
      }
      t_ms[6] = t_kern[KT_ATOM1];
    }
  }
  cur_step = 0;
}

// The atom chain and the element chain of a mixed step, from this point on the
// handle's stream: the atom chain on a second stream of higher priority (it is
// the longer one), the element chain on the handle's stream, which waits for
// the atom chain before its next operation.  Both streams take part in a
// graph capture of the handle's stream.
template <class A, class E>
void cacg_context::forked(A atoms, E elems, bool elems_first) {
  if (!astream) {
    int least = 0, greatest = 0;
    check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    check(cudaStreamCreateWithPriority(&astream, cudaStreamNonBlocking, greatest), "atom stream");
  }
  if (!fork_ev) check(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming), "fork event");
  if (!join_ev) check(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming), "join event");
  check(cudaEventRecord(fork_ev, stream), "fork");
  check(cudaStreamWaitEvent(astream, fork_ev, 0), "fork wait");
  const cudaStream_t main_stream = stream;
  auto atom_chain = [&] {
    stream = astream;
    try {
      atoms();
    } catch (...) {
      stream = main_stream;
      cudaEventRecord(join_ev, astream);
      cudaStreamWaitEvent(stream, join_ev, 0);
      throw;
    }
    stream = main_stream;
    check(cudaEventRecord(join_ev, astream), "join");
  };
  // the chain enqueued first is the one whose kernels the device can start first
  if (elems_first) {
    try {
      elems();
    } catch (...) {
      cudaEventRecord(join_ev, astream);
      cudaStreamWaitEvent(stream, join_ev, 0);
      throw;
    }
    atom_chain();
  } else {
    atom_chain();
    try {
      elems();
    } catch (...) {
      cudaStreamWaitEvent(stream, join_ev, 0);
      throw;
    }
  }
  check(cudaStreamWaitEvent(stream, join_ev, 0), "join wait");
}

// Pair::compute for atoms (density, then force pass) and Pair::ecompute for
// elements: in order on the handle's stream, marking the phases (b + 2,
// b + 3; b < 0: no marks), or as two chains (forked) when that is on.
void cacg_context::force_passes(long long b) {
  if (fork_ok()) {
    forked(
        [&] {
          pair_compute_pass(1);
          pair_compute_pass(2);
        },
        [&] { pair_ecompute(); });
    return;
  }
  pair_compute_pass(1);
  if (b >= 0) mark((size_t) b + 2);
  pair_compute_pass(2);
  if (b >= 0) mark((size_t) b + 3);
  pair_ecompute();
}

// Host-resident state advanced by n steps: x, v of the owned atoms and nodex,
// nodev of the owned elements are copied in from the caller's buffers, the
// steps run, and the new state is copied back before the call returns.  When
// the last step is a mixed step (two chains), its copies overlap the
// computation.  In a step without a rebuild decision the smaller of the two
// states (atoms or nodes) is copied in first and its chain runs while the
// other is still in flight; outputs start once every input is in (the link
// carries both directions at once, but an early output slows the input the
// other chain waits for): positions as soon as the step's initial
// integration has moved them (nothing later in such a step writes owned
// positions), atom velocities when the atom chain has integrated them, and,
// when no fix acts on the forces, node velocities part by part as the
// element force pass finishes each part of the elements (out_parts).  A step
// with a rebuild decision on distances (no post-force fix) runs its atom
// chain ahead of the host decision and, without a rebuild, goes on as a plain
// step; other decision steps wait for all their inputs.  Positions go out
// after the decision (a rebuild wraps them into the box).  Otherwise the
// copies and the steps run in order.
// Results are those of the same steps run on device-resident state.
void cacg_context::run_host(int n, double *x, double *v, double *nodex, double *nodev) {
  if (n < 1) fail(CACG_EINVAL, "run_host: at least one step");
  require_init();
  if ((nlocal && (!x || !v)) || (enlocal && (!nodex || !nodev)))
    fail(CACG_EINVAL, "run_host: null state buffer");
  if (!fix_nve) fail(CACG_ESTATE, "run without fix nve");
  d_stage.ensure(3 * (size_t) std::max(nlocal, 1), stream);
  const long long ago_last = (long long) ago + n - 1;
  const bool last_plain = !(ago_last + 1 >= delay && (ago_last + 1) % every == 0);
  const bool overlap = fork_ok() && setup_done && list_built && elists_built && !deform_on;
  const size_t xb = sizeof(double) * 3 * (size_t) nlocal, nb = sizeof(double) * 24 * (size_t) enlocal;
  if (!overlap) {
    cudaStream_t s = stream;
    if (nlocal) {
      check(cudaMemcpyAsync(d_stage.p, x, xb, cudaMemcpyHostToDevice, s), "x in");
      launch_pack3to4(d_stage.p, d_x.p, nlocal, s);
      check(cudaMemcpyAsync(d_v.p, v, xb, cudaMemcpyHostToDevice, s), "v in");
    }
    if (enlocal) {
      check(cudaMemcpyAsync(d_nodex.p, nodex, nb, cudaMemcpyHostToDevice, s), "nodex in");
      check(cudaMemcpyAsync(d_nodev.p, nodev, nb, cudaMemcpyHostToDevice, s), "nodev in");
    }
    run(n);
    if (nlocal) {
      launch_unpack4to3(d_x.p, d_stage.p, nlocal, s);
      check(cudaMemcpyAsync(x, d_stage.p, xb, cudaMemcpyDeviceToHost, s), "x out");
      check(cudaMemcpyAsync(v, d_v.p, xb, cudaMemcpyDeviceToHost, s), "v out");
    }
    if (enlocal) {
      check(cudaMemcpyAsync(nodex, d_nodex.p, nb, cudaMemcpyDeviceToHost, s), "nodex out");
      check(cudaMemcpyAsync(nodev, d_nodev.p, nb, cudaMemcpyDeviceToHost, s), "nodev out");
    }
    sync();
    return;
  }
  if (!cin) check(cudaStreamCreateWithFlags(&cin, cudaStreamNonBlocking), "copy-in stream");
  if (!cout_s) check(cudaStreamCreateWithFlags(&cout_s, cudaStreamNonBlocking), "copy-out stream");
  for (cudaEvent_t *e : {&ev_ain, &ev_nin, &ev_xout, &ev_nxout, &ev_nvout, &ev_end, &ev_hstart,
                         &ev_hdone, &ev_vout, &ev_acheck, &ev_apass})
    if (!*e) check(cudaEventCreateWithFlags(e, cudaEventDisableTiming), "copy event");
  for (cudaEvent_t &e : ev_nvpart)
    if (!e) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "copy event");
  const bool early_nodes = last_plain && post_fixes.empty();
  // a step with a rebuild decision on distances runs its atom chain ahead of the
  // decision (see below)
  const bool ahead = !last_plain && dist_check != 0 && post_fixes.empty();
  const bool oob_read = d_misc.p && oob_zeroed;
  // the smaller state goes in first: its chain starts while the other's is in
  // flight (the link moves ~0.2 TB/s each way, a step's state in is ~1 ms)
  const bool atoms_first = xb <= nb;
  // inputs, the last step with the copies hooked in, outputs; the copy
  // streams fork from the handle's stream and join it again, so the whole
  // call can be captured as one graph
  auto body = [&](bool pending) {
    check(cudaEventRecord(ev_hstart, stream), "host step start");
    check(cudaStreamWaitEvent(cin, ev_hstart, 0), "copy-in fork");
    check(cudaStreamWaitEvent(cout_s, ev_hstart, 0), "copy-out fork");
    if (pending) {
      auto nodes_in = [&] {
        check(cudaMemcpyAsync(d_nodex.p, nodex, nb, cudaMemcpyHostToDevice, cin), "nodex in");
        check(cudaMemcpyAsync(d_nodev.p, nodev, nb, cudaMemcpyHostToDevice, cin), "nodev in");
        check(cudaEventRecord(ev_nin, cin), "nodes in");
      };
      auto atoms_in = [&] {
        check(cudaMemcpyAsync(d_stage.p, x, xb, cudaMemcpyHostToDevice, cin), "x in");
        check(cudaMemcpyAsync(d_v.p, v, xb, cudaMemcpyHostToDevice, cin), "v in");
        check(cudaEventRecord(ev_ain, cin), "atoms in");
      };
      if (atoms_first) {
        atoms_in();
        nodes_in();
      } else {
        nodes_in();
        atoms_in();
      }
    } else {
      check(cudaEventRecord(ev_ain, cin), "no inputs");
      check(cudaEventRecord(ev_nin, cin), "no inputs");
    }
    ran = true;
    ntimestep++;
    bool early = early_nodes;  // velocities out as each chain integrates them
    if (ahead) {
      // Neighbor::decide (neighbor.cpp:1150-1163) on this step's integrated
      // positions, with the atom chain run ahead of it: the atoms' initial
      // integration and distance check, then their ghost update and force
      // passes, go on while the node state is still in flight and the host
      // waits for the two checks (the main stream only).  Without a rebuild
      // the step goes on as a plain one; with one, the atoms' ghost update
      // and forces are discarded (the rebuild re-makes the ghosts, the lists
      // and every force), so the trajectory is the one decide() gives.
      ago++;
      host_decisions++;
      d_misc.ensure(32, stream);
      check(cudaMemsetAsync(d_misc.p + 6, 0, sizeof(int), stream), "memset");
      BoxWrap box{};
      for (int d = 0; d < 3; d++) {
        box.lo[d] = lo[d];
        box.hi[d] = hi[d];
        box.periodic[d] = periodic[d];
      }
      if (!astream) forked([] {}, [] {});  // creates the atom stream and its events
      check(cudaEventRecord(fork_ev, stream), "fork");
      check(cudaStreamWaitEvent(astream, fork_ev, 0), "fork wait");
      const cudaStream_t main_stream = stream;
      stream = astream;
      try {
        check(cudaStreamWaitEvent(stream, ev_ain, 0), "wait atoms in");
        if (pending) {
          launch_pack3to4(d_stage.p, d_x.p, nlocal, stream);
          launches++;
        }
        nve_initial(1);
        launch_check_distance(d_x.p, d_xhold.p, nlocal, nullptr, nullptr, 0, nullptr, box,
                              triggersq, d_misc.p + 6, stream);
        check(cudaEventRecord(ev_acheck, stream), "atom check");
        forward_comm(1);
        pair_compute_pass(1);
        pair_compute_pass(2);
        check(cudaEventRecord(ev_apass, stream), "atom passes");
      } catch (...) {
        stream = main_stream;
        throw;
      }
      stream = main_stream;
      check(cudaStreamWaitEvent(stream, ev_nin, 0), "wait nodes in");
      nve_initial(2);
      launch_check_distance(nullptr, nullptr, 0, d_nodex.p, d_nodexhold.p, enlocal,
                            enlocal ? d_ex.p : nullptr, box, triggersq, d_misc.p + 6, stream);
      check(cudaStreamWaitEvent(stream, ev_acheck, 0), "wait atom check");
      check(cudaMemcpyAsync(h_pin + 6, d_misc.p + 6, sizeof(int), cudaMemcpyDeviceToHost, stream),
            "flag");
      launches += 2;
      sync();
      // a wrap alone needs no rebuild (the reference's check tests distances only)
      const int nflag = (h_pin[6] & 3) ? h_pin[6] : 0;
      check(cudaEventRecord(ev_xout, stream), "x final");  // (after the decision)
      check(cudaEventRecord(ev_nxout, stream), "nodex final");
      if (nflag == 0) {
        early = true;
        forward_comm(2);
        out_split = true;
        parts_done = 1;
        try {
          pair_ecompute();
        } catch (...) {
          out_split = false;
          throw;
        }
        out_split = false;
        if (parts_done > 1) nve_nodes_final_range(part_bounds[parts_done - 1], enlocal);
        else nve_final(2);
        check(cudaEventRecord(ev_nvout, stream), "nodev final");
        stream = astream;
        try {
          nve_final(1);
          check(cudaEventRecord(ev_vout, stream), "v final");
          check(cudaEventRecord(join_ev, stream), "join");
        } catch (...) {
          stream = main_stream;
          throw;
        }
        stream = main_stream;
        check(cudaStreamWaitEvent(stream, join_ev, 0), "join wait");
      } else {
        check(cudaStreamSynchronize(astream), "atom chain");
        rebuild(nflag);
        check(cudaEventRecord(ev_xout, stream), "x final");
        check(cudaEventRecord(ev_nxout, stream), "nodex final");
        force_passes(-1);
        post_force();
        nve_final();
      }
    } else if (!last_plain) {
      // Neighbor::decide reads this step's integrated positions on the host,
      // so the step waits for all its inputs; positions go out after the
      // decision (a rebuild wraps them into the box first)
      check(cudaStreamWaitEvent(stream, ev_nin, 0), "wait nodes in");
      check(cudaStreamWaitEvent(stream, ev_ain, 0), "wait atoms in");
      if (pending) {
        launch_pack3to4(d_stage.p, d_x.p, nlocal, stream);
        launches++;
      }
      nve_initial();
      const int nflag = decide();
      if (nflag == 0) forward_comm();
      else rebuild(nflag);
      check(cudaEventRecord(ev_xout, stream), "x final");
      check(cudaEventRecord(ev_nxout, stream), "nodex final");
      force_passes(-1);
      post_force();
      nve_final();
    } else {
      ago++;
      forked(
          [&] {
            check(cudaStreamWaitEvent(stream, ev_ain, 0), "wait atoms in");
            if (pending) {
              launch_pack3to4(d_stage.p, d_x.p, nlocal, stream);
              launches++;
            }
            nve_initial(1);
            check(cudaEventRecord(ev_xout, stream), "x final");
            forward_comm(1);
            pair_compute_pass(1);
            pair_compute_pass(2);
            if (early_nodes) {  // the atoms' velocities go out while the elements run
              nve_final(1);
              check(cudaEventRecord(ev_vout, stream), "v final");
            }
          },
          [&] {
            check(cudaStreamWaitEvent(stream, ev_nin, 0), "wait nodes in");
            nve_initial(2);
            check(cudaEventRecord(ev_nxout, stream), "nodex final");
            forward_comm(2);
            out_split = early_nodes;
            parts_done = 1;
            try {
              pair_ecompute();
            } catch (...) {
              out_split = false;
              throw;
            }
            out_split = false;
            if (early_nodes) {  // no fix acts between the force passes and the integration
              if (parts_done > 1) nve_nodes_final_range(part_bounds[parts_done - 1], enlocal);
              else nve_final(2);
              check(cudaEventRecord(ev_nvout, stream), "nodev final");
            }
          },
          true);
      if (!early_nodes) {
        post_force();
        nve_final();
        check(cudaEventRecord(ev_vout, stream), "v final");
      }
      eager_since++;
    }
    check(cudaEventRecord(ev_end, stream), "step end");
    // outputs, once the inputs are in (an early output would share the link
    // with the inputs the element chain waits for)
    check(cudaStreamWaitEvent(cout_s, ev_ain, 0), "wait atoms in");
    check(cudaStreamWaitEvent(cout_s, ev_nin, 0), "wait nodes in");
    check(cudaStreamWaitEvent(cout_s, ev_xout, 0), "wait x final");
    launch_unpack4to3(d_x.p, d_stage.p, nlocal, cout_s);
    check(cudaMemcpyAsync(x, d_stage.p, xb, cudaMemcpyDeviceToHost, cout_s), "x out");
    check(cudaStreamWaitEvent(cout_s, ev_nxout, 0), "wait nodex final");
    check(cudaMemcpyAsync(nodex, d_nodex.p, nb, cudaMemcpyDeviceToHost, cout_s), "nodex out");
    auto v_out = [&] {
      check(cudaStreamWaitEvent(cout_s, last_plain || early ? ev_vout : ev_end, 0), "wait v final");
      check(cudaMemcpyAsync(v, d_v.p, xb, cudaMemcpyDeviceToHost, cout_s), "v out");
    };
    // the chain that ends first has its velocities copied first: the atoms'
    // when their state went in first
    if (!early || atoms_first) v_out();
    if (early) {
      for (int p = 0; p < parts_done; p++) {
        const size_t b0 = 24 * (size_t) (parts_done > 1 ? part_bounds[p] : 0);
        const size_t b1 = 24 * (size_t) (p + 1 < parts_done ? part_bounds[p + 1] : enlocal);
        check(cudaStreamWaitEvent(cout_s, p + 1 < parts_done ? ev_nvpart[p] : ev_nvout, 0),
              "wait nodev final");
        check(cudaMemcpyAsync(nodev + b0, d_nodev.p + b0, sizeof(double) * (b1 - b0),
                              cudaMemcpyDeviceToHost, cout_s),
              "nodev out");
      }
      if (!atoms_first) v_out();
    }
    check(cudaStreamWaitEvent(cout_s, ev_end, 0), "wait step end");
    if (!early)
      check(cudaMemcpyAsync(nodev, d_nodev.p, nb, cudaMemcpyDeviceToHost, cout_s), "nodev out");
    if (oob_read)
      check(cudaMemcpyAsync(h_pin + 9, d_misc.p + 9, sizeof(int), cudaMemcpyDeviceToHost, cout_s),
            "oob");
    check(cudaEventRecord(ev_hdone, cout_s), "copies out");
    check(cudaStreamWaitEvent(stream, ev_hdone, 0), "copy-out join");
  };
  auto finish = [&] {
    check(cudaStreamSynchronize(stream), "host step");
    if (oob_read && h_pin[9]) {
      const int nout = h_pin[9];
      check(cudaMemsetAsync(d_misc.p + 9, 0, sizeof(int), stream), "oob reset");
      fail(CACG_EINVAL, "%d atoms or element sites outside the packed-coordinate range of the mixed passes", nout);
    }
  };
  // A single plain step on pinned buffers replays a graph of the whole call
  // (copies, both chains, copies back), captured after an eager step on the
  // same buffers and dropped like the step graph (rebuild, command,
  // reallocation); other buffers run eagerly until they too are reused.
  auto pinned = [](const void *p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    return at.type == cudaMemoryTypeHost;
  };
  const void *bufs[4] = {x, v, nodex, nodev};
  const bool same_bufs = std::equal(bufs, bufs + 4, hlast_bufs);
  std::copy(bufs, bufs + 4, hlast_bufs);
  const bool graphable = n == 1 && last_plain && use_graphs && hgraph_ok && pinned(x) &&
                         pinned(v) && pinned(nodex) && pinned(nodev);
  if (graphable && hgraph_valid && hgraph_epoch == dbuf_epoch() &&
      std::equal(bufs, bufs + 4, hgraph_bufs)) {
    ran = true;
    ntimestep++;
    ago++;
    eager_since++;
    launches += hgraph_launches;
    check(cudaGraphLaunch(hexec, stream), "host step graph");
    graph_steps++;
    finish();
    return;
  }
  if (graphable && eager_since >= 1 && same_bufs) {  // buffers reused: worth a capture
    const long long l0 = launches, ts0 = ntimestep;
    const int ago0 = ago, es0 = eager_since;
    const unsigned long long e0 = dbuf_epoch();
    bool ok = cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      capturing = true;
      try {
        body(true);
      } catch (...) {
        ok = false;
      }
      capturing = false;
      cudaGraph_t g = nullptr;
      if (cudaStreamEndCapture(stream, &g) != cudaSuccess || !g || dbuf_epoch() != e0) ok = false;
      cudaGraphExec_t ex = nullptr;
      if (ok && cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) ok = false;
      if (g) cudaGraphDestroy(g);
      cudaGetLastError();  // a failed capture leaves its error behind
      if (ok) {
        if (hexec) cudaGraphExecDestroy(hexec);
        hexec = ex;
        hgraph_launches = launches - l0;
        hgraph_epoch = e0;
        std::copy(bufs, bufs + 4, hgraph_bufs);
        hgraph_valid = true;
        check(cudaGraphLaunch(hexec, stream), "host step graph");
        graph_steps++;
        finish();
        return;
      }
      if (ex) cudaGraphExecDestroy(ex);
    } else {
      cudaGetLastError();
    }
    // the capture failed: the step runs eagerly, and graphs of this call stay off
    hgraph_ok = false;
    launches = l0;
    ntimestep = ts0;
    ago = ago0;
    eager_since = es0;
  }
  bool pending = true;
  if (n > 1) {
    // the inputs, then the steps before the last one, in order
    check(cudaEventRecord(ev_hstart, stream), "host steps start");
    check(cudaStreamWaitEvent(cin, ev_hstart, 0), "copy-in fork");
    check(cudaMemcpyAsync(d_nodex.p, nodex, nb, cudaMemcpyHostToDevice, cin), "nodex in");
    check(cudaMemcpyAsync(d_nodev.p, nodev, nb, cudaMemcpyHostToDevice, cin), "nodev in");
    check(cudaMemcpyAsync(d_stage.p, x, xb, cudaMemcpyHostToDevice, cin), "x in");
    check(cudaMemcpyAsync(d_v.p, v, xb, cudaMemcpyHostToDevice, cin), "v in");
    check(cudaEventRecord(ev_ain, cin), "inputs in");
    check(cudaStreamWaitEvent(stream, ev_ain, 0), "wait inputs");
    launch_pack3to4(d_stage.p, d_x.p, nlocal, stream);
    launches++;
    pending = false;
    run(n - 1);
  }
  body(pending);
  finish();
}

// The device step loop: a WHILE node whose body is a step's initial
// integration, the gated distance check and the decision kernel, then an IF
// node around the step's communication, force passes, post-force fixes and
// final integration (the body of a plain step).  The decision kernel sets
// both conditions.  Anything that would allocate or synchronise ends a
// capture with an error; the steps then run the host way and the device loop
// stays off for this handle.
// Prepares the handle for a loop capture: masks uploaded, the loop state and
// the second chain's stream allocated (nothing of this may happen inside a
// capture).
void cacg_context::loop_prepare() {
  upload_masks();
  d_loop.ensure(LOOP_SLOTS, stream);
  if (!astream && fork_ok()) {
    int least = 0, greatest = 0;
    check(cudaDeviceGetStreamPriorityRange(&least, &greatest), "stream priorities");
    check(cudaStreamCreateWithPriority(&astream, cudaStreamNonBlocking, greatest), "atom stream");
  }
}

// Adds this handle's step loop to `top` as one WHILE node (see capture_loop);
// pre / post: the kernels of an iteration before and after the decision.  A
// capture into a conditional body that ends invalidated may leave that body
// released by the runtime while its node still refers to it: *destroyable is
// then cleared and the caller leaves the whole graph alone.
bool cacg_context::add_loop(cudaGraph_t top, long long &pre, long long &post, bool *destroyable) {
  const long long l0 = launches;
  cudaGraphConditionalHandle again = 0, proceed = 0;
  cudaGraph_t body = nullptr, then = nullptr;
  bool ok = cudaGraphConditionalHandleCreate(&again, top, 1, cudaGraphCondAssignDefault) == cudaSuccess;
  if (ok) {
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = again;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node = nullptr;
    ok = cudaGraphAddNode(&node, top, nullptr, nullptr, 0, &p) == cudaSuccess;
    if (ok) body = p.conditional.phGraph_out[0];
  }
  ok = ok && cudaGraphConditionalHandleCreate(&proceed, body, 0, 0) == cudaSuccess;
  capturing = true;
  // the step up to the decision
  if (ok && cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    std::vector<cudaGraphNode_t> leaves;
    try {
      nve_initial();
      if (dist_check) {
        BoxWrap box{};
        for (int d = 0; d < 3; d++) {
          box.lo[d] = lo[d];
          box.hi[d] = hi[d];
          box.periodic[d] = periodic[d];
        }
        launch_loop_check(d_x.p, d_xhold.p, nlocal, d_nodex.p, d_nodexhold.p, enlocal,
                          enlocal ? d_ex.p : nullptr, box, triggersq, d_loop.p, every, delay, stream);
        launches++;
      }
      launch_loop_decide(d_loop.p, every, delay, dist_check, again, proceed, stream);
      launches++;
      cudaStreamCaptureStatus st;
      const cudaGraphNode_t *deps = nullptr;
      size_t nd = 0;
      if (cudaStreamGetCaptureInfo(stream, &st, nullptr, nullptr, &deps, nullptr, &nd) != cudaSuccess)
        ok = false;
      else
        leaves.assign(deps, deps + nd);
    } catch (...) {
      ok = false;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(stream, &g) != cudaSuccess) ok = *destroyable = false;
    pre = launches - l0;
    if (ok) {
      cudaGraphNodeParams p = {};
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = proceed;
      p.conditional.type = cudaGraphCondTypeIf;
      p.conditional.size = 1;
      cudaGraphNode_t node = nullptr;
      ok = cudaGraphAddNode(&node, body, leaves.data(), nullptr, leaves.size(), &p) == cudaSuccess;
      if (ok) then = p.conditional.phGraph_out[0];
    }
  } else {
    ok = false;
  }
  // the rest of the step, as a plain step runs it
  if (ok && cudaStreamBeginCaptureToGraph(stream, then, nullptr, nullptr, 0,
                                          cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
    const long long l1 = launches;
    try {
      if (fork_ok()) {
        const bool nodes_done = post_fixes.empty();
        forked(
            [&] {
              forward_comm(1);
              pair_compute_pass(1);
              pair_compute_pass(2);
            },
            [&] {
              forward_comm(2);
              pair_ecompute();
              if (nodes_done) nve_final(2);
            });
        post_force();
        nve_final(nodes_done ? 1 : 3);
      } else {
        forward_comm();
        force_passes(-1);
        post_force();
        nve_final();
      }
    } catch (...) {
      ok = false;
    }
    cudaGraph_t g = nullptr;
    if (cudaStreamEndCapture(stream, &g) != cudaSuccess) ok = *destroyable = false;
    post = launches - l1;
  } else {
    ok = false;
  }
  capturing = false;
  launches = l0;
  cudaGetLastError();  // a failed capture leaves its error behind
  return ok;
}

// The device step loop: a WHILE node whose body is a step's initial
// integration, the gated distance check and the decision kernel, then an IF
// node around the step's communication, force passes, post-force fixes and
// final integration (the body of a plain step).  The decision kernel sets
// both conditions.  Anything that would allocate or synchronise ends a
// capture with an error; the steps then run the host way and the device loop
// stays off for this handle.
bool cacg_context::capture_loop() {
  loop_prepare();
  const unsigned long long e0 = dbuf_epoch();
  cudaGraph_t top = nullptr;
  cudaGraphExec_t ex = nullptr;
  long long pre = 0, post = 0;
  bool destroyable = true;
  bool ok = cudaGraphCreate(&top, 0) == cudaSuccess && add_loop(top, pre, post, &destroyable);
  if (ok && dbuf_epoch() != e0) ok = false;
  if (ok && cudaGraphInstantiate(&ex, top, 0) != cudaSuccess) ok = false;
  if (top && destroyable) cudaGraphDestroy(top);
  cudaGetLastError();
  if (!ok) {
    if (ex) cudaGraphExecDestroy(ex);
    loop_device = false;
    return false;
  }
  if (lexec) cudaGraphExecDestroy(lexec);
  lexec = ex;
  lgraph_pre = pre;
  lgraph_post = post;
  lgraph_epoch = e0;
  lgraph_valid = true;
  return true;
}

// The loop state of a launch that wanted `want` steps, into the pinned slots
// (before the launch), and its outcome (after it): the steps done are
// accounted, and a step that needs a rebuild is rebuilt and finished here.
// Returns the steps taken, that one included.
void cacg_context::loop_arm(int want) {
  int *hl = h_pin + 16;
  hl[LOOP_AGO] = ago;
  hl[LOOP_DONE] = 0;
  hl[LOOP_WANT] = want;
  hl[LOOP_PENDING] = 0;
  hl[LOOP_ITERS] = 0;
  hl[LOOP_BITS] = 0;
}

int cacg_context::loop_finish(int want, long long pre, long long post) {
  const int *hl = h_pin + 16;
  loop_launches++;
  const int steps = hl[LOOP_DONE], iters = hl[LOOP_ITERS], flags = hl[LOOP_PENDING];
  if (steps < 0 || steps > want || iters < steps || iters > steps + 1)
    fail(CACG_ECUDA, "device step loop: %d steps in %d iterations of %d wanted", steps, iters, want);
  ago = hl[LOOP_AGO];
  ntimestep += steps;
  graph_steps += steps;
  launches += pre * iters + post * steps;
  if (flags) {  // the step after those: initial integration and decision done
    ntimestep++;
    cur_step = (size_t) steps;
    rebuild(flags);
    force_passes(-1);
    post_force();
    nve_final();
    return steps + 1;
  }
  if (steps == 0) fail(CACG_ECUDA, "device step loop made no progress");
  return steps;
}

// Up to n steps through the device loop; returns the steps taken.  Each
// launch runs until the wanted steps are done or a step needs a rebuild:
// that step's initial integration and decision ran on the device, the host
// rebuilds and finishes it, and the next launch goes on.  A capture waits for
// one eager step since the last set-up, rebuild or change (fewer steps are
// returned, and the caller runs that step); a failed capture turns the device
// loop off for the handle.
int cacg_context::run_loop(int n) {
  int done = 0;
  int *hl = h_pin + 16;
  while (done < n) {
    if (!lgraph_valid || lgraph_epoch != dbuf_epoch()) {
      if (eager_since < 1 || !capture_loop()) return done;
    }
    loop_arm(n - done);
    check(cudaMemcpyAsync(d_loop.p, hl, LOOP_SLOTS * sizeof(int), cudaMemcpyHostToDevice, stream), "loop in");
    check(cudaGraphLaunch(lexec, stream), "loop launch");
    check(cudaMemcpyAsync(hl, d_loop.p, LOOP_SLOTS * sizeof(int), cudaMemcpyDeviceToHost, stream), "loop out");
    sync();
    done += loop_finish(n - done, lgraph_pre, lgraph_post);
  }
  return done;
}

// The body of a step without a rebuild decision, captured into a CUDA graph.
// Anything that would allocate or synchronise ends the capture with an error;
// the step then runs eagerly and graphs stay off for this handle.
bool cacg_context::capture_plain_step() {
  cudaStream_t s = stream;
  upload_masks();  // host-to-device copies stay outside the capture
  if (cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
    cudaGetLastError();
    graph_ok = false;
    return false;
  }
  const long long l0 = launches;
  const unsigned long long e0 = dbuf_epoch();
  bool ok = true;
  capturing = true;
  try {
    if (fork_ok()) {
      const bool nodes_done = post_fixes.empty();
      forked(
          [&] {
            nve_initial(1);
            forward_comm(1);
            pair_compute_pass(1);
            pair_compute_pass(2);
          },
          [&] {
            nve_initial(2);
            forward_comm(2);
            pair_ecompute();
            if (nodes_done) nve_final(2);  // no fix acts on the forces in between
          });
      post_force();
      nve_final(nodes_done ? 1 : 3);
    } else {
      nve_initial();
      forward_comm();
      force_passes(-1);
      post_force();
      nve_final();
    }
  } catch (...) {
    ok = false;
  }
  capturing = false;
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamEndCapture(s, &g);
  if (e != cudaSuccess || !g || !ok || dbuf_epoch() != e0) ok = false;
  cudaGraphExec_t ex = nullptr;
  if (ok && cudaGraphInstantiate(&ex, g, 0) != cudaSuccess) ok = false;
  if (g) cudaGraphDestroy(g);
  cudaGetLastError();  // a failed capture leaves its error behind
  if (!ok) {
    if (ex) cudaGraphExecDestroy(ex);
    graph_ok = false;
    launches = l0;
    return false;
  }
  if (gexec) cudaGraphExecDestroy(gexec);
  gexec = ex;
  graph_launches = launches - l0;
  launches = l0;
  graph_epoch = dbuf_epoch();
  graph_valid = true;
  return true;
}

// ------------------------------------------------------------------ ABI

#define API_BEGIN                 \
  if (!h) return CACG_EINVAL;     \
  EpochScope epoch_scope_(&h->epoch);  \
  try {                           \
    check(cudaSetDevice(h->device), "cudaSetDevice");
#define API_END                                                              \
  return CACG_OK;                                                            \
  }                                                                          \
  catch (const ApiError &e) {                                                \
    h->err = e.msg;                                                          \
    return e.code;                                                           \
  }                                                                          \
  catch (const CudaError &e) {                                               \
    h->err = std::string(e.where) + ": " + cudaGetErrorString(e.code);       \
    return e.code == cudaErrorMemoryAllocation ? CACG_ENOMEM : CACG_ECUDA;   \
  }

extern "C" {

const char *cacg_version(void) { return "cacg 0.1 (sm_103a)"; }

int cacg_create(cacg_handle *out, int device) {
  if (!out) return CACG_EINVAL;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return CACG_ECUDA;
  if (device < 0 || device >= n) return CACG_EINVAL;
  cacg_context *h = new cacg_context();
  h->device = device;
  if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete h;
    return CACG_ECUDA;
  }
  *out = h;
  return CACG_OK;
}

int cacg_destroy(cacg_handle h) {
  if (!h) return CACG_EINVAL;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  delete h;
  return CACG_OK;
}

const char *cacg_error(cacg_handle h) { return h ? h->err.c_str() : "null handle"; }

int cacg_command(cacg_handle h, const char *line) {
  API_BEGIN
  if (!line) fail(CACG_EINVAL, "null command");
  h->command(line);
  API_END
}

int cacg_file(cacg_handle h, const char *path) {
  API_BEGIN
  std::ifstream in(path ? path : "");
  if (!in) fail(CACG_EIO, "Cannot open input script %s", path ? path : "(null)");
  std::string line, acc;
  while (std::getline(in, line)) {
    // '&' continues a line (input.cpp:119-125)
    size_t e = line.find_last_not_of(" \t\r\n");
    if (e != std::string::npos && line[e] == '&') {
      acc += line.substr(0, e) + " ";
      continue;
    }
    acc += line;
    h->command(acc);
    acc.clear();
  }
  if (!acc.empty()) h->command(acc);
  API_END
}

int cacg_set_box(cacg_handle h, const double *lo, const double *hi, const int *periodic) {
  API_BEGIN
  if (!lo || !hi || !periodic) fail(CACG_EINVAL, "null argument");
  for (int d = 0; d < 3; d++) {
    if (!(lo[d] < hi[d])) fail(CACG_EINVAL, "Box bounds are invalid");
    h->lo[d] = lo[d];
    h->hi[d] = hi[d];
    h->prd[d] = hi[d] - lo[d];
    h->periodic[d] = periodic[d] ? 1 : 0;
  }
  h->box_set = true;
  h->inited = false;
  API_END
}

int cacg_set_lj(cacg_handle h, int ntypes, const double *lj1, const double *lj2,
                const double *cutsq) {
  API_BEGIN
  if (h->pair_style != 1) fail(CACG_ESTATE, "cacg_set_lj after pair_style lj/cut");
  if (ntypes < 1 || ntypes > MAXT || !lj1 || !lj2 || !cutsq) fail(CACG_EINVAL, "bad LJ tables");
  if (h->ntypes > 0 && ntypes != h->ntypes) fail(CACG_EINVAL, "LJ tables for another type count");
  const size_t n = (size_t) (ntypes + 1) * (ntypes + 1);
  h->raw_lj1.assign(lj1, lj1 + n);
  h->raw_lj2.assign(lj2, lj2 + n);
  h->raw_cutsq.assign(cutsq, cutsq + n);
  for (int i = 1; i <= ntypes; i++)
    for (int j = 1; j <= ntypes; j++) {
      const size_t r = (size_t) i * (ntypes + 1) + j;
      if (!(cutsq[r] > 0.0) || !std::isfinite(lj1[r]) || !std::isfinite(lj2[r]))
        fail(CACG_EINVAL, "bad LJ tables");
    }
  for (int i = 1; i <= ntypes; i++)
    for (int j = i; j <= ntypes; j++) h->setflag[i][j] = 1;
  h->lj_raw = true;
  h->inited = false;
  API_END
}

int cacg_set_eam(cacg_handle h, int nr, double dr, int nrho, double drho, const double *frho7,
                 const double *rhor7, const double *z2r7, double cutforcesq, double mass) {
  API_BEGIN
  if (h->pair_style != 2) fail(CACG_ESTATE, "cacg_set_eam after pair_style eam");
  if (nr < 5 || nrho < 5 || !(dr > 0.0) || !(drho > 0.0) || !frho7 || !rhor7 || !z2r7 ||
      !(cutforcesq > 0.0) || !(mass > 0.0))
    fail(CACG_EINVAL, "bad EAM tables");
  h->nr = nr;
  h->dr = dr;
  h->rdr = 1.0 / dr;
  h->nrho = nrho;
  h->drho = drho;
  h->rdrho = 1.0 / drho;
  h->frho_sp.assign(frho7, frho7 + (size_t) (nrho + 1) * 7);
  h->rhor_sp.assign(rhor7, rhor7 + (size_t) (nr + 1) * 7);
  h->z2r_sp.assign(z2r7, z2r7 + (size_t) (nr + 1) * 7);
  h->cutforcesq = cutforcesq;
  h->eam_cut = std::sqrt(cutforcesq);
  h->eam_mass = mass;
  const int nt = std::max(h->ntypes, 1);
  for (int i = 1; i <= nt; i++) {
    h->setflag[i][i] = 1;
    h->amass[i] = mass;  // PairEAM::coeff sets the type mass (pair_eam.cpp:152-161)
  }
  h->inited = false;
  API_END
}

int cacg_set_masses(cacg_handle h, int ntypes, const double *mass) {
  API_BEGIN
  if (ntypes < 1 || ntypes > MAXT || !mass) fail(CACG_EINVAL, "bad mass table");
  h->ntypes = ntypes;
  for (int t = 1; t <= ntypes; t++) {
    if (mass[t - 1] <= 0.0) fail(CACG_EINVAL, "Invalid mass value");
    h->amass[t] = mass[t - 1];
  }
  h->inited = false;
  API_END
}

int cacg_set_atoms(cacg_handle h, int n, const double *x, const double *v, const int *type) {
  API_BEGIN
  if (n < 0 || (n > 0 && !x)) fail(CACG_EINVAL, "bad atom arrays");
  h->nlocal = n;
  h->h_x.assign(x, x + 3 * (size_t) n);
  h->h_v.assign(3 * (size_t) n, 0.0);
  if (v) h->h_v.assign(v, v + 3 * (size_t) n);
  h->h_type.assign(n, 1);
  if (type)
    for (int i = 0; i < n; i++) {
      if (type[i] < 1 || type[i] > std::max(h->ntypes, 1)) fail(CACG_EINVAL, "Invalid atom type");
      h->h_type[i] = type[i];
    }
  h->h_tag.resize(n);
  for (int i = 0; i < n; i++) h->h_tag[i] = i + 1;
  h->inited = false;
  API_END
}

int cacg_set_element_types(cacg_handle h, int ntypes, const int *nae, const int *numint,
                           const int *intp, const double *weight) {
  API_BEGIN
  if (ntypes < 1 || ntypes > MAXT || !nae || !numint || !intp || !weight) fail(CACG_EINVAL, "bad element types");
  h->netypes = ntypes;
  int off = 0;
  for (int t = 1; t <= ntypes; t++) {
    for (int d = 0; d < 3; d++) h->nae[t][d] = nae[3 * (t - 1) + d];
    if (h->nae[t][0] < 2 || h->nae[t][1] < 2 || h->nae[t][2] < 2) fail(CACG_EINVAL, "Invalid naae values");
    h->numint[t] = numint[t - 1];
    h->intp[t].assign(intp + 3 * off, intp + 3 * (off + numint[t - 1]));
    h->weight[t].assign(weight + off, weight + off + numint[t - 1]);
    off += numint[t - 1];
  }
  h->inited = false;
  API_END
}

int cacg_set_elements(cacg_handle h, int n, const int *etype, const double *centre,
                      const double *nodex, const double *nodev) {
  API_BEGIN
  if (n < 0 || (n > 0 && (!etype || !centre || !nodex))) fail(CACG_EINVAL, "bad element arrays");
  h->enlocal = n;
  h->h_etype.resize(n);
  for (int i = 0; i < n; i++) {
    if (etype[i] < 1 || etype[i] > h->netypes) fail(CACG_EINVAL, "Invalid element type");
    h->h_etype[i] = etype[i];
  }
  h->h_ex.assign(centre, centre + 3 * (size_t) n);
  h->h_nodex.assign(nodex, nodex + 24 * (size_t) n);
  h->h_nodev.assign(24 * (size_t) n, 0.0);
  if (nodev) h->h_nodev.assign(nodev, nodev + 24 * (size_t) n);
  h->h_etag.resize(n);
  for (int i = 0; i < n; i++) h->h_etag[i] = i + 1;
  h->inited = false;
  API_END
}

int cacg_set_precision(cacg_handle h, int mode) {
  API_BEGIN
  if (mode != CACG_FP64_EXACT && mode != CACG_FP64 && mode != CACG_MIXED) fail(CACG_EINVAL, "unknown precision mode");
  h->mode = mode;
  h->invalidate_graph();
  API_END
}

int cacg_init(cacg_handle h) {
  API_BEGIN
  h->init();
  API_END
}

int cacg_setup(cacg_handle h) {
  API_BEGIN
  h->setup();
  API_END
}

int cacg_neighbor_build(cacg_handle h) {
  API_BEGIN
  if (!h->setup_done) h->setup();
  h->neighbor_build();
  API_END
}

int cacg_neighbor_ebuild(cacg_handle h) {
  API_BEGIN
  if (!h->setup_done) h->setup();
  h->neighbor_ebuild();
  API_END
}

int cacg_neighbor_nbuild(cacg_handle h) {
  API_BEGIN
  if (!h->setup_done) h->setup();
  h->neighbor_nbuild();
  API_END
}

int cacg_pair_compute(cacg_handle h, int eflag, int vflag) {
  API_BEGIN
  (void) eflag;
  (void) vflag;
  h->pair_compute();
  h->sync();
  API_END
}

int cacg_pair_ecompute(cacg_handle h) {
  API_BEGIN
  h->pair_ecompute();
  h->sync();
  API_END
}

int cacg_fix_nve_initial_integrate(cacg_handle h) {
  API_BEGIN
  h->require_init();
  h->nve_initial();
  API_END
}

int cacg_fix_nve_final_integrate(cacg_handle h) {
  API_BEGIN
  h->require_init();
  h->nve_final();
  API_END
}

int cacg_run(cacg_handle h, int nsteps) {
  API_BEGIN
  h->run(nsteps);
  API_END
}

// Several handles' step loops as the branches of one CUDA graph: each launch
// runs every handle until its wanted steps are done or it needs a rebuild;
// the host performs those rebuilds (then one eager step each, so that the
// next capture holds no first-call work), captures again and relaunches.
// Where the combined graph cannot be built, each handle runs its remaining
// steps on its own.  An error is reported on the handle whose call raised it
// (its cacg_error); the other handles keep the steps they completed.
int cacg_run_batch(cacg_handle *hs, int nh, int nsteps) {
  if (!hs || nh < 1 || nsteps < 0) return CACG_EINVAL;
  for (int k = 0; k < nh; k++)
    if (!hs[k] || hs[k]->device != hs[0]->device) return CACG_EINVAL;
  for (int k = 0; k < nh; k++) hs[k]->err.clear();  // only the failing handle reports
  cacg_handle cur = hs[0];
  try {
    check(cudaSetDevice(hs[0]->device), "cudaSetDevice");
    std::vector<int> left(nh, nsteps);
    for (int k = 0; k < nh; k++) {
      cur = hs[k];
      EpochScope es(&cur->epoch);
      if (!cur->loop_device || !cur->use_graphs || !cur->graph_ok || cur->deform_on)
        fail(CACG_ESTATE, "run_batch takes handles with the device loop on (tune loop device), "
                          "graphs on and no box deformation");
      cur->run(0);  // set-up and lists, as a run starts
    }
    while (true) {
      std::vector<int> in;
      for (int k = 0; k < nh; k++) {
        cur = hs[k];
        EpochScope es(&cur->epoch);
        while (left[k] > 0 && cur->eager_since < 1) {  // first-call work outside the capture
          cur->run(1);
          left[k]--;
        }
        if (left[k] > 0) in.push_back(k);
      }
      if (in.empty()) break;
      cudaGraph_t top = nullptr;
      cudaGraphExec_t ex = nullptr;
      check(cudaGraphCreate(&top, 0), "batch graph");
      std::vector<long long> pre(nh, 0), post(nh, 0);
      std::vector<unsigned long long> e0(nh, 0);
      bool ok = true, destroyable = true;
      for (int k : in) {
        cur = hs[k];
        EpochScope es(&cur->epoch);
        cur->loop_prepare();
        e0[k] = dbuf_epoch();
        if (!cur->add_loop(top, pre[k], post[k], &destroyable)) {
          ok = false;
          break;
        }
      }
      for (int k : in) {
        EpochScope es(&hs[k]->epoch);
        if (dbuf_epoch() != e0[k]) ok = false;
      }
      if (ok && cudaGraphInstantiate(&ex, top, 0) != cudaSuccess) ok = false;
      if (destroyable) cudaGraphDestroy(top);
      cudaGetLastError();
      if (!ok) {  // each handle finishes its steps on its own
        if (ex) cudaGraphExecDestroy(ex);
        for (int k : in) {
          cur = hs[k];
          EpochScope es(&cur->epoch);
          cur->run(left[k]);
          left[k] = 0;
        }
        break;
      }
      const cudaStream_t s0 = hs[in[0]]->stream;
      for (int k : in) {
        cur = hs[k];
        check(cudaStreamSynchronize(cur->stream), "batch in");  // the handle's own work first
        cur->loop_arm(left[k]);
        check(cudaMemcpyAsync(cur->d_loop.p, cur->h_pin + 16, LOOP_SLOTS * sizeof(int),
                              cudaMemcpyHostToDevice, s0), "batch loop in");
      }
      cur = hs[in[0]];
      const cudaError_t le = cudaGraphLaunch(ex, s0);
      for (int k : in)
        if (le == cudaSuccess)
          check(cudaMemcpyAsync(hs[k]->h_pin + 16, hs[k]->d_loop.p, LOOP_SLOTS * sizeof(int),
                                cudaMemcpyDeviceToHost, s0), "batch loop out");
      const cudaError_t se = cudaStreamSynchronize(s0);
      cudaGraphExecDestroy(ex);
      check(le, "batch launch");
      check(se, "batch sync");
      for (int k : in) {
        cur = hs[k];
        EpochScope es(&cur->epoch);
        left[k] -= cur->loop_finish(left[k], pre[k], post[k]);
      }
    }
    return CACG_OK;
  } catch (const ApiError &e) {
    cur->err = e.msg;
    return e.code;
  } catch (const CudaError &e) {
    cur->err = std::string(e.where) + ": " + cudaGetErrorString(e.code);
    return e.code == cudaErrorMemoryAllocation ? CACG_ENOMEM : CACG_ECUDA;
  }
}

int cacg_run_host(cacg_handle h, int nsteps, double *x, double *v, double *nodex, double *nodev) {
  API_BEGIN
  h->run_host(nsteps, x, v, nodex, nodev);
  API_END
}

int cacg_get_counts(cacg_handle h, long long *c, int n) {
  API_BEGIN
  long long v[31] = {h->nlocal, h->nghost, 0, h->enlocal, h->enghost, 0, h->nrows, 0,
                     h->nrebuild, (long long) h->stencil.size(), h->ntimestep, h->nsites,
                     h->launches, h->nneed, h->nforce, 0, h->sur ? h->nfar : 0, 0, 0,
                     h->graph_steps, 0, 0, 0, h->nrebuild_atoms, 0,
                     (long long) h->h_nlines[0], (long long) h->h_nlines[1],
                     h->fused_used ? 1LL : 0LL, h->loop_launches, h->host_decisions, 0};
  if (h->d_band.p) {
    int b = 0;
    check(cudaMemcpyAsync(&b, h->d_band.p + 2, sizeof(b), cudaMemcpyDeviceToHost, h->stream), "band");
    h->sync();
    v[30] = b;
  }
  if (h->areorders_zeroed && h->d_misc.p) {
    unsigned r = 0;
    check(cudaMemcpyAsync(&r, h->d_misc.p + 16, sizeof(r), cudaMemcpyDeviceToHost, h->stream), "areorders");
    h->sync();
    v[24] = r;
  }
  if (h->sur && h->d_scount.p) {
    unsigned long long c2[2] = {0, 0};
    check(cudaMemcpyAsync(c2, h->d_scount.p, sizeof(c2), cudaMemcpyDeviceToHost, h->stream), "scount");
    h->sync();
    v[17] = (long long) c2[0];
    v[18] = (long long) c2[1];
  }
  if (h->list_built && h->nlocal) {
    std::vector<int> num(h->nlocal);
    check(cudaMemcpyAsync(num.data(), h->d_num.p, sizeof(int) * h->nlocal, cudaMemcpyDeviceToHost, h->stream), "num");
    h->sync();
    for (int x : num) v[2] += x;
  }
  if (h->enlocal && h->d_enum.p) {
    std::vector<int> num(h->enlocal);
    check(cudaMemcpyAsync(num.data(), h->d_enum.p, sizeof(int) * h->enlocal, cudaMemcpyDeviceToHost, h->stream), "enum");
    h->sync();
    for (int x : num) v[5] += x;
  }
  if (h->elists_built && h->nrows) {
    std::vector<int> num(h->nrows);
    check(cudaMemcpyAsync(num.data(), h->d_ipnum.p, sizeof(int) * h->nrows, cudaMemcpyDeviceToHost, h->stream), "ipnum");
    h->sync();
    for (int x : num) v[7] += x;
  }
  if (h->list_built && h->nlocal && h->d_snum.p && h->d_snum.cap >= (size_t) h->nlocal) {
    std::vector<int> num(h->nlocal);
    check(cudaMemcpyAsync(num.data(), h->d_snum.p, sizeof(int) * h->nlocal, cudaMemcpyDeviceToHost, h->stream), "snum");
    h->sync();
    for (int x : num) v[15] += x;
  }
  // entries the last mixed density pass scanned: the near parts of the
  // reordered lists when the displacement since the reorder allowed culling
  // (the device test of k_eam_rho_atoms, repeated here), else every entry
  v[20] = v[2];
  if (h->mode == CACG_MIXED && h->pair_style == 2 && !h->mixed_union && h->mixed_cull &&
      h->part_of == h->list_builds && h->nlocal && h->d_nnear.p && h->d_misc.p) {
    unsigned dm[2] = {0, 0};
    check(cudaMemcpyAsync(dm, h->d_misc.p + 11, sizeof(dm), cudaMemcpyDeviceToHost, h->stream), "dmax");
    std::vector<int4> nn(h->nlocal);
    check(cudaMemcpyAsync(nn.data(), h->d_nnear.p, sizeof(int4) * h->nlocal, cudaMemcpyDeviceToHost, h->stream), "nnear");
    h->sync();
    float d2;
    std::memcpy(&d2, &dm[0], sizeof(float));
    const int level = mixed::cull_level_host(d2, dm[1]);
    if (level < 4) {
      v[20] = 0;
      for (const int4 &x : nn) v[20] += level == 1 ? x.x : level == 2 ? x.y : x.z;
    }
  }
  // integration-point entries the last mixed passes scanned (near parts while
  // the node displacement allowed culling) and the list reorders so far
  v[21] = v[7];
  if (h->mode == CACG_MIXED && h->epart_of == h->elist_builds && h->nrows && h->d_nnear_row.p &&
      h->d_misc.p) {
    unsigned dm[3] = {0, 0, 0};
    check(cudaMemcpyAsync(dm, h->d_misc.p + 13, sizeof(dm), cudaMemcpyDeviceToHost, h->stream), "edmax");
    h->sync();
    v[22] = dm[2];
    float d2;
    std::memcpy(&d2, &dm[0], sizeof(float));
    const int level = mixed::cull_level_host(d2, dm[1]);
    if (h->mixed_cull && level < 4) {
      std::vector<int4> nn(h->nrows);
      check(cudaMemcpyAsync(nn.data(), h->d_nnear_row.p, sizeof(int4) * h->nrows, cudaMemcpyDeviceToHost, h->stream), "nnear_row");
      h->sync();
      v[21] = 0;
      for (const int4 &x : nn) v[21] += level == 1 ? x.x : level == 2 ? x.y : x.z;
    }
  }
  for (int i = 0; i < n && i < 31; i++) c[i] = v[i];
  API_END
}

int cacg_get_atoms(cacg_handle h, int all, double *x, double *v, double *f, int *tag) {
  API_BEGIN
  if (!h->inited) fail(CACG_ESTATE, "no device state yet (cacg_init)");
  int n = all ? h->nlocal + h->nghost : h->nlocal;
  cudaStream_t s = h->stream;
  if (x && n) {
    h->d_stage.ensure(3 * (size_t) n, s);
    launch_unpack4to3(h->d_x.p, h->d_stage.p, n, s);
    check(cudaMemcpyAsync(x, h->d_stage.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s), "x");
  }
  if (v && h->nlocal) check(cudaMemcpyAsync(v, h->d_v.p, sizeof(double) * 3 * h->nlocal, cudaMemcpyDeviceToHost, s), "v");
  if (f && h->nlocal) check(cudaMemcpyAsync(f, h->d_f.p, sizeof(double) * 3 * h->nlocal, cudaMemcpyDeviceToHost, s), "f");
  if (tag && n) check(cudaMemcpyAsync(tag, h->d_tag.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s), "tag");
  h->sync();
  API_END
}

int cacg_get_elements(cacg_handle h, int all, double *centre, double *nodex, double *nodev,
                      double *nodef, int *tag) {
  API_BEGIN
  if (!h->inited) fail(CACG_ESTATE, "no device state yet (cacg_init)");
  int n = all ? h->enlocal + h->enghost : h->enlocal;
  cudaStream_t s = h->stream;
  if (centre && n) check(cudaMemcpyAsync(centre, h->d_ex.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, s), "ex");
  if (nodex && n) check(cudaMemcpyAsync(nodex, h->d_nodex.p, sizeof(double) * 24 * n, cudaMemcpyDeviceToHost, s), "nodex");
  if (nodev && h->enlocal) check(cudaMemcpyAsync(nodev, h->d_nodev.p, sizeof(double) * 24 * h->enlocal, cudaMemcpyDeviceToHost, s), "nodev");
  if (nodef && h->enlocal) check(cudaMemcpyAsync(nodef, h->d_nodef.p, sizeof(double) * 24 * h->enlocal, cudaMemcpyDeviceToHost, s), "nodef");
  if (tag && n) check(cudaMemcpyAsync(tag, h->d_etag.p, sizeof(int) * n, cudaMemcpyDeviceToHost, s), "etag");
  h->sync();
  API_END
}

int cacg_get_atom_list(cacg_handle h, int *numneigh, int *neigh) {
  API_BEGIN
  if (!h->list_built) fail(CACG_ESTATE, "atom list not built");
  int n = h->nlocal;
  if (!n) return CACG_OK;
  std::vector<int> num(n), lst((size_t) h->maxneigh * h->stride);
  check(cudaMemcpyAsync(num.data(), h->d_num.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream), "num");
  check(cudaMemcpyAsync(lst.data(), h->d_list.p, sizeof(int) * lst.size(), cudaMemcpyDeviceToHost, h->stream), "list");
  h->sync();
  size_t o = 0;
  for (int i = 0; i < n; i++) {
    if (numneigh) numneigh[i] = num[i];
    for (int k = 0; k < num[i]; k++)
      if (neigh) neigh[o++] = lst[(size_t) k * h->stride + i];
  }
  API_END
}

int cacg_get_elem_list(cacg_handle h, int *numneigh, int *neigh) {
  API_BEGIN
  int n = h->enlocal;
  if (!n) return CACG_OK;
  if (!h->d_enum.p) fail(CACG_ESTATE, "element list not built");
  std::vector<int> num(n), lst((size_t) h->maxeneigh * h->estride);
  check(cudaMemcpyAsync(num.data(), h->d_enum.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream), "enum");
  check(cudaMemcpyAsync(lst.data(), h->d_elist.p, sizeof(int) * lst.size(), cudaMemcpyDeviceToHost, h->stream), "elist");
  h->sync();
  size_t o = 0;
  for (int i = 0; i < n; i++) {
    if (numneigh) numneigh[i] = num[i];
    for (int k = 0; k < num[i]; k++)
      if (neigh) neigh[o++] = lst[(size_t) k * h->estride + i];
  }
  API_END
}

int cacg_get_ip_list(cacg_handle h, int *numneigh, int *jelem, int *jsite) {
  API_BEGIN
  if (!h->elists_built) fail(CACG_ESTATE, "node neighbor list not built");
  int n = h->nrows;
  if (!n) return CACG_OK;
  std::vector<int> num(n), lst((size_t) h->maxip * h->rowstride);
  check(cudaMemcpyAsync(num.data(), h->d_ipnum.p, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream), "ipnum");
  check(cudaMemcpyAsync(lst.data(), h->d_ipent.p, sizeof(int) * lst.size(), cudaMemcpyDeviceToHost, h->stream), "ipent");
  h->sync();
  size_t o = 0;
  const std::vector<int> &sb = h->h_site_base;
  for (int r = 0; r < n; r++) {
    if (numneigh) numneigh[r] = num[r];
    for (int k = 0; k < num[r]; k++) {
      int sid = lst[(size_t) k * h->rowstride + r];
      int e = (int) (std::upper_bound(sb.begin(), sb.end(), sid) - sb.begin()) - 1;
      if (jelem) jelem[o] = e;
      if (jsite) jsite[o] = sid - sb[e];
      o++;
    }
  }
  API_END
}

int cacg_get_cut(cacg_handle h, int what, double *value) {
  API_BEGIN
  if (!value) fail(CACG_EINVAL, "null argument");
  double v[6] = {h->cutneighmax, h->cut_all, h->cut_ele, h->cut_subele, h->max_size, (double) h->nsub};
  if (what < 0 || what > 5) fail(CACG_EINVAL, "unknown cutoff index");
  *value = v[what];
  API_END
}

int cacg_set_timing(cacg_handle h, int enable) {
  API_BEGIN
  h->timing = enable != 0;
  API_END
}

int cacg_compute_thermo(cacg_handle h, double *out, int n) {
  API_BEGIN
  if (!out || n < 1) fail(CACG_EINVAL, "bad output array");
  double v[17];
  h->compute_thermo(v);
  for (int i = 0; i < n && i < 17; i++) out[i] = v[i];
  API_END
}

int cacg_get_box(cacg_handle h, double *lo, double *hi) {
  API_BEGIN
  for (int d = 0; d < 3; d++) {
    if (lo) lo[d] = h->lo[d];
    if (hi) hi[d] = h->hi[d];
  }
  API_END
}

int cacg_set_group(cacg_handle h, const char *name, const int *atom_in, const int *elem_in) {
  API_BEGIN
  if (!name || !*name) fail(CACG_EINVAL, "null group name");
  h->set_group(name, atom_in, elem_in);
  API_END
}

int cacg_set_graphs(cacg_handle h, int enable) {
  API_BEGIN
  h->use_graphs = enable != 0;
  h->graph_ok = true;
  h->hgraph_ok = true;
  h->invalidate_graph();
  API_END
}

int cacg_fix_post_force(cacg_handle h) {
  API_BEGIN
  if (!h->inited) fail(CACG_ESTATE, "no device state yet (cacg_init)");
  h->post_force();
  API_END
}

int cacg_compute_centro(cacg_handle h, double *centro, int n) {
  API_BEGIN
  if (!centro) fail(CACG_EINVAL, "null output array");
  if (n != h->nlocal) fail(CACG_EINVAL, "n must equal the number of local atoms (%d)", h->nlocal);
  h->compute_centro(centro);
  API_END
}

int cacg_dump_xyz(cacg_handle h, const char *path) {
  API_BEGIN
  if (!path) fail(CACG_EINVAL, "null path");
  h->dump_xyz(path);
  API_END
}

int cacg_dump_elements(cacg_handle h, const char *path, int append) {
  API_BEGIN
  if (!path) fail(CACG_EINVAL, "null path");
  h->dump_elements(path, append);
  API_END
}

int cacg_surrogate_reference(cacg_handle h, const double *nodex0) {
  API_BEGIN
  h->surrogate_reference(nodex0);
  h->sync();
  API_END
}

int cacg_surrogate_samples(cacg_handle h, float *x, float *t, int n) {
  API_BEGIN
  if (!x || !t) fail(CACG_EINVAL, "null output array");
  if (n != h->enlocal) fail(CACG_EINVAL, "n must equal the number of local elements (%d)", h->enlocal);
  h->surrogate_samples(x, t);
  API_END
}

int cacg_surrogate_attach(cacg_handle h, cacg_mlp m, double tol, double dist) {
  API_BEGIN
  h->surrogate_attach(m, tol, dist);
  API_END
}

int cacg_get_kernel_timing(cacg_handle h, double *ms, int n) {
  API_BEGIN
  for (int i = 0; i < n && i < cacg_context::KT_N; i++) ms[i] = h->t_kern[i];
  if (n > cacg_context::KT_N) ms[cacg_context::KT_N] = h->rebuild_ms_total;
  API_END
}

int cacg_get_timing(cacg_handle h, double *ms, int n) {
  API_BEGIN
  for (int i = 0; i < n && i < 8; i++) ms[i] = h->t_ms[i];
  API_END
}

int cacg_put_atoms(cacg_handle h, const double *x, const double *v) {
  API_BEGIN
  if (!h->inited) fail(CACG_ESTATE, "no device state yet (cacg_init)");
  int n = h->nlocal;
  cudaStream_t s = h->stream;
  if (n && x) {
    h->d_stage.ensure(3 * (size_t) n, s);
    check(cudaMemcpyAsync(h->d_stage.p, x, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s), "put x");
    launch_pack3to4(h->d_stage.p, h->d_x.p, n, s);
  }
  if (n && v) check(cudaMemcpyAsync(h->d_v.p, v, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, s), "put v");
  API_END
}

int cacg_put_nodes(cacg_handle h, const double *nodex, const double *nodev) {
  API_BEGIN
  if (!h->inited) fail(CACG_ESTATE, "no device state yet (cacg_init)");
  int n = h->enlocal;
  if (n && nodex) check(cudaMemcpyAsync(h->d_nodex.p, nodex, sizeof(double) * 24 * n, cudaMemcpyHostToDevice, h->stream), "put nodex");
  if (n && nodev) check(cudaMemcpyAsync(h->d_nodev.p, nodev, sizeof(double) * 24 * n, cudaMemcpyHostToDevice, h->stream), "put nodev");
  API_END
}

int cacg_measure_fp64_peak(cacg_handle h, double *flops) {
  API_BEGIN
  if (!flops) fail(CACG_EINVAL, "null argument");
  *flops = fp64_fma_rate(h->stream);
  API_END
}

}  // extern "C"
