/*
 * cacg.h -- C ABI of the GB300 CAC force path (libcacg.so).
 *
 * One handle owns one CAC system resident on one GPU: atoms (x, v, f, type),
 * 8-node elements (nodes, centres, velocities, forces), their ghost images,
 * bins, the three neighbor lists and the pair-style tables.  Every entry
 * point returns 0 on success or a negative status; cacg_error() gives the
 * message.  Plain pointers and sizes only; host arrays are caller-owned and
 * copied in or out.  One host thread per handle.
 *
 * Each entry point replaces the reference routine named beside it (file:line in
 * fangyuanxiao/CAC_Code).  Where the reference is a C++ virtual (Pair,
 * Neighbor, Fix), a reference-side subclass of that virtual calls these entry
 * points from its overrides.
 */
#ifndef CACG_H
#define CACG_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct cacg_context *cacg_handle;

/* status codes */
#define CACG_OK 0
#define CACG_EINVAL (-1)     /* bad argument or command (error->all in the reference) */
#define CACG_ESTATE (-2)     /* call out of order (e.g. forces before lists) */
#define CACG_ECUDA (-3)      /* CUDA runtime error */
#define CACG_EOVERFLOW (-4)  /* neighbor list overflow that regrowing could not fix */
#define CACG_EIO (-5)        /* file could not be read */
#define CACG_ENOMEM (-6)     /* device allocation failed */
#define CACG_ETIMEOUT (-7)   /* a bounded device wait ran out */
#define CACG_ESCRATCH (-8)   /* request larger than a fixed scratch array */

/* precision modes (cacg_set_precision) */
#define CACG_FP64_EXACT 0    /* reference operation order, no contraction: bit-identical */
#define CACG_FP64 1          /* FP64 with fused multiply-add */
#define CACG_MIXED 2         /* FP32 pair terms, FP64 accumulation and integration */

/* ---- lifetime (CAC::CAC / CAC::~CAC, cac.cpp:29-148) ---- */
int cacg_create(cacg_handle *out, int device);
int cacg_destroy(cacg_handle h);
const char *cacg_error(cacg_handle h);
const char *cacg_version(void);

/* ---- input commands (Input::execute_command, input.cpp:362-404) ----
 * Accepts: units lj|metal, boundary, dimension 3, timestep, elementsplit,
 * read_data FILE, pair_style lj/cut RC | eam, pair_coeff, neighbor SKIN bin,
 * neigh_modify every/delay/check/binsize/one/page, fix ID all nve, run N. */
int cacg_command(cacg_handle h, const char *line);
/* Input::file, input.cpp:95-194: every line of an input script */
int cacg_file(cacg_handle h, const char *path);

/* ---- direct state (ReadData::command sections, read_data.cpp:166-211) ---- */
int cacg_set_box(cacg_handle h, const double *lo, const double *hi, const int *periodic);
/* Domain::boxlo/boxhi now (they move under "fix ID all deform 1 x erate R":
   L(t) = L0 (1 + R t) about the box centre, positions remapped affinely at the
   end of each step; the reference has no box deformation) */
int cacg_get_box(cacg_handle h, double *lo, double *hi);
int cacg_set_masses(cacg_handle h, int ntypes, const double *mass);         /* Masses */
int cacg_set_atoms(cacg_handle h, int n, const double *x, const double *v,
                   const int *type);                                          /* Atoms */
int cacg_set_element_types(cacg_handle h, int ntypes, const int *nae,
                           const int *numint, const int *intp,
                           const double *weight);                 /* NAAE, Numint, Intp */
int cacg_set_elements(cacg_handle h, int n, const int *etype, const double *centre,
                      const double *nodex, const double *nodev);      /* Elements, Nodes */
int cacg_set_precision(cacg_handle h, int mode);

/* ---- pair tables handed over as the reference built them ----
   For a Pair subclass whose base already read the potential: after
   pair_style lj/cut, the PairLJCut tables after init_one
   (pair_lj_cut.cpp:140-198), lj1, lj2, cutsq as [ntypes + 1][ntypes + 1]
   (the contiguous memory->create 2-d arrays, row 0 and column 0 unused);
   they replace pair_coeff's epsilon, sigma and cutoff. */
int cacg_set_lj(cacg_handle h, int ntypes, const double *lj1, const double *lj2,
                const double *cutsq);
/* After pair_style eam: the splines PairEAM::array2spline made for the one
   species (pair_eam.cpp:527-580), frho_spline[type2frho[1]] [nrho + 1][7],
   rhor_spline[type2rhor[1][1]] and z2r_spline[type2z2r[1][1]] [nr + 1][7],
   with the grids nr, dr, nrho, drho, cutforcesq (pair_eam.cpp:274-282) and
   the potential's mass; they replace pair_coeff's file. */
int cacg_set_eam(cacg_handle h, int nr, double dr, int nrho, double drho, const double *frho7,
                 const double *rhor7, const double *z2r7, double cutforcesq, double mass);

/* ---- init and setup ---- */
int cacg_init(cacg_handle h);       /* CAC::init, cac.cpp:202-213 (tables, cutoffs) */
int cacg_setup(cacg_handle h);      /* Verlet::setup through comm->borders, verlet.cpp:70-90 */

/* ---- neighbor (Neighbor::build/ebuild/nbuild, neighbor.h:74-76) ---- */
int cacg_neighbor_build(cacg_handle h);    /* neighbor.cpp:984-1018 half_bin_no_newton (full) */
int cacg_neighbor_ebuild(cacg_handle h);   /* neighbor.cpp:1022-1062 element_neighbor */
int cacg_neighbor_nbuild(cacg_handle h);   /* neighbor.cpp:1096-1106 node_neighbor */

/* ---- pair (Pair::compute / Pair::ecompute, pair.h:82-105) ---- */
int cacg_pair_compute(cacg_handle h, int eflag, int vflag);  /* atoms: f = sum over list */
int cacg_pair_ecompute(cacg_handle h);  /* integration points -> nodef (zeroed first) */

/* ---- FixNVE (fix_nve.cpp:54-242), atoms and nodes ---- */
int cacg_fix_nve_initial_integrate(cacg_handle h);
int cacg_fix_nve_final_integrate(cacg_handle h);

/* ---- Verlet::run, verlet.cpp:149-219 (atoms also get Pair::compute) ---- */
int cacg_run(cacg_handle h, int nsteps);
/* nsteps Verlet steps on each of nh handles (one device, "tune loop device",
   graphs on, no deformation) as the branches of one CUDA graph: a launch runs
   every handle until its steps are done or it needs a rebuild, which the host
   then performs before the next launch (Verlet::run, verlet.cpp:149-219, for
   independent systems at once).  Results equal cacg_run on each handle. */
int cacg_run_batch(cacg_handle *hs, int nh, int nsteps);

/* ---- host-owned state in (drop-in callers keep Atom::x/v and Element::nodex/nodev,
   atom.h:40, element.h:25, in host memory and push them every step) ---- */
int cacg_put_atoms(cacg_handle h, const double *x, const double *v);      /* [nlocal][3] */
int cacg_put_nodes(cacg_handle h, const double *nodex, const double *nodev); /* [n][8][3] */
/* Verlet::run (verlet.cpp:149-219) on host-resident state: x, v [nlocal][3] and
   nodex, nodev [enlocal][8][3] are copied in, nsteps steps run, and the new
   state is copied back into the same buffers before the call returns (pinned
   buffers give the full link bandwidth).  In mixed precision the last step's
   copies overlap its computation (the smaller of the atom and node states in
   first, outputs once every input is in: positions after the step's initial
   integration, velocities as each chain integrates them, the node velocities
   part by part behind the element force pass, "tune out_parts"), and a
   single-step call on pinned
   buffers used in the previous call replays one captured graph of the whole
   call (with cacg_set_graphs on); the results equal cacg_put_atoms +
   cacg_put_nodes + cacg_run + cacg_get_atoms + cacg_get_elements. */
int cacg_run_host(cacg_handle h, int nsteps, double *x, double *v, double *nodex, double *nodev);

/* ---- state out ---- */
/* counts: 0 nlocal 1 nghost 2 atom-list entries 3 elem nlocal 4 elem nghost
   5 element-list entries 6 integration-point rows 7 ip-list entries
   8 rebuilds so far 9 stencil bins 10 step number 11 interpolated sites
   12 kernel launches issued 13 sites referenced by the lists
   14 integration points of nonzero weight 15 atom short-list entries of the
   last force evaluation 16 elements handed to the surrogate 17 surrogate
   evaluations (element-steps) 18 of which accepted 19 steps replayed from a
   captured CUDA graph 20 atom-list entries the last mixed EAM density pass
   scanned (fewer than 2 while displacement culling holds) 21 integration-point
   list entries the last mixed element passes scanned per pass (fewer than 7
   while culling holds) 22 reorders of the mixed integration-point lists so far
   23 rebuilds that kept the element lists (only atoms had moved past the
   trigger; "tune elists lazy", FP64 and mixed modes) 24 reorders of the mixed
   atom lists so far 25 lattice lines (element, line) with a site in some
   integration-point list 26 of these, lines with a site in a list of a row of
   nonzero weight 27 1 if the last mixed element pass ran fused (one warp per
   element: every list entry references its row's own element) 28 graph
   launches of the device step loop so far ("tune loop device") 29 rebuild
   decisions taken on the host so far (the device loop takes its own)
   30 element passes re-run so far because a pair of the element fell in the
   guard band of the FP32 cutoff decision (fused passes; decided in FP64) */
int cacg_get_counts(cacg_handle h, long long *counts, int n);
/* Atom::x/v/f (atom.h:40); all != 0 includes ghosts for x and tag */
int cacg_get_atoms(cacg_handle h, int all, double *x, double *v, double *f, int *tag);
/* Element::x/nodex/nodev/nodef (element.h:25) */
int cacg_get_elements(cacg_handle h, int all, double *centre, double *nodex, double *nodev,
                      double *nodef, int *tag);
/* NeighList ilist/numneigh/firstneigh (neigh_list.h:26-33), indices in the
   reference's local+ghost numbering, rows concatenated */
int cacg_get_atom_list(cacg_handle h, int *numneigh, int *neigh);
int cacg_get_elem_list(cacg_handle h, int *numneigh, int *neigh);
/* NodeNeighList numneigh/firstneigh/nfirstneigh (node_neigh_list.h:23-27) */
int cacg_get_ip_list(cacg_handle h, int *numneigh, int *jelem, int *jsite);
/* 0 cutneighmax 1 cut_all 2 cut_ele 3 cut_subele 4 max_size 5 nsubele */
int cacg_get_cut(cacg_handle h, int what, double *value);

/* ---- thermo (the reference's compute pe/temp/pressure are stubs,
   compute_pe.cpp:16-49; these are the standard pair-style energies) ----
   FP64 at the current positions: out[0] potential energy of atoms, [1] of
   elements (integration-point weights), [2] kinetic energy of atoms, [3] of
   nodes (nodal mass M_e/8), [4..9] pair virial sum r_a f_b (xx yy zz xy xz yz,
   atoms + weighted integration points), [10..15] kinetic tensor sum m v_a v_b,
   [16] box volume.  Energies in the unit style's energy unit.  Returns the
   number filled (n <= 17). */
int cacg_compute_thermo(cacg_handle h, double *out, int n);

/* ---- kinetic sums without device allocation (no counterpart in the
   reference) ----
   For callers that may not allocate device memory when they call: a driver
   reporting thermo from its per-step output hook, where cudaMalloc/cudaFree
   would synchronise the device, or one whose device memory is reserved by
   another framework's allocator.  v[n][3], type[n / per_item] (1-based, or
   element types for nodes) and mass[type] are the caller's device arrays;
   out[7] (device) receives mvv2e * (sum 1/2 m v^2, sum m vx vx, m vy vy,
   m vz vz, m vx vy, m vx vz, m vy vz) with m = mass[type[i / per_item]] *
   scale, launched on `stream` (a cudaStream_t; NULL = default stream).
   Partial sums live in a fixed 448 KiB device array: n above
   CACG_NOALLOC_MAX_ITEMS returns CACG_ESCRATCH.  Nothing has to be zeroed
   first.  Calls share that array per device, so calls that can overlap
   race: serialise them.  The first call on a device resolves the array's
   address (make it, n = 0 is enough, before any stream capture) and caches
   it per device ordinal: the address is the primary context's, so it does
   not outlive cudaDeviceReset and does not serve another current context.
   A CUDA error already pending from earlier work is reported as CACG_ECUDA
   and left pending (nothing is launched).  Returns CACG_OK once both kernels
   are queued. */
#define CACG_NOALLOC_MAX_ITEMS (8192 * 256)
int cacg_kinetic_noalloc(const double *v, const int *type, const double *mass, int n,
                         int per_item, double scale, double mvv2e, double *out, void *stream);

/* Modify::post_force (modify.cpp:663-669): the fix setforce / fix viscous
   commands of the input, in order, on the current forces (cacg_run applies
   them itself between the force passes and the final integration). */
int cacg_fix_post_force(cacg_handle h);
/* Group membership from flags per local atom and element (nonzero = in the
   group; NULL = none), for groups no region describes (the reference builds
   groups with "group ID region ...", group.cpp:80-200, also accepted by
   cacg_command). */
int cacg_set_group(cacg_handle h, const char *name, const int *atom_in, const int *elem_in);

/* ---- analysis and output ----
   Output::centro_atom (output.cpp:352-447): centro-symmetry of the n local
   atoms (n = local atoms) over the atom neighbor list, bit-identical to the
   reference; 0 for atoms with fewer than 12 neighbors in range. */
int cacg_compute_centro(cacg_handle h, double *centro, int n);
/* DumpXyz (dump_xyz.cpp): "N\nXYZ\n" then "Cu x y z centro" for the atoms
   with 1 < centro < 10 (the reference's dump after Verlet::setup). */
int cacg_dump_xyz(cacg_handle h, const char *path);
/* DumpElement (dump_element.cpp:69-128): a Tecplot FE-brick zone (header,
   one "x y z vx vy vz fx fy fz" line per node, 8 node numbers per element);
   append != 0 adds a zone to an existing file. */
int cacg_dump_elements(cacg_handle h, const char *path, int append);

/* ---- nodal-force surrogate (no counterpart in the reference, which
   evaluates every element by integration-point quadrature) ----
   An ensemble of MLPs 32 -> 256 -> 256 -> 256 -> 24 (SiLU) maps an element's
   features (24 nodal displacements about their mean, relative to the ideal
   lattice, then 8 nodal densities) to its 24 nodal forces.  Forward and
   backward passes run on the tensor cores (BF16 operands, FP32 accumulation);
   weights are FP32 masters trained with Adam.  Parameters per member, in
   order: W1[256][32] b1[256] W2[256][256] b2[256] W3[256][256] b3[256]
   W4[24][256] b4[24].  Arrays are host arrays. */
typedef struct cacg_mlp_t *cacg_mlp;
/* members: 1..4 */
int cacg_mlp_create(cacg_mlp *m, int device, int members, unsigned long long seed);
int cacg_mlp_destroy(cacg_mlp m);
const char *cacg_mlp_error(cacg_mlp m);
/* sizes: 0 members 1 parameters per member 2 inputs 3 outputs 4 hidden width
   5 optimizer steps taken */
int cacg_mlp_sizes(cacg_mlp m, long long *sizes, int n);
int cacg_mlp_get_params(cacg_mlp m, int member, float *params);
int cacg_mlp_set_params(cacg_mlp m, int member, const float *params);
/* inputs are standardised as (x - in_mean) / in_std; outputs are
   out_mean + out_std * y; force_scale (rms nodal-force magnitude) is the unit
   of the ensemble-spread tolerance */
int cacg_mlp_set_normalization(cacg_mlp m, const float *in_mean, const float *in_std,
                               const float *out_mean, const float *out_std, double force_scale);
int cacg_mlp_get_normalization(cacg_mlp m, float *in_mean, float *in_std, float *out_mean,
                               float *out_std, double *force_scale);
/* mean-squared error of member's normalised outputs on n samples x[n][32],
   t[n][24] and its gradient with respect to every parameter (no update) */
int cacg_mlp_loss_grad(cacg_mlp m, int member, const float *x, const float *t, int n,
                       double *loss, float *grad);
/* Adam over shuffled whole batches (batch a multiple of 128) for every member;
   *loss = mean normalised loss of the last epoch */
int cacg_mlp_train(cacg_mlp m, const float *x, const float *t, long long n, int epochs, int batch,
                   float lr, unsigned long long seed, double *loss);
/* ensemble mean[n][24] (force units) and spread[n] (largest per-output
   standard deviation across members, force units) */
int cacg_mlp_predict(cacg_mlp m, const float *x, long long n, float *mean, float *spread);
/* C[m][n] = A[m][k] B[n][k]^T on device arrays (bf16 A, B; fp32 C), k a
   multiple of 64, lda/ldb multiples of 8; *err (device int) is set if a
   bounded wait in the kernel ran out */
int cacg_gemm_bf16_tn(const void *a, int lda, const void *b, int ldb, float *c, int ldc, int m,
                      int n, int k, int *err, void *stream);

/* Surrogate in the step (CACG_MIXED element pass).  Reference node
   positions [enlocal][8][3] for the displacement features (NULL: the current
   nodes); by default the nodes at the first surrogate call. */
int cacg_surrogate_reference(cacg_handle h, const double *nodex0);
/* Features x[n][32] and plain-quadrature nodal forces t[n][24] of every local
   element at the current state (n = local elements), in the handle's
   precision mode: the surrogate's training samples. */
int cacg_surrogate_samples(cacg_handle h, float *x, float *t, int n);
/* Use m for the elements lying farther than dist from every atom; an
   element whose ensemble spread exceeds tol * force_scale falls back to the
   quadrature that step.  m = NULL detaches. */
int cacg_surrogate_attach(cacg_handle h, cacg_mlp m, double tol, double dist);

/* ---- measurement ---- */
/* Phase timing of the last cacg_run from CUDA events on the handle's stream
   (recorded only after cacg_set_timing(h, 1)): ms[0] total, [1] integrate +
   rebuild decision + ghost refresh or rebuild, [2] atom pass 1 (LJ force or
   EAM density), [3] atom pass 2 (EAM force), [4] element forces and nodal
   gather, [5] final integrate; each summed over the steps of the run. */
int cacg_set_timing(cacg_handle h, int enable);
/* Steps that reach no rebuild decision (Neighbor::decide returns 0 without a
   check) are captured once into a CUDA graph and replayed until a rebuild,
   a reallocation or any command; on by default.  Phase timing covers the
   steps run eagerly only. */
int cacg_set_graphs(cacg_handle h, int enable);
/* Milliseconds of the last cacg_run: [0] all steps (device events), and with
   timing on, summed over the eagerly run steps: [1] integration + ghost update
   or rebuild, [2] atom pass 1, [3] atom pass 2, [4] element passes and fixes,
   [5] final integration, [6] the EAM atom density kernel alone.  n <= 8. */
int cacg_get_timing(cacg_handle h, double *ms, int n);
/* Device milliseconds of the main kernels in the last cacg_run, from CUDA
   events around each launch on the handle's stream (recorded only with
   cacg_set_timing(h, 1), summed over the eagerly run steps): [0] atom pass 1
   (LJ forces or EAM densities and F'), [1] atom pass 2 (EAM forces), [2]
   nodal densities (element density pass), [3] integration-point forces, [4]
   surrogate (features, ensemble, acceptance), [5] element sites (FP64 modes)
   or lattice lines (mixed), [6] mixed atom-list reorder, [7] mixed
   integration-point rows, reorder and line masks, [8] site F'(rho); then [9]
   the device milliseconds of every rebuild since the handle was created
   (Neighbor::decide -> reneighbor branch of verlet.cpp:184-198, timing on or
   off).  n <= 10. */
int cacg_get_kernel_timing(cacg_handle h, double *ms, int n);
/* Device-time of a FP64 fused-multiply-add loop on this GPU, for the FP64 roof:
   returns achieved FP64 FLOP/s in *flops. */
int cacg_measure_fp64_peak(cacg_handle h, double *flops);

#ifdef __cplusplus
}
#endif

#endif
