/*
 * CPU restatement of the reference CAC per-step force path.
 *
 * TEST INFRASTRUCTURE ONLY: used by tests/, the fixture generator and the
 * CPU-baseline leg of bench.py, never by the product.  Pinned against the
 * unmodified reference (oracle/_ref) and the fixtures in tests/golden/.
 *
 * Every routine restates a reference routine (file:line in the reference
 * tree) with the same floating-point operation order, so that its neighbor
 * lists are identical to the reference's and its FP64 forces agree bit for
 * bit when compiled without contraction (-ffp-contract=off).  Where the
 * reference's driver never runs a piece of the path, the restatement follows
 * the code as written and the oracle harness (oracle/ref/harness.cpp) drives
 * the reference the same way.
 */
#include "cac_oracle.h"

#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define NPE 8
#define MAXTYPES 8
#define BIGV 1.0e20
#define SMALLB 1.0e-6 /* neighbor.cpp:32 */
#define TOLNODE 0.01  /* element.cpp:21 */

typedef struct {
  int n, cap;
  int *v;
} ivec;

static void iv_push(ivec *a, int x) {
  if (a->n == a->cap) {
    a->cap = a->cap ? 2 * a->cap : 1024;
    a->v = (int *) realloc(a->v, (size_t) a->cap * sizeof(int));
  }
  a->v[a->n++] = x;
}

typedef struct {
  int dim;
  int pbc;          /* +1, -1 or 0 */
  double lo, hi;    /* atom slab */
  double mlo[MAXTYPES + 1], mhi[MAXTYPES + 1]; /* element slabs by type */
  ivec send;        /* atom indices sent */
  int firstrecv;
  ivec esend;
  int efirstrecv;
} swap_t;

struct orc_sys {
  char err[512];
  /* units, update.cpp:83-132 */
  double ftm2v, dt;
  /* domain */
  double boxlo[3], boxhi[3], prd[3];
  int periodic[3];
  /* neighbor settings */
  double skin, cutneighmax, cutneighmaxsq, binsize_user, triggersq;
  int every, delay, dist_check, binsizeflag;
  int nsplit;
  /* atoms */
  int ntypes;
  double amass[MAXTYPES + 1];
  int nlocal, nghost, amax;
  double *x, *v, *f;
  int *type, *tag;
  double *xhold;
  /* element types */
  int netypes;
  int nae[MAXTYPES + 1][3];
  int numint[MAXTYPES + 1];
  int *intp[MAXTYPES + 1];
  double *weight[MAXTYPES + 1];
  double emass[MAXTYPES + 1];
  double *spa_int[MAXTYPES + 1];       /* [numint][8] */
  int inter_num[MAXTYPES + 1];
  double *inter_pc[MAXTYPES + 1];      /* [ninter][3] */
  double *spa_inter[MAXTYPES + 1];     /* [ninter][8] */
  int node_list[MAXTYPES + 1][NPE];
  int nsubele;
  double *sub_pc;                      /* [nsub][8][3] */
  double *center_sub_pc;               /* [nsub][3] */
  double *spa_center_sub;              /* [nsub][8] */
  int *natom_sub;                      /* [nsub] */
  int *sub_first;                      /* offsets into the per-sub site lists */
  double *spa_inter_sub;               /* [total][8] */
  int *list_inter_sub;                 /* [total] */
  /* elements */
  int enlocal, enghost, emax_;
  double *ex, *nodex, *nodev, *nodef, *nodexhold;
  int *etype, *etag;
  double esize[MAXTYPES + 1], max_size;
  /* cutoffs */
  double cut_all, cut_allsq, cut_ele, cut_elesq, cut_subele, cut_subelesq;
  double cutghost[3], cutghostmulti[MAXTYPES + 1];
  /* comm */
  int nswap;
  swap_t swaps[64];
  /* bins */
  int nbinx, nbiny, nbinz, mbinx, mbiny, mbinz, mbinxlo, mbinylo, mbinzlo, mbins;
  double binsizex, binsizey, binsizez, bininvx, bininvy, bininvz;
  int nstencil;
  int *stencil;
  int *binhead, *bins, *ebinhead, *ebins;
  /* atom list (CSR) */
  int *numneigh;
  int *firstneigh;   /* offsets */
  ivec neigh;
  /* element list */
  int *enumneigh, *efirstneigh;
  ivec eneigh;
  /* integration-point list */
  int ninum;
  int *elist;        /* first row of each local element */
  ivec ip_num, ip_first, ip_j, ip_nj;
  /* pair */
  int pair_style;    /* 0 none, 1 lj/cut, 2 eam */
  double lj1[MAXTYPES + 1][MAXTYPES + 1], lj2[MAXTYPES + 1][MAXTYPES + 1];
  double lj3[MAXTYPES + 1][MAXTYPES + 1], lj4[MAXTYPES + 1][MAXTYPES + 1];
  double cutsq[MAXTYPES + 1][MAXTYPES + 1];
  /* eam */
  int nr, nrho;
  double dr, drho, rdr, rdrho, cutforcesq, eam_mass;
  double *frho_spline, *rhor_spline, *z2r_spline; /* [(n+1)*7] */
  double *rho, *fp, *erho;
  /* group masks and post-force fixes (fix_setforce.cpp, fix_viscous.cpp) */
  int *amask, *emask;
  int nfix;
  struct { int viscous, bit, set[3]; double val[3], gamma; } fixes[16];
  /* box deformation (engineering strain rate about the centre) */
  int deform;
  double erate[3], dL0[3], dc0[3];
  long long deform_t0;
  /* run state */
  long long ntimestep;
  int ago, nrebuild;
  int have_list, have_elists;
};

static int fail(orc_sys *s, const char *fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(s->err, sizeof(s->err), fmt, ap);
  va_end(ap);
  return -1;
}

orc_sys *orc_create(void) {
  orc_sys *s = (orc_sys *) calloc(1, sizeof(orc_sys));
  s->ftm2v = 1.0;
  s->dt = 0.005;
  s->skin = 0.3;
  s->every = 1;       /* neighbor.cpp:46-48 */
  s->delay = 10;
  s->dist_check = 1;
  s->nsplit = 2;      /* element.cpp:36 */
  s->periodic[0] = s->periodic[1] = s->periodic[2] = 1;
  return s;
}

void orc_destroy(orc_sys *s) {
  if (!s) return;
  free(s->amask);
  free(s->emask);
  free(s->x); free(s->v); free(s->f); free(s->type); free(s->tag); free(s->xhold);
  for (int t = 0; t <= MAXTYPES; t++) {
    free(s->intp[t]); free(s->weight[t]); free(s->spa_int[t]);
    free(s->inter_pc[t]); free(s->spa_inter[t]);
  }
  free(s->sub_pc); free(s->center_sub_pc); free(s->spa_center_sub); free(s->natom_sub);
  free(s->sub_first); free(s->spa_inter_sub); free(s->list_inter_sub);
  free(s->ex); free(s->nodex); free(s->nodev); free(s->nodef); free(s->nodexhold);
  free(s->etype); free(s->etag);
  for (int i = 0; i < 64; i++) { free(s->swaps[i].send.v); free(s->swaps[i].esend.v); }
  free(s->stencil); free(s->binhead); free(s->bins); free(s->ebinhead); free(s->ebins);
  free(s->numneigh); free(s->firstneigh); free(s->neigh.v);
  free(s->enumneigh); free(s->efirstneigh); free(s->eneigh.v);
  free(s->elist); free(s->ip_num.v); free(s->ip_first.v); free(s->ip_j.v); free(s->ip_nj.v);
  free(s->frho_spline); free(s->rhor_spline); free(s->z2r_spline);
  free(s->rho); free(s->fp); free(s->erho);
  free(s);
}

const char *orc_error(orc_sys *s) { return s->err; }

/* update.cpp:83-132 */
int orc_set_units(orc_sys *s, int metal) {
  if (metal) {
    s->ftm2v = 1.0 / 1.0364269e-4;
    s->dt = 0.001;
    s->skin = 2.0;
  } else {
    s->ftm2v = 1.0;
    s->dt = 0.005;
    s->skin = 0.3;
  }
  return 0;
}

int orc_set_timestep(orc_sys *s, double dt) { s->dt = dt; return 0; }

int orc_set_box(orc_sys *s, const double *lo, const double *hi, const int *periodic) {
  for (int d = 0; d < 3; d++) {
    if (!(lo[d] < hi[d])) return fail(s, "Box bounds are invalid");
    s->boxlo[d] = lo[d];
    s->boxhi[d] = hi[d];
    s->prd[d] = hi[d] - lo[d]; /* domain.cpp:312-314 */
    s->periodic[d] = periodic[d] ? 1 : 0;
  }
  return 0;
}

int orc_set_neighbor(orc_sys *s, double skin, int every, int delay, int check,
                     double binsize_user) {
  if (skin < 0.0) return fail(s, "Illegal neighbor command");
  if (every <= 0 || delay < 0) return fail(s, "Illegal neigh_modify command");
  s->skin = skin;
  s->every = every;
  s->delay = delay;
  s->dist_check = check ? 1 : 0;
  s->binsize_user = binsize_user;
  s->binsizeflag = binsize_user > 0.0;
  return 0;
}

int orc_set_elementsplit(orc_sys *s, int nsplit) {
  if (nsplit < 1) return fail(s, "Illegal elementsplit command");
  s->nsplit = nsplit;
  return 0;
}

int orc_set_atom_types(orc_sys *s, int ntypes, const double *mass) {
  if (ntypes < 1 || ntypes > MAXTYPES) return fail(s, "unsupported atom type count");
  s->ntypes = ntypes;
  for (int t = 1; t <= ntypes; t++) s->amass[t] = mass[t - 1];
  return 0;
}

static void grow_atoms(orc_sys *s, int n) {
  if (n <= s->amax) return;
  int cap = s->amax ? s->amax : 1024;
  while (cap < n) cap *= 2;
  s->x = (double *) realloc(s->x, (size_t) cap * 3 * sizeof(double));
  s->v = (double *) realloc(s->v, (size_t) cap * 3 * sizeof(double));
  s->f = (double *) realloc(s->f, (size_t) cap * 3 * sizeof(double));
  s->type = (int *) realloc(s->type, (size_t) cap * sizeof(int));
  s->tag = (int *) realloc(s->tag, (size_t) cap * sizeof(int));
  s->xhold = (double *) realloc(s->xhold, (size_t) cap * 3 * sizeof(double));
  s->rho = (double *) realloc(s->rho, (size_t) cap * sizeof(double));
  s->fp = (double *) realloc(s->fp, (size_t) cap * sizeof(double));
  s->amax = cap;
}

int orc_set_atoms(orc_sys *s, int n, const double *x, const double *v, const int *type) {
  grow_atoms(s, n > 0 ? n : 1);
  for (int i = 0; i < n; i++) {
    for (int d = 0; d < 3; d++) {
      s->x[3 * i + d] = x[3 * i + d];
      s->v[3 * i + d] = v ? v[3 * i + d] : 0.0;
      s->f[3 * i + d] = 0.0;
    }
    s->type[i] = type ? type[i] : 1;
    s->tag[i] = i + 1;
  }
  s->nlocal = n;
  s->nghost = 0;
  return 0;
}

/* shape function of parent coordinate (px,py,pz), node order of
   element.cpp:1340-1347, products evaluated left to right */
static void shape8(double px, double py, double pz, double *N) {
  N[0] = 0.125 * (1 - px) * (1 - py) * (1 - pz);
  N[1] = 0.125 * (1 + px) * (1 - py) * (1 - pz);
  N[2] = 0.125 * (1 + px) * (1 + py) * (1 - pz);
  N[3] = 0.125 * (1 - px) * (1 + py) * (1 - pz);
  N[4] = 0.125 * (1 - px) * (1 - py) * (1 + pz);
  N[5] = 0.125 * (1 + px) * (1 - py) * (1 + pz);
  N[6] = 0.125 * (1 + px) * (1 + py) * (1 + pz);
  N[7] = 0.125 * (1 - px) * (1 + py) * (1 + pz);
}

int orc_set_element_types(orc_sys *s, int ntypes, const int *nae, const int *numint,
                          const int *intp, const double *weight) {
  if (ntypes < 1 || ntypes > MAXTYPES) return fail(s, "unsupported element type count");
  s->netypes = ntypes;
  int off = 0;
  for (int t = 1; t <= ntypes; t++) {
    for (int d = 0; d < 3; d++) s->nae[t][d] = nae[3 * (t - 1) + d];
    if (s->nae[t][0] < 2 || s->nae[t][1] < 2 || s->nae[t][2] < 2)
      return fail(s, "Invalid naae values"); /* element.cpp:1106 */
    s->numint[t] = numint[t - 1];
    free(s->intp[t]);
    free(s->weight[t]);
    s->intp[t] = (int *) malloc((size_t) (s->numint[t] * 3 + 1) * sizeof(int));
    s->weight[t] = (double *) malloc((size_t) (s->numint[t] + 1) * sizeof(double));
    for (int m = 0; m < s->numint[t]; m++) {
      for (int d = 0; d < 3; d++) s->intp[t][3 * m + d] = intp[3 * (off + m) + d];
      s->weight[t][m] = weight[off + m];
    }
    off += s->numint[t];
  }
  return 0;
}

static void grow_elements(orc_sys *s, int n) {
  if (n <= s->emax_) return;
  int cap = s->emax_ ? s->emax_ : 256;
  while (cap < n) cap *= 2;
  s->ex = (double *) realloc(s->ex, (size_t) cap * 3 * sizeof(double));
  s->nodex = (double *) realloc(s->nodex, (size_t) cap * 24 * sizeof(double));
  s->nodev = (double *) realloc(s->nodev, (size_t) cap * 24 * sizeof(double));
  s->nodef = (double *) realloc(s->nodef, (size_t) cap * 24 * sizeof(double));
  s->nodexhold = (double *) realloc(s->nodexhold, (size_t) cap * 24 * sizeof(double));
  s->erho = (double *) realloc(s->erho, (size_t) cap * NPE * sizeof(double));
  s->etype = (int *) realloc(s->etype, (size_t) cap * sizeof(int));
  s->etag = (int *) realloc(s->etag, (size_t) cap * sizeof(int));
  s->emax_ = cap;
}

int orc_set_elements(orc_sys *s, int n, const int *etype, const double *centre,
                     const double *nodex, const double *nodev) {
  grow_elements(s, n > 0 ? n : 1);
  for (int i = 0; i < n; i++) {
    if (etype[i] < 1 || etype[i] > s->netypes)
      return fail(s, "Invalid atom type in Elements section of data file");
    s->etype[i] = etype[i];
    s->etag[i] = i + 1;
    for (int d = 0; d < 3; d++) s->ex[3 * i + d] = centre[3 * i + d];
    for (int k = 0; k < 24; k++) {
      s->nodex[24 * i + k] = nodex[24 * i + k];
      s->nodev[24 * i + k] = nodev ? nodev[24 * i + k] : 0.0;
      s->nodef[24 * i + k] = 0.0;
    }
  }
  s->enlocal = n;
  s->enghost = 0;
  return 0;
}

/* PairLJCut::init_one, pair_lj_cut.cpp:140-198 (mixing: pair.cpp:174-199,
   geometric by default, pair.cpp:61) */
int orc_set_lj(orc_sys *s, int ntypes, const double *eps, const double *sigma,
               const double *cut) {
  if (ntypes < 1 || ntypes > MAXTYPES) return fail(s, "unsupported atom type count");
  s->pair_style = 1;
  if (s->ntypes == 0) s->ntypes = ntypes;
  for (int i = 1; i <= ntypes; i++)
    for (int j = 1; j <= ntypes; j++) {
      double e = eps[(i - 1) * ntypes + (j - 1)];
      double sg = sigma[(i - 1) * ntypes + (j - 1)];
      double c = cut[(i - 1) * ntypes + (j - 1)];
      s->lj1[i][j] = 48.0 * e * pow(sg, 12.0);
      s->lj2[i][j] = 24.0 * e * pow(sg, 6.0);
      s->lj3[i][j] = 4.0 * e * pow(sg, 12.0);
      s->lj4[i][j] = 4.0 * e * pow(sg, 6.0);
      s->cutsq[i][j] = c * c;
    }
  return 0;
}

/* PairEAM::grab, pair_eam.cpp:255-267 */
static int grab(FILE *fp, int n, double *list) {
  char line[1024];
  int i = 0;
  while (i < n) {
    if (!fgets(line, sizeof(line), fp)) return -1;
    char *ptr = strtok(line, " \t\n\r\f");
    if (!ptr) continue;
    list[i++] = atof(ptr);
    while ((ptr = strtok(NULL, " \t\n\r\f")) && i < n) list[i++] = atof(ptr);
  }
  return 0;
}

/* PairEAM::interpolate, pair_eam.cpp:552-580; spline rows are 1-based */
static void interpolate(int n, double delta, const double *f, double *sp) {
#define S(m, k) sp[(m) * 7 + (k)]
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
#undef S
}

/* 4-point Lagrange regrid of one file table, pair_eam.cpp:356-377 */
static void regrid(int n, double delta, int nfile, double dfile, const double *src,
                   double *dst) {
  const double sixth = 1.0 / 6.0;
  for (int m = 1; m <= n; m++) {
    double r = (m - 1) * delta;
    double p = r / dfile + 1.0;
    int k = (int) p;
    k = k < nfile - 2 ? k : nfile - 2;
    k = k > 2 ? k : 2;
    p -= k;
    p = p < 2.0 ? p : 2.0;
    double cof1 = -sixth * p * (p - 1.0) * (p - 2.0);
    double cof2 = 0.5 * (p * p - 1.0) * (p - 2.0);
    double cof3 = -0.5 * p * (p + 1.0) * (p - 2.0);
    double cof4 = sixth * p * (p * p - 1.0);
    dst[m] = cof1 * src[k - 1] + cof2 * src[k] + cof3 * src[k + 1] + cof4 * src[k + 2];
  }
}

/* PairEAM::read_file + file2array + array2spline + init_one for one funcfl-variant
   file mapped to every type (pair_eam.cpp:197-248, 311-523, 527-550, 285-307) */
int orc_set_eam_file(orc_sys *s, const char *path) {
  FILE *fp = fopen(path, "r");
  if (!fp) return fail(s, "Cannot open EAM potential file %s", path);
  char line[1024];
  int tmp, nrho_f, nr_f;
  double mass, drho_f, dr_f, cut;
  if (!fgets(line, sizeof(line), fp) || !fgets(line, sizeof(line), fp)) {
    fclose(fp);
    return fail(s, "EAM file truncated");
  }
  sscanf(line, "%d %lg", &tmp, &mass);
  if (!fgets(line, sizeof(line), fp)) { fclose(fp); return fail(s, "EAM file truncated"); }
  sscanf(line, "%d %lg %d %lg %lg", &nrho_f, &drho_f, &nr_f, &dr_f, &cut);
  double *F = (double *) calloc((size_t) nrho_f + 1, sizeof(double));
  double *R = (double *) calloc((size_t) nr_f + 1, sizeof(double));
  double *Z = (double *) calloc((size_t) nr_f + 1, sizeof(double));
  int bad = grab(fp, nrho_f, F + 1) || grab(fp, nr_f, R + 1) || grab(fp, nr_f, Z + 1);
  fclose(fp);
  if (bad) { free(F); free(R); free(Z); return fail(s, "EAM file truncated"); }

  s->pair_style = 2;
  s->eam_mass = mass;
  s->dr = dr_f;
  s->drho = drho_f;
  double rmax = (nr_f - 1) * dr_f;
  double rhomax = (nrho_f - 1) * drho_f;
  s->nr = (int) (rmax / s->dr + 0.5);
  s->nrho = (int) (rhomax / s->drho + 0.5);
  double *frho = (double *) calloc((size_t) s->nrho + 1, sizeof(double));
  double *rhor = (double *) calloc((size_t) s->nr + 1, sizeof(double));
  double *z2r = (double *) calloc((size_t) s->nr + 1, sizeof(double));
  regrid(s->nrho, s->drho, nrho_f, drho_f, F, frho);
  regrid(s->nr, s->dr, nr_f, dr_f, R, rhor);
  regrid(s->nr, s->dr, nr_f, dr_f, Z, z2r);
  s->rdr = 1.0 / s->dr;
  s->rdrho = 1.0 / s->drho;
  free(s->frho_spline); free(s->rhor_spline); free(s->z2r_spline);
  s->frho_spline = (double *) calloc((size_t) (s->nrho + 1) * 7, sizeof(double));
  s->rhor_spline = (double *) calloc((size_t) (s->nr + 1) * 7, sizeof(double));
  s->z2r_spline = (double *) calloc((size_t) (s->nr + 1) * 7, sizeof(double));
  interpolate(s->nrho, s->drho, frho, s->frho_spline);
  interpolate(s->nr, s->dr, rhor, s->rhor_spline);
  interpolate(s->nr, s->dr, z2r, s->z2r_spline);
  s->cutforcesq = cut * cut;
  /* pair_coeff sets the atom and element masses (pair_eam.cpp:152-161,
     element.cpp:1117-1123) */
  for (int t = 1; t <= MAXTYPES; t++) s->amass[t] = mass;
  free(F); free(R); free(Z); free(frho); free(rhor); free(z2r);
  return 0;
}

/* ---------------------------------------------------------------- tables */

/* Element::inter_ele + shape_array_inter_ele, element.cpp:1361-1423 */
static void tables_inter(orc_sys *s) {
  for (int t = 1; t <= s->netypes; t++) {
    int nx = s->nae[t][0], ny = s->nae[t][1], nz = s->nae[t][2];
    int nn = nx * ny * nz;
    s->inter_num[t] = nn;
    free(s->inter_pc[t]);
    free(s->spa_inter[t]);
    s->inter_pc[t] = (double *) malloc((size_t) nn * 3 * sizeof(double));
    s->spa_inter[t] = (double *) malloc((size_t) nn * NPE * sizeof(double));
    double inx = 2 / ((double) nx - 1);
    double iny = 2 / ((double) ny - 1);
    double inz = 2 / ((double) nz - 1);
    int inum = 0;
    for (int ii = 0; ii < nx; ii++)
      for (int jj = 0; jj < ny; jj++)
        for (int kk = 0; kk < nz; kk++) {
          double *pc = s->inter_pc[t] + 3 * inum;
          pc[0] = inx * (double) ii - 1;
          pc[1] = iny * (double) jj - 1;
          pc[2] = inz * (double) kk - 1;
          shape8(pc[0], pc[1], pc[2], s->spa_inter[t] + NPE * inum);
          inum++;
        }
  }
}

/* Element::intp_pcoord + shape_array_int, element.cpp:1170-1191, 1326-1354 */
static void tables_int(orc_sys *s) {
  for (int t = 1; t <= s->netypes; t++) {
    int nint = s->numint[t];
    free(s->spa_int[t]);
    s->spa_int[t] = (double *) malloc((size_t) (nint + 1) * NPE * sizeof(double));
    double dx = 2 / ((double) s->nae[t][0] - 1);
    double dy = 2 / ((double) s->nae[t][1] - 1);
    double dz = 2 / ((double) s->nae[t][2] - 1);
    for (int jj = 0; jj < nint; jj++) {
      double px = dx * ((double) s->intp[t][3 * jj + 0]) - 1;
      double py = dy * ((double) s->intp[t][3 * jj + 1]) - 1;
      double pz = dz * ((double) s->intp[t][3 * jj + 2]) - 1;
      shape8(px, py, pz, s->spa_int[t] + NPE * jj);
    }
  }
}

/* Element::specify_sub_ele_pc, count_sub_element, shape_array_inter_subele
   (element.cpp:725-906); sub-element tables use type-1 geometry only, as the
   reference does (inter_in_ele[0], element.cpp:786-787, 835-836) */
static int tables_sub(orc_sys *s) {
  int ns = s->nsplit;
  int nsub = ns * ns * ns;
  s->nsubele = nsub;
  double ls = 2.0 / ns;
  free(s->sub_pc); free(s->center_sub_pc); free(s->spa_center_sub); free(s->natom_sub);
  free(s->sub_first); free(s->spa_inter_sub); free(s->list_inter_sub);
  s->sub_pc = (double *) malloc((size_t) nsub * NPE * 3 * sizeof(double));
  s->center_sub_pc = (double *) malloc((size_t) nsub * 3 * sizeof(double));
  s->spa_center_sub = (double *) malloc((size_t) nsub * NPE * sizeof(double));
  s->natom_sub = (int *) calloc((size_t) nsub, sizeof(int));
  s->sub_first = (int *) calloc((size_t) nsub + 1, sizeof(int));
#define PC(i, l, d) s->sub_pc[((i) * NPE + (l)) * 3 + (d)]
  const double c0[8][3] = {{-1.0, -1.0, -1.0}, {ls - 1.0, -1.0, -1.0},
                           {ls - 1.0, ls - 1.0, -1.0}, {-1.0, ls - 1.0, -1.0},
                           {-1.0, -1.0, ls - 1.0}, {ls - 1.0, -1.0, ls - 1.0},
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
  for (int i = 0; i < nsub; i++) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int l = 0; l < NPE; l++)
      for (int d = 0; d < 3; d++) c[d] += PC(i, l, d);
    for (int d = 0; d < 3; d++) s->center_sub_pc[3 * i + d] = c[d] / NPE;
  }
  int ninter = s->inter_num[1];
  const double *pinter = s->inter_pc[1];
  double lo[3], hi[3];
  /* count, then fill */
  for (int pass = 0; pass < 2; pass++) {
    for (int i = 0; i < nsub; i++) {
      lo[0] = PC(i, 0, 0); hi[0] = PC(i, 1, 0);
      lo[1] = PC(i, 0, 1); hi[1] = PC(i, 3, 1);
      lo[2] = PC(i, 0, 2); hi[2] = PC(i, 4, 2);
      for (int d = 0; d < 3; d++) {
        if (lo[d] < -0.99) lo[d] = -1.01;
        if (hi[d] > 0.99) hi[d] = 1.01;
      }
      int cnt = 0;
      for (int j = 0; j < ninter; j++) {
        const double *p = pinter + 3 * j;
        if (p[0] > lo[0] && p[0] <= hi[0] && p[1] > lo[1] && p[1] <= hi[1] && p[2] > lo[2] &&
            p[2] <= hi[2]) {
          if (pass == 1) {
            int slot = s->sub_first[i] + cnt;
            shape8(p[0], p[1], p[2], s->spa_inter_sub + NPE * slot);
            s->list_inter_sub[slot] = j;
          }
          cnt++;
        }
      }
      if (pass == 0) s->natom_sub[i] = cnt;
    }
    if (pass == 0) {
      int tot = 0;
      for (int i = 0; i < nsub; i++) {
        s->sub_first[i] = tot;
        tot += s->natom_sub[i];
      }
      s->sub_first[nsub] = tot;
      if (tot != ninter) return fail(s, "sub atom total donot match total atom number");
      s->spa_inter_sub = (double *) malloc((size_t) (tot + 1) * NPE * sizeof(double));
      s->list_inter_sub = (int *) malloc((size_t) (tot + 1) * sizeof(int));
    }
  }
  for (int i = 0; i < nsub; i++)
    shape8(s->center_sub_pc[3 * i], s->center_sub_pc[3 * i + 1], s->center_sub_pc[3 * i + 2],
           s->spa_center_sub + NPE * i);
#undef PC
  return 0;
}

/* Element::find_node_list, element.cpp:1296-1319 */
static int tables_node_list(orc_sys *s) {
  for (int t = 1; t <= s->netypes; t++) {
    for (int jj = 0; jj < NPE; jj++) {
      int kk;
      for (kk = 0; kk < s->numint[t]; kk++)
        if (fabs(s->spa_int[t][NPE * kk + jj] - 1.0) < TOLNODE) {
          s->node_list[t][jj] = kk;
          break;
        }
      if (kk == s->numint[t]) return fail(s, "didn't contain all node integration point");
    }
  }
  return 0;
}

/* Element::element_size, element.cpp:567-625 (running max, never reset) */
static int element_size(orc_sys *s) {
  double mx[MAXTYPES + 1];
  for (int t = 1; t <= s->netypes; t++) mx[t] = 0.0;
  double length = 0.0;
  for (int i = 0; i < s->enlocal; i++) {
    const double *nx = s->nodex + 24 * i;
    for (int j = 0; j < 4; j++) {
      int o = j < 2 ? j + 6 : j + 2;
      double lx = nx[3 * j] - nx[3 * o];
      double ly = nx[3 * j + 1] - nx[3 * o + 1];
      double lz = nx[3 * j + 2] - nx[3 * o + 2];
      double l = sqrt(lx * lx + ly * ly + lz * lz);
      length = length > l ? length : l;
    }
    mx[s->etype[i]] = length;
  }
  for (int t = 1; t <= s->netypes; t++) {
    s->esize[t] = mx[t];
    s->max_size = s->max_size > s->esize[t] ? s->max_size : s->esize[t];
  }
  for (int i = 0; i < s->enlocal; i++) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < NPE; j++)
      for (int d = 0; d < 3; d++) c[d] += s->nodex[24 * i + 3 * j + d];
    for (int d = 0; d < 3; d++) c[d] = c[d] / NPE;
    double dist = (c[0] - s->ex[3 * i]) * (c[0] - s->ex[3 * i]) +
                  (c[1] - s->ex[3 * i + 1]) * (c[1] - s->ex[3 * i + 1]) +
                  (c[2] - s->ex[3 * i + 2]) * (c[2] - s->ex[3 * i + 2]);
    if (dist > TOLNODE) return fail(s, "element data has error");
  }
  return 0;
}

/* Neighbor::setup_cut, neighbor.cpp:284-293 */
static void setup_cut(orc_sys *s) {
  s->cut_all = s->cutneighmax + s->max_size;
  s->cut_allsq = s->cut_all * s->cut_all;
  s->cut_ele = s->cutneighmax + s->max_size / 2;
  s->cut_elesq = s->cut_ele * s->cut_ele;
  s->cut_subele = s->cutneighmax + s->max_size / (2 * s->nsplit);
  s->cut_subelesq = s->cut_subele * s->cut_subele;
}

/* CommBrick::setup for one proc, comm_brick.cpp:182-367 */
static void comm_setup(orc_sys *s) {
  double cut = s->cutneighmax; /* MAX(cutneighmax, cutghostuser = 0) */
  for (int d = 0; d < 3; d++) s->cutghost[d] = s->cut_all;
  for (int t = 1; t <= s->netypes; t++) s->cutghostmulti[t] = cut + s->esize[t];
  int maxneed[3];
  for (int d = 0; d < 3; d++) {
    maxneed[d] = (int) (s->cutghost[d] * 1 / s->prd[d]) + 1;
    if (!s->periodic[d]) maxneed[d] = maxneed[d] < 0 ? maxneed[d] : 0; /* MIN(.., procgrid-1) */
  }
  int iswap = 0;
  for (int dim = 0; dim < 3; dim++)
    for (int ineed = 0; ineed < 2 * maxneed[dim]; ineed++) {
      swap_t *w = &s->swaps[iswap];
      w->dim = dim;
      double sublo = s->boxlo[dim], subhi = s->boxhi[dim];
      if (ineed % 2 == 0) {
        w->lo = ineed < 2 ? -BIGV : 0.5 * (sublo + subhi);
        w->hi = sublo + s->cutghost[dim];
        for (int t = 1; t <= s->netypes; t++) {
          w->mlo[t] = ineed < 2 ? -BIGV : 0.5 * (sublo + subhi);
          w->mhi[t] = sublo + s->cutghostmulti[t];
        }
        w->pbc = 1;
      } else {
        w->lo = subhi - s->cutghost[dim];
        w->hi = ineed < 2 ? BIGV : 0.5 * (sublo + subhi);
        for (int t = 1; t <= s->netypes; t++) {
          w->mlo[t] = subhi - s->cutghostmulti[t];
          w->mhi[t] = ineed < 2 ? BIGV : 0.5 * (sublo + subhi);
        }
        w->pbc = -1;
      }
      iswap++;
    }
  s->nswap = iswap;
}

/* CommBrick::borders, comm_brick.cpp:641-914: ghosts appended in swap order,
   coordinates x + pbc*prd (atom_vec_atomic.cpp:185-226, element.cpp:923-955) */
static void borders(orc_sys *s) {
  s->nghost = 0;
  int iswap = 0, nfirst = 0, nlast = 0;
  for (int dim = 0; dim < 3; dim++) {
    nlast = 0;
    for (; iswap < s->nswap && s->swaps[iswap].dim == dim; iswap++) {
      swap_t *w = &s->swaps[iswap];
      /* even ineed (send toward -dim, image +prd) starts a new source range */
      if (w->pbc == 1) {
        nfirst = nlast;
        nlast = s->nlocal + s->nghost;
      }
      w->send.n = 0;
      for (int i = nfirst; i < nlast; i++)
        if (s->x[3 * i + dim] >= w->lo && s->x[3 * i + dim] <= w->hi) iv_push(&w->send, i);
      int n0 = s->nlocal + s->nghost;
      grow_atoms(s, n0 + w->send.n);
      double d[3] = {0.0, 0.0, 0.0};
      if (w->pbc) {
        d[0] = (dim == 0 ? w->pbc : 0) * s->prd[0];
        d[1] = (dim == 1 ? w->pbc : 0) * s->prd[1];
        d[2] = (dim == 2 ? w->pbc : 0) * s->prd[2];
      }
      for (int m = 0; m < w->send.n; m++) {
        int j = w->send.v[m];
        int g = n0 + m;
        s->x[3 * g + 0] = s->x[3 * j + 0] + d[0];
        s->x[3 * g + 1] = s->x[3 * j + 1] + d[1];
        s->x[3 * g + 2] = s->x[3 * j + 2] + d[2];
        s->tag[g] = s->tag[j];
        s->type[g] = s->type[j];
      }
      w->firstrecv = n0;
      s->nghost += w->send.n;
    }
  }
  /* elements (comm_brick.cpp:804-905) */
  s->enghost = 0;
  iswap = 0;
  for (int dim = 0; dim < 3; dim++) {
    nlast = 0;
    for (; iswap < s->nswap && s->swaps[iswap].dim == dim; iswap++) {
      swap_t *w = &s->swaps[iswap];
      if (w->pbc == 1) {
        nfirst = nlast;
        nlast = s->enlocal + s->enghost;
      }
      w->esend.n = 0;
      for (int i = nfirst; i < nlast; i++) {
        int t = s->etype[i];
        if (s->ex[3 * i + dim] >= w->mlo[t] && s->ex[3 * i + dim] <= w->mhi[t])
          iv_push(&w->esend, i);
      }
      int n0 = s->enlocal + s->enghost;
      grow_elements(s, n0 + w->esend.n);
      double d[3] = {0.0, 0.0, 0.0};
      if (w->pbc) {
        d[0] = (dim == 0 ? w->pbc : 0) * s->prd[0];
        d[1] = (dim == 1 ? w->pbc : 0) * s->prd[1];
        d[2] = (dim == 2 ? w->pbc : 0) * s->prd[2];
      }
      for (int m = 0; m < w->esend.n; m++) {
        int j = w->esend.v[m];
        int g = n0 + m;
        for (int c = 0; c < 3; c++) s->ex[3 * g + c] = s->ex[3 * j + c] + d[c];
        for (int k = 0; k < NPE; k++)
          for (int c = 0; c < 3; c++)
            s->nodex[24 * g + 3 * k + c] = s->nodex[24 * j + 3 * k + c] + d[c];
        s->etag[g] = s->etag[j];
        s->etype[g] = s->etype[j];
      }
      w->efirstrecv = n0;
      s->enghost += w->esend.n;
    }
  }
}

/* CommBrick::forward_comm / eforward_comm (comm_brick.cpp:1017-1112) */
static void forward_comm(orc_sys *s) {
  for (int iswap = 0; iswap < s->nswap; iswap++) {
    swap_t *w = &s->swaps[iswap];
    int dim = w->dim;
    double d[3] = {0.0, 0.0, 0.0};
    if (w->pbc) {
      d[0] = (dim == 0 ? w->pbc : 0) * s->prd[0];
      d[1] = (dim == 1 ? w->pbc : 0) * s->prd[1];
      d[2] = (dim == 2 ? w->pbc : 0) * s->prd[2];
    }
    for (int m = 0; m < w->send.n; m++) {
      int j = w->send.v[m], g = w->firstrecv + m;
      for (int c = 0; c < 3; c++) s->x[3 * g + c] = s->x[3 * j + c] + d[c];
    }
  }
}

static void eforward_comm(orc_sys *s) {
  for (int iswap = 0; iswap < s->nswap; iswap++) {
    swap_t *w = &s->swaps[iswap];
    int dim = w->dim;
    double d[3] = {0.0, 0.0, 0.0};
    if (w->pbc) {
      d[0] = (dim == 0 ? w->pbc : 0) * s->prd[0];
      d[1] = (dim == 1 ? w->pbc : 0) * s->prd[1];
      d[2] = (dim == 2 ? w->pbc : 0) * s->prd[2];
    }
    for (int m = 0; m < w->esend.n; m++) {
      int j = w->esend.v[m], g = w->efirstrecv + m;
      for (int k = 0; k < NPE; k++)
        for (int c = 0; c < 3; c++)
          s->nodex[24 * g + 3 * k + c] = s->nodex[24 * j + 3 * k + c] + d[c];
    }
  }
}

/* Neighbor::bin_distance, neighbor.cpp:811-826 */
static double bin_distance(orc_sys *s, int i, int j, int k) {
  double dx, dy, dz;
  if (i > 0) dx = (i - 1) * s->binsizex;
  else if (i == 0) dx = 0.0;
  else dx = (i + 1) * s->binsizex;
  if (j > 0) dy = (j - 1) * s->binsizey;
  else if (j == 0) dy = 0.0;
  else dy = (j + 1) * s->binsizey;
  if (k > 0) dz = (k - 1) * s->binsizez;
  else if (k == 0) dz = 0.0;
  else dz = (k + 1) * s->binsizez;
  return dx * dx + dy * dy + dz * dz;
}

/* Neighbor::setup_bins, neighbor.cpp:828-976 */
static int setup_bins(orc_sys *s) {
  double bsublo[3], bsubhi[3], bbox[3];
  for (int d = 0; d < 3; d++) {
    bsublo[d] = s->boxlo[d] - s->cutghost[d] - s->max_size / 2.0;
    bsubhi[d] = s->boxhi[d] + s->cutghost[d] + s->max_size / 2.0;
    bbox[d] = s->boxhi[d] - s->boxlo[d];
  }
  double binsize_optimal = s->binsizeflag ? s->binsize_user : 0.5 * s->cutneighmax;
  if (binsize_optimal == 0.0) binsize_optimal = bbox[0];
  double binsizeinv = 1.0 / binsize_optimal;
  s->nbinx = (int) (bbox[0] * binsizeinv);
  s->nbiny = (int) (bbox[1] * binsizeinv);
  s->nbinz = (int) (bbox[2] * binsizeinv);
  if (s->nbinx == 0) s->nbinx = 1;
  if (s->nbiny == 0) s->nbiny = 1;
  if (s->nbinz == 0) s->nbinz = 1;
  s->binsizex = bbox[0] / s->nbinx;
  s->binsizey = bbox[1] / s->nbiny;
  s->binsizez = bbox[2] / s->nbinz;
  s->bininvx = 1.0 / s->binsizex;
  s->bininvy = 1.0 / s->binsizey;
  s->bininvz = 1.0 / s->binsizez;
  if (binsize_optimal * s->bininvx > 100 || binsize_optimal * s->bininvy > 100 ||
      binsize_optimal * s->bininvz > 100)
    return fail(s, "Cannot use neighbor bins - box size << cutoff");
  int lo[3], hi[3];
  double inv[3] = {s->bininvx, s->bininvy, s->bininvz};
  for (int d = 0; d < 3; d++) {
    double coord = bsublo[d] - SMALLB * bbox[d];
    lo[d] = (int) ((coord - s->boxlo[d]) * inv[d]);
    if (coord < s->boxlo[d]) lo[d] = lo[d] - 1;
    coord = bsubhi[d] + SMALLB * bbox[d];
    hi[d] = (int) ((coord - s->boxlo[d]) * inv[d]);
    lo[d] -= 1;
    hi[d] += 1;
  }
  s->mbinxlo = lo[0]; s->mbinylo = lo[1]; s->mbinzlo = lo[2];
  s->mbinx = hi[0] - lo[0] + 1;
  s->mbiny = hi[1] - lo[1] + 1;
  s->mbinz = hi[2] - lo[2] + 1;
  long long bb = (long long) s->mbinx * s->mbiny * s->mbinz;
  if (bb > 2147483647LL) return fail(s, "Too many neighbor bins");
  s->mbins = (int) bb;
  s->binhead = (int *) realloc(s->binhead, (size_t) s->mbins * sizeof(int));
  s->ebinhead = (int *) realloc(s->ebinhead, (size_t) s->mbins * sizeof(int));
  int sx = (int) (s->cutneighmax * s->bininvx);
  if (sx * s->binsizex < s->cutneighmax) sx++;
  int sy = (int) (s->cutneighmax * s->bininvy);
  if (sy * s->binsizey < s->cutneighmax) sy++;
  int sz = (int) (s->cutneighmax * s->bininvz);
  if (sz * s->binsizez < s->cutneighmax) sz++;
  int smax = (2 * sx + 1) * (2 * sy + 1) * (2 * sz + 1);
  s->stencil = (int *) realloc(s->stencil, (size_t) smax * sizeof(int));
  s->nstencil = 0;
  for (int k = -sz; k <= sz; k++)
    for (int j = -sy; j <= sy; j++)
      for (int i = -sx; i <= sx; i++)
        if (bin_distance(s, i, j, k) < s->cutneighmaxsq)
          s->stencil[s->nstencil++] = k * s->mbiny * s->mbinx + j * s->mbinx + i;
  return 0;
}

/* Neighbor::coord2bin, neighbor.cpp:688-717 */
static int coord2bin(orc_sys *s, const double *x) {
  int ix, iy, iz;
  if (x[0] >= s->boxhi[0]) ix = (int) ((x[0] - s->boxhi[0]) * s->bininvx) + s->nbinx;
  else if (x[0] >= s->boxlo[0]) {
    ix = (int) ((x[0] - s->boxlo[0]) * s->bininvx);
    ix = ix < s->nbinx - 1 ? ix : s->nbinx - 1;
  } else ix = (int) ((x[0] - s->boxlo[0]) * s->bininvx) - 1;
  if (x[1] >= s->boxhi[1]) iy = (int) ((x[1] - s->boxhi[1]) * s->bininvy) + s->nbiny;
  else if (x[1] >= s->boxlo[1]) {
    iy = (int) ((x[1] - s->boxlo[1]) * s->bininvy);
    iy = iy < s->nbiny - 1 ? iy : s->nbiny - 1;
  } else iy = (int) ((x[1] - s->boxlo[1]) * s->bininvy) - 1;
  if (x[2] >= s->boxhi[2]) iz = (int) ((x[2] - s->boxhi[2]) * s->bininvz) + s->nbinz;
  else if (x[2] >= s->boxlo[2]) {
    iz = (int) ((x[2] - s->boxlo[2]) * s->bininvz);
    iz = iz < s->nbinz - 1 ? iz : s->nbinz - 1;
  } else iz = (int) ((x[2] - s->boxlo[2]) * s->bininvz) - 1;
  return (iz - s->mbinzlo) * s->mbiny * s->mbinx + (iy - s->mbinylo) * s->mbinx +
         (ix - s->mbinxlo);
}

/* Neighbor::init (cutoffs, neighbor.cpp:297-374) + Element::init tables +
   Verlet::setup through comm->borders (verlet.cpp:70-90) */
int orc_setup(orc_sys *s) {
  s->cutneighmax = s->skin;  /* per-type cutoff is hard-coded 0 (neighbor.cpp:357-364) */
  s->cutneighmaxsq = s->cutneighmax * s->cutneighmax;
  s->triggersq = 0.25 * s->skin * s->skin;
  if (s->enlocal > 0) {
    for (int t = 1; t <= s->netypes; t++) {
      /* element mass, element.cpp:1104 / 1117-1123 */
      s->emass[t] = s->nae[t][0] * s->nae[t][1] * s->nae[t][2] * s->amass[1];
    }
    if (element_size(s)) return -1;
    tables_inter(s);
    tables_int(s);
    if (tables_sub(s)) return -1;
    if (s->pair_style == 2 && tables_node_list(s)) return -1;
  }
  s->cut_all = s->cutneighmax + s->max_size;
  s->cut_ele = s->cutneighmax + s->max_size / 2;
  s->cut_allsq = s->cut_all * s->cut_all;
  s->cut_elesq = s->cut_ele * s->cut_ele;
  comm_setup(s);
  if (setup_bins(s)) return -1;
  borders(s);
  s->ago = 0;
  s->ntimestep = 0;
  return 0;
}

/* Neighbor::bin_atoms + half_bin_no_newton (a FULL list), neighbor.cpp:546-674 */
int orc_atom_list(orc_sys *s) {
  int nall = s->nlocal + s->nghost;
  s->bins = (int *) realloc(s->bins, (size_t) (nall + 1) * sizeof(int));
  for (int i = 0; i < s->mbins; i++) s->binhead[i] = -1;
  /* the reference bins without a range check (an atom that left the bin
     grid indexes past binhead); here that is an error, as on the device */
  for (int i = nall - 1; i >= 0; i--) {
    int ib = coord2bin(s, s->x + 3 * i);
    if (ib < 0 || ib >= s->mbins) return fail(s, "atoms outside the bin grid (lost atoms)");
    s->bins[i] = s->binhead[ib];
    s->binhead[ib] = i;
  }
  s->numneigh = (int *) realloc(s->numneigh, (size_t) (s->nlocal + 1) * sizeof(int));
  s->firstneigh = (int *) realloc(s->firstneigh, (size_t) (s->nlocal + 1) * sizeof(int));
  s->neigh.n = 0;
  for (int i = 0; i < s->nlocal; i++) {
    double xt = s->x[3 * i], yt = s->x[3 * i + 1], zt = s->x[3 * i + 2];
    int ib = coord2bin(s, s->x + 3 * i);
    int n = 0;
    s->firstneigh[i] = s->neigh.n;
    for (int k = 0; k < s->nstencil; k++)
      for (int j = s->binhead[ib + s->stencil[k]]; j >= 0; j = s->bins[j]) {
        if (i == j) continue;
        double dx = xt - s->x[3 * j], dy = yt - s->x[3 * j + 1], dz = zt - s->x[3 * j + 2];
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq <= s->cutneighmaxsq) {
          iv_push(&s->neigh, j);
          n++;
        }
      }
    s->numneigh[i] = n;
  }
  for (int i = 0; i < s->nlocal; i++)
    for (int d = 0; d < 3; d++) s->xhold[3 * i + d] = s->x[3 * i + d];
  s->have_list = 1;
  return 0;
}

/* Neighbor::ebuild + element_neighbor + nbuild + node_neighbor
   (neighbor.cpp:1022-1106, element_neighbor.cpp:11-75, full_node_neighbor.cpp:19-239) */
int orc_elem_lists(orc_sys *s) {
  setup_cut(s);
  int nall = s->enlocal + s->enghost;
  if (s->dist_check)
    memcpy(s->nodexhold, s->nodex, (size_t) s->enlocal * 24 * sizeof(double));
  s->ebins = (int *) realloc(s->ebins, (size_t) (nall + 1) * sizeof(int));
  for (int i = 0; i < s->mbins; i++) s->ebinhead[i] = -1;
  for (int i = nall - 1; i >= 0; i--) {
    int ib = coord2bin(s, s->ex + 3 * i);
    if (ib < 0 || ib >= s->mbins) return fail(s, "elements outside the bin grid (lost elements)");
    s->ebins[i] = s->ebinhead[ib];
    s->ebinhead[ib] = i;
  }
  s->enumneigh = (int *) realloc(s->enumneigh, (size_t) (s->enlocal + 1) * sizeof(int));
  s->efirstneigh = (int *) realloc(s->efirstneigh, (size_t) (s->enlocal + 1) * sizeof(int));
  s->eneigh.n = 0;
  for (int i = 0; i < s->enlocal; i++) {
    double xt = s->ex[3 * i], yt = s->ex[3 * i + 1], zt = s->ex[3 * i + 2];
    int ib = coord2bin(s, s->ex + 3 * i);
    int n = 0;
    s->efirstneigh[i] = s->eneigh.n;
    for (int k = 0; k < s->nstencil; k++)
      for (int j = s->ebinhead[ib + s->stencil[k]]; j >= 0; j = s->ebins[j]) {
        if (j == i) continue;
        double dx = xt - s->ex[3 * j], dy = yt - s->ex[3 * j + 1], dz = zt - s->ex[3 * j + 2];
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq <= s->cut_allsq) {
          iv_push(&s->eneigh, j);
          n++;
        }
      }
    s->enumneigh[i] = n;
  }

  /* node_neighbor */
  s->elist = (int *) realloc(s->elist, (size_t) (s->enlocal + 1) * sizeof(int));
  s->ip_num.n = s->ip_first.n = s->ip_j.n = s->ip_nj.n = 0;
  int ninum = 0;
  double cutsq = s->cutneighmaxsq;
  for (int i = 0; i < s->enlocal; i++) {
    s->elist[i] = ninum;
    int t = s->etype[i];
    const double *nxi = s->nodex + 24 * i;
    for (int jj = 0; jj < s->numint[t]; jj++) {
      const double *N = s->spa_int[t] + NPE * jj;
      double ix = 0, iy = 0, iz = 0;
      for (int kk = 0; kk < NPE; kk++) {
        ix += N[kk] * nxi[3 * kk];
        iy += N[kk] * nxi[3 * kk + 1];
        iz += N[kk] * nxi[3 * kk + 2];
      }
      int n = 0;
      iv_push(&s->ip_first, s->ip_j.n);
      for (int ll = 0; ll < s->enumneigh[i]; ll++) {
        int j = s->eneigh.v[s->efirstneigh[i] + ll];
        const double *xj = s->ex + 3 * j;
        const double *nxj = s->nodex + 24 * j;
        double npdis = (ix - xj[0]) * (ix - xj[0]) + (iy - xj[1]) * (iy - xj[1]) +
                       (iz - xj[2]) * (iz - xj[2]);
        if (npdis <= s->cut_elesq) {
          for (int isub = 0; isub < s->nsubele; isub++) {
            const double *C = s->spa_center_sub + NPE * isub;
            double sx = 0.0, sy = 0.0, sz = 0.0;
            for (int kk = 0; kk < NPE; kk++) {
              sx += C[kk] * nxj[3 * kk];
              sy += C[kk] * nxj[3 * kk + 1];
              sz += C[kk] * nxj[3 * kk + 2];
            }
            double nps = (ix - sx) * (ix - sx) + (iy - sy) * (iy - sy) + (iz - sz) * (iz - sz);
            if (nps <= s->cut_subelesq) {
              for (int mm = 0; mm < s->natom_sub[isub]; mm++) {
                int slot = s->sub_first[isub] + mm;
                const double *M = s->spa_inter_sub + NPE * slot;
                double jx = 0, jy = 0, jz = 0;
                for (int kk = 0; kk < NPE; kk++) {
                  jx += M[kk] * nxj[3 * kk];
                  jy += M[kk] * nxj[3 * kk + 1];
                  jz += M[kk] * nxj[3 * kk + 2];
                }
                double dx = jx - ix, dy = jy - iy, dz = jz - iz;
                double rsq = dx * dx + dy * dy + dz * dz;
                if (rsq <= cutsq) {
                  iv_push(&s->ip_j, j);
                  iv_push(&s->ip_nj, s->list_inter_sub[slot]);
                  n++;
                }
              }
            }
          }
        }
      }
      /* self element */
      for (int isub = 0; isub < s->nsubele; isub++) {
        const double *C = s->spa_center_sub + NPE * isub;
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int kk = 0; kk < NPE; kk++) {
          sx += C[kk] * nxi[3 * kk];
          sy += C[kk] * nxi[3 * kk + 1];
          sz += C[kk] * nxi[3 * kk + 2];
        }
        double nps = (ix - sx) * (ix - sx) + (iy - sy) * (iy - sy) + (iz - sz) * (iz - sz);
        if (nps <= s->cut_subelesq) {
          for (int mm = 0; mm < s->natom_sub[isub]; mm++) {
            int slot = s->sub_first[isub] + mm;
            const double *M = s->spa_inter_sub + NPE * slot;
            double jx = 0, jy = 0, jz = 0;
            for (int kk = 0; kk < NPE; kk++) {
              jx += M[kk] * nxi[3 * kk];
              jy += M[kk] * nxi[3 * kk + 1];
              jz += M[kk] * nxi[3 * kk + 2];
            }
            double dx = jx - ix, dy = jy - iy, dz = jz - iz;
            double rsq = dx * dx + dy * dy + dz * dz;
            if (rsq <= cutsq && rsq > 1.0e-4) {
              iv_push(&s->ip_j, i);
              iv_push(&s->ip_nj, s->list_inter_sub[slot]);
              n++;
            }
          }
        }
      }
      iv_push(&s->ip_num, n);
      ninum++;
    }
  }
  s->ninum = ninum;
  s->have_elists = 1;
  return 0;
}

/* forward comm of one value per atom / 8 per element through the swap chain
   (comm_brick.cpp:941-1010, pair_eam.cpp:1145-1199) */
static void forward_fp(orc_sys *s) {
  for (int iswap = 0; iswap < s->nswap; iswap++) {
    swap_t *w = &s->swaps[iswap];
    for (int m = 0; m < w->send.n; m++) s->fp[w->firstrecv + m] = s->fp[w->send.v[m]];
  }
}

static void forward_erho(orc_sys *s) {
  for (int iswap = 0; iswap < s->nswap; iswap++) {
    swap_t *w = &s->swaps[iswap];
    for (int m = 0; m < w->esend.n; m++)
      for (int k = 0; k < NPE; k++)
        s->erho[NPE * (w->efirstrecv + m) + k] = s->erho[NPE * w->esend.v[m] + k];
  }
}

/* PairLJCut::compute, pair_lj_cut.cpp:227-288 */
static void lj_compute(orc_sys *s) {
  for (int i = 0; i < s->nlocal; i++) {
    double xt = s->x[3 * i], yt = s->x[3 * i + 1], zt = s->x[3 * i + 2];
    int it = s->type[i];
    double *fi = s->f + 3 * i;
    const int *jl = s->neigh.v + s->firstneigh[i];
    for (int jj = 0; jj < s->numneigh[i]; jj++) {
      int j = jl[jj];
      double dx = xt - s->x[3 * j], dy = yt - s->x[3 * j + 1], dz = zt - s->x[3 * j + 2];
      double rsq = dx * dx + dy * dy + dz * dz;
      int jt = s->type[j];
      if (rsq < s->cutsq[it][jt]) {
        double r2inv = 1.0 / rsq;
        double r6inv = r2inv * r2inv * r2inv;
        double forcelj = r6inv * (s->lj1[it][jt] * r6inv - s->lj2[it][jt]);
        double fpair = 1.0 * forcelj * r2inv; /* factor_lj = special_lj[0] = 1 */
        fi[0] += dx * fpair;
        fi[1] += dy * fpair;
        fi[2] += dz * fpair;
      }
    }
  }
}

/* PairEAM::compute, pair_eam.cpp:584-746 (single potential file) */
static void eam_compute(orc_sys *s) {
  int nall = s->nlocal + s->nghost;
  for (int i = 0; i < nall; i++) s->rho[i] = 0.0;
  for (int i = 0; i < s->nlocal; i++) {
    double xt = s->x[3 * i], yt = s->x[3 * i + 1], zt = s->x[3 * i + 2];
    const int *jl = s->neigh.v + s->firstneigh[i];
    for (int jj = 0; jj < s->numneigh[i]; jj++) {
      int j = jl[jj];
      double dx = xt - s->x[3 * j], dy = yt - s->x[3 * j + 1], dz = zt - s->x[3 * j + 2];
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < s->cutforcesq) {
        double p = sqrt(rsq) * s->rdr + 1.0;
        int m = (int) p;
        m = m < s->nr - 1 ? m : s->nr - 1;
        p -= m;
        p = p < 1.0 ? p : 1.0;
        const double *c = s->rhor_spline + 7 * m;
        s->rho[i] += ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
      }
    }
  }
  for (int i = 0; i < s->nlocal; i++) {
    double p = s->rho[i] * s->rdrho + 1.0;
    int m = (int) p;
    m = m < s->nrho - 1 ? m : s->nrho - 1;
    m = 1 > m ? 1 : m;
    p -= m;
    p = p < 1.0 ? p : 1.0;
    const double *c = s->frho_spline + 7 * m;
    s->fp[i] = (c[0] * p + c[1]) * p + c[2];
  }
  forward_fp(s);
  for (int i = 0; i < s->nlocal; i++) {
    double xt = s->x[3 * i], yt = s->x[3 * i + 1], zt = s->x[3 * i + 2];
    double *fi = s->f + 3 * i;
    const int *jl = s->neigh.v + s->firstneigh[i];
    for (int jj = 0; jj < s->numneigh[i]; jj++) {
      int j = jl[jj];
      double dx = xt - s->x[3 * j], dy = yt - s->x[3 * j + 1], dz = zt - s->x[3 * j + 2];
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < s->cutforcesq) {
        double r = sqrt(rsq);
        double p = r * s->rdr + 1.0;
        int m = (int) p;
        m = m < s->nr - 1 ? m : s->nr - 1;
        p -= m;
        p = p < 1.0 ? p : 1.0;
        const double *c = s->rhor_spline + 7 * m;
        double rhoip = (c[0] * p + c[1]) * p + c[2];
        double rhojp = (c[0] * p + c[1]) * p + c[2];
        const double *z = s->z2r_spline + 7 * m;
        double z2p = (z[0] * p + z[1]) * p + z[2];
        double z2 = ((z[3] * p + z[4]) * p + z[5]) * p + z[6];
        double recip = 1.0 / r;
        double phi = z2 * recip;
        double phip = z2p * recip - phi * recip;
        double psip = s->fp[i] * rhojp + s->fp[j] * rhoip + phip;
        double fpair = -psip * recip;
        fi[0] += dx * fpair;
        fi[1] += dy * fpair;
        fi[2] += dz * fpair;
      }
    }
  }
}

/* PairLJCut::ecompute, pair_lj_cut.cpp:295-442 (type-1 parameters only) */
static void lj_ecompute(orc_sys *s) {
  double ecutsq = s->cutsq[1][1], elj1 = s->lj1[1][1], elj2 = s->lj2[1][1];
  for (int i = 0; i < s->enlocal; i++) {
    int t = s->etype[i];
    int np = s->elist[i];
    const double *nxi = s->nodex + 24 * i;
    for (int jj = 0; jj < s->numint[t]; jj++, np++) {
      const double *N = s->spa_int[t] + NPE * jj;
      double ix = 0, iy = 0, iz = 0, fx = 0, fy = 0, fz = 0;
      for (int kk = 0; kk < NPE; kk++) {
        ix += N[kk] * nxi[3 * kk];
        iy += N[kk] * nxi[3 * kk + 1];
        iz += N[kk] * nxi[3 * kk + 2];
      }
      int base = s->ip_first.v[np];
      for (int ll = 0; ll < s->ip_num.v[np]; ll++) {
        int j = s->ip_j.v[base + ll], nj = s->ip_nj.v[base + ll];
        const double *M = s->spa_inter[s->etype[j]] + NPE * nj;
        const double *nxj = s->nodex + 24 * j;
        double jx = 0, jy = 0, jz = 0;
        for (int kk = 0; kk < NPE; kk++) {
          jx += M[kk] * nxj[3 * kk];
          jy += M[kk] * nxj[3 * kk + 1];
          jz += M[kk] * nxj[3 * kk + 2];
        }
        double dx = ix - jx, dy = iy - jy, dz = iz - jz;
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < ecutsq) {
          double r2inv = 1.0 / rsq;
          double r6inv = r2inv * r2inv * r2inv;
          double forcelj = r6inv * (elj1 * r6inv - elj2);
          double fpair = forcelj * r2inv;
          fx += dx * fpair;
          fy += dy * fpair;
          fz += dz * fpair;
        }
      }
      double w = s->weight[t][jj];
      double *nf = s->nodef + 24 * i;
      for (int kk = 0; kk < NPE; kk++) {
        nf[3 * kk] += w * N[kk] * fx;
        nf[3 * kk + 1] += w * N[kk] * fy;
        nf[3 * kk + 2] += w * N[kk] * fz;
      }
    }
  }
}

/* PairEAM::ecompute, pair_eam.cpp:761-1141 without the step>334 debug block */
static void eam_ecompute(orc_sys *s) {
  int nall = s->enlocal + s->enghost;
  for (int i = 0; i < nall * NPE; i++) s->erho[i] = 0.0;
  for (int i = 0; i < s->enlocal; i++) {
    int t = s->etype[i];
    int np = s->elist[i];
    const double *nxi = s->nodex + 24 * i;
    for (int jj = 0; jj < NPE; jj++) {
      int nt = np + s->node_list[t][jj];
      double ix = nxi[3 * jj], iy = nxi[3 * jj + 1], iz = nxi[3 * jj + 2];
      int base = s->ip_first.v[nt];
      for (int ll = 0; ll < s->ip_num.v[nt]; ll++) {
        int j = s->ip_j.v[base + ll], nj = s->ip_nj.v[base + ll];
        const double *M = s->spa_inter[s->etype[j]] + NPE * nj;
        const double *nxj = s->nodex + 24 * j;
        double jx = 0, jy = 0, jz = 0;
        for (int kk = 0; kk < NPE; kk++) {
          jx += M[kk] * nxj[3 * kk];
          jy += M[kk] * nxj[3 * kk + 1];
          jz += M[kk] * nxj[3 * kk + 2];
        }
        double dx = ix - jx, dy = iy - jy, dz = iz - jz;
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < s->cutforcesq) {
          double p = sqrt(rsq) * s->rdr + 1.0;
          int m = (int) p;
          m = m < s->nr - 1 ? m : s->nr - 1;
          p -= m;
          p = p < 1.0 ? p : 1.0;
          const double *c = s->rhor_spline + 7 * m;
          s->erho[NPE * i + jj] += ((c[3] * p + c[4]) * p + c[5]) * p + c[6];
        }
      }
    }
  }
  forward_erho(s);
  for (int i = 0; i < s->enlocal; i++) {
    int t = s->etype[i];
    int np = s->elist[i];
    const double *nxi = s->nodex + 24 * i;
    const double *eri = s->erho + NPE * i;
    for (int jj = 0; jj < s->numint[t]; jj++, np++) {
      const double *N = s->spa_int[t] + NPE * jj;
      double ix = 0, iy = 0, iz = 0, fx = 0, fy = 0, fz = 0, rhoi = 0;
      for (int kk = 0; kk < NPE; kk++) {
        ix += N[kk] * nxi[3 * kk];
        iy += N[kk] * nxi[3 * kk + 1];
        iz += N[kk] * nxi[3 * kk + 2];
        rhoi += N[kk] * eri[kk];
      }
      double p = rhoi * s->rdrho + 1.0;
      int m = (int) p;
      m = m < s->nrho - 1 ? m : s->nrho - 1;
      m = 1 > m ? 1 : m;
      p -= m;
      p = p < 1.0 ? p : 1.0;
      const double *c = s->frho_spline + 7 * m;
      double fpi = (c[0] * p + c[1]) * p + c[2];
      int base = s->ip_first.v[np];
      for (int ll = 0; ll < s->ip_num.v[np]; ll++) {
        int j = s->ip_j.v[base + ll], nj = s->ip_nj.v[base + ll];
        const double *M = s->spa_inter[s->etype[j]] + NPE * nj;
        const double *nxj = s->nodex + 24 * j;
        const double *erj = s->erho + NPE * j;
        double jx = 0, jy = 0, jz = 0, rhoj = 0;
        for (int kk = 0; kk < NPE; kk++) {
          jx += M[kk] * nxj[3 * kk];
          jy += M[kk] * nxj[3 * kk + 1];
          jz += M[kk] * nxj[3 * kk + 2];
          rhoj += M[kk] * erj[kk];
        }
        double dx = ix - jx, dy = iy - jy, dz = iz - jz;
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < s->cutforcesq) {
          double q = rhoj * s->rdrho + 1.0;
          int mq = (int) q;
          mq = mq < s->nrho - 1 ? mq : s->nrho - 1;
          mq = 1 > mq ? 1 : mq;
          q -= mq;
          q = q < 1.0 ? q : 1.0;
          const double *cf = s->frho_spline + 7 * mq;
          double fpj = (cf[0] * q + cf[1]) * q + cf[2];
          double r = sqrt(rsq);
          double pr = r * s->rdr + 1.0;
          int mr = (int) pr;
          mr = mr < s->nr - 1 ? mr : s->nr - 1;
          pr -= mr;
          pr = pr < 1.0 ? pr : 1.0;
          const double *cr = s->rhor_spline + 7 * mr;
          double rhoip = (cr[0] * pr + cr[1]) * pr + cr[2];
          const double *z = s->z2r_spline + 7 * mr;
          double z2p = (z[0] * pr + z[1]) * pr + z[2];
          double z2 = ((z[3] * pr + z[4]) * pr + z[5]) * pr + z[6];
          double recip = 1.0 / r;
          double phi = z2 * recip;
          double phip = z2p * recip - phi * recip;
          double psip = (fpi + fpj) * rhoip + phip;
          double fpair = -psip * recip;
          fx += dx * fpair;
          fy += dy * fpair;
          fz += dz * fpair;
        }
      }
      double w = s->weight[t][jj];
      double *nf = s->nodef + 24 * i;
      for (int kk = 0; kk < NPE; kk++) {
        nf[3 * kk] += w * N[kk] * fx;
        nf[3 * kk + 1] += w * N[kk] * fy;
        nf[3 * kk + 2] += w * N[kk] * fz;
      }
    }
  }
}

int orc_atom_forces(orc_sys *s) {
  if (!s->have_list) return fail(s, "atom neighbor list not built");
  for (int i = 0; i < 3 * s->nlocal; i++) s->f[i] = 0.0;
  if (s->pair_style == 1) lj_compute(s);
  else if (s->pair_style == 2) eam_compute(s);
  else return fail(s, "no pair style");
  return 0;
}

int orc_elem_forces(orc_sys *s) {
  if (!s->have_elists) return fail(s, "element lists not built");
  for (int i = 0; i < 24 * s->enlocal; i++) s->nodef[i] = 0.0;
  if (s->pair_style == 1) lj_ecompute(s);
  else if (s->pair_style == 2) eam_ecompute(s);
  else return fail(s, "no pair style");
  return 0;
}

/* ---- energy and virial (standard lj/cut and eam definitions; the reference's
   compute pe/temp/pressure are stubs, compute_pe.cpp:16-49) ---- */

static double spl_value(const double *c, double p) { return ((c[3] * p + c[4]) * p + c[5]) * p + c[6]; }
static double spl_deriv(const double *c, double p) { return (c[0] * p + c[1]) * p + c[2]; }

static const double *r_coef(orc_sys *s, const double *tab, double r, double *p) {
  double q = r * s->rdr + 1.0;
  int m = (int) q;
  m = m < s->nr - 1 ? m : s->nr - 1;
  q -= m;
  *p = q < 1.0 ? q : 1.0;
  return tab + 7 * m;
}

static const double *rho_coef(orc_sys *s, double rho, double *p) {
  double q = rho * s->rdrho + 1.0;
  int m = (int) q;
  m = m < s->nrho - 1 ? m : s->nrho - 1;
  m = 1 > m ? 1 : m;
  q -= m;
  *p = q < 1.0 ? q : 1.0;
  return s->frho_spline + 7 * m;
}

static void add_vir(double *v, double w, double dx, double dy, double dz, double fpair) {
  v[0] += w * dx * dx * fpair;
  v[1] += w * dy * dy * fpair;
  v[2] += w * dz * dz * fpair;
  v[3] += w * dx * dy * fpair;
  v[4] += w * dx * dz * fpair;
  v[5] += w * dy * dz * fpair;
}

/* position of integration site nj of element j */
static void site_pos(orc_sys *s, int j, int nj, double *out) {
  const double *M = s->spa_inter[s->etype[j]] + NPE * nj;
  const double *nxj = s->nodex + 24 * j;
  out[0] = out[1] = out[2] = 0.0;
  for (int kk = 0; kk < NPE; kk++)
    for (int d = 0; d < 3; d++) out[d] += M[kk] * nxj[3 * kk + d];
}

/* out: pe atoms, pe elements, ke atoms, ke nodes, virial[6], kinetic tensor[6],
   volume.  Pair energies are halved (full lists); integration points carry
   their weight.  EAM densities are recomputed at the current positions. */
int orc_thermo(orc_sys *s, double *out) {
  if (!s->have_list && s->nlocal) return fail(s, "atom neighbor list not built");
  if (!s->have_elists && s->enlocal) return fail(s, "element lists not built");
  for (int k = 0; k < 17; k++) out[k] = 0.0;
  double *vir = out + 4, p;
  if (s->pair_style == 2 && s->nlocal) {
    int nall = s->nlocal + s->nghost;
    for (int i = 0; i < nall; i++) s->rho[i] = 0.0;
    for (int i = 0; i < s->nlocal; i++) {
      const int *jl = s->neigh.v + s->firstneigh[i];
      for (int jj = 0; jj < s->numneigh[i]; jj++) {
        int j = jl[jj];
        double dx = s->x[3 * i] - s->x[3 * j], dy = s->x[3 * i + 1] - s->x[3 * j + 1],
               dz = s->x[3 * i + 2] - s->x[3 * j + 2];
        double rsq = dx * dx + dy * dy + dz * dz;
        if (rsq < s->cutforcesq) {
          const double *c = r_coef(s, s->rhor_spline, sqrt(rsq), &p);
          s->rho[i] += spl_value(c, p);
        }
      }
      const double *c = rho_coef(s, s->rho[i], &p);
      s->fp[i] = spl_deriv(c, p);
    }
    forward_fp(s);
  }
  for (int i = 0; i < s->nlocal; i++) {
    int it = s->type[i];
    double e = 0.0;
    if (s->pair_style == 2) {
      const double *c = rho_coef(s, s->rho[i], &p);
      e = spl_value(c, p);
    }
    const int *jl = s->neigh.v + s->firstneigh[i];
    for (int jj = 0; jj < s->numneigh[i]; jj++) {
      int j = jl[jj], jt = s->type[j];
      double dx = s->x[3 * i] - s->x[3 * j], dy = s->x[3 * i + 1] - s->x[3 * j + 1],
             dz = s->x[3 * i + 2] - s->x[3 * j + 2];
      double rsq = dx * dx + dy * dy + dz * dz;
      if (s->pair_style == 1 && rsq < s->cutsq[it][jt]) {
        double r2inv = 1.0 / rsq, r6inv = r2inv * r2inv * r2inv;
        e += 0.5 * r6inv * (s->lj3[it][jt] * r6inv - s->lj4[it][jt]);
        add_vir(vir, 0.5, dx, dy, dz, r6inv * (s->lj1[it][jt] * r6inv - s->lj2[it][jt]) * r2inv);
      } else if (s->pair_style == 2 && rsq < s->cutforcesq) {
        double r = sqrt(rsq);
        const double *cr = r_coef(s, s->rhor_spline, r, &p);
        const double *z = r_coef(s, s->z2r_spline, r, &p);
        double phi = spl_value(z, p) / r;
        double phip = spl_deriv(z, p) / r - phi / r;
        e += 0.5 * phi;
        add_vir(vir, 0.5, dx, dy, dz, -((s->fp[i] + s->fp[j]) * spl_deriv(cr, p) + phip) / r);
      }
    }
    out[0] += e;
  }
  if (s->enlocal && s->pair_style == 2) {
    int nall = s->enlocal + s->enghost;
    for (int i = 0; i < nall * NPE; i++) s->erho[i] = 0.0;
    for (int i = 0; i < s->enlocal; i++) {
      int t = s->etype[i];
      for (int jj = 0; jj < NPE; jj++) {
        int nt = s->elist[i] + s->node_list[t][jj];
        const double *xi = s->nodex + 24 * i + 3 * jj;
        int base = s->ip_first.v[nt];
        for (int ll = 0; ll < s->ip_num.v[nt]; ll++) {
          double xj[3];
          site_pos(s, s->ip_j.v[base + ll], s->ip_nj.v[base + ll], xj);
          double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
          double rsq = dx * dx + dy * dy + dz * dz;
          if (rsq < s->cutforcesq) {
            const double *c = r_coef(s, s->rhor_spline, sqrt(rsq), &p);
            s->erho[NPE * i + jj] += spl_value(c, p);
          }
        }
      }
    }
    forward_erho(s);
  }
  for (int i = 0; i < s->enlocal; i++) {
    int t = s->etype[i];
    int np = s->elist[i];
    for (int jj = 0; jj < s->numint[t]; jj++, np++) {
      double w = s->weight[t][jj];
      if (w == 0.0) continue;
      const double *N = s->spa_int[t] + NPE * jj;
      double xi[3] = {0, 0, 0}, rhoi = 0.0;
      for (int kk = 0; kk < NPE; kk++) {
        for (int d = 0; d < 3; d++) xi[d] += N[kk] * s->nodex[24 * i + 3 * kk + d];
        if (s->pair_style == 2) rhoi += N[kk] * s->erho[NPE * i + kk];
      }
      double e = 0.0, fpi = 0.0;
      if (s->pair_style == 2) {
        const double *c = rho_coef(s, rhoi, &p);
        fpi = spl_deriv(c, p);
        e = spl_value(c, p);
      }
      int base = s->ip_first.v[np];
      for (int ll = 0; ll < s->ip_num.v[np]; ll++) {
        int j = s->ip_j.v[base + ll], nj = s->ip_nj.v[base + ll];
        double xj[3];
        site_pos(s, j, nj, xj);
        double dx = xi[0] - xj[0], dy = xi[1] - xj[1], dz = xi[2] - xj[2];
        double rsq = dx * dx + dy * dy + dz * dz;
        if (s->pair_style == 1 && rsq < s->cutsq[1][1]) {
          double r2inv = 1.0 / rsq, r6inv = r2inv * r2inv * r2inv;
          e += 0.5 * r6inv * (s->lj3[1][1] * r6inv - s->lj4[1][1]);
          add_vir(vir, 0.5 * w, dx, dy, dz, r6inv * (s->lj1[1][1] * r6inv - s->lj2[1][1]) * r2inv);
        } else if (s->pair_style == 2 && rsq < s->cutforcesq) {
          const double *M = s->spa_inter[s->etype[j]] + NPE * nj;
          double rhoj = 0.0;
          for (int kk = 0; kk < NPE; kk++) rhoj += M[kk] * s->erho[NPE * j + kk];
          const double *cf = rho_coef(s, rhoj, &p);
          double fpj = spl_deriv(cf, p);
          double r = sqrt(rsq);
          const double *cr = r_coef(s, s->rhor_spline, r, &p);
          const double *z = r_coef(s, s->z2r_spline, r, &p);
          double phi = spl_value(z, p) / r;
          double phip = spl_deriv(z, p) / r - phi / r;
          e += 0.5 * phi;
          add_vir(vir, 0.5 * w, dx, dy, dz, -((fpi + fpj) * spl_deriv(cr, p) + phip) / r);
        }
      }
      out[1] += w * e;
    }
  }
  double mvv2e = s->ftm2v == 1.0 ? 1.0 : 1.0364269e-4; /* update.cpp:90,110 */
  for (int i = 0; i < s->nlocal; i++) {
    double m = s->amass[s->type[i]];
    const double *v = s->v + 3 * i;
    out[2] += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * mvv2e;
    double t6[6] = {v[0] * v[0], v[1] * v[1], v[2] * v[2], v[0] * v[1], v[0] * v[2], v[1] * v[2]};
    for (int k = 0; k < 6; k++) out[10 + k] += m * t6[k] * mvv2e;
  }
  for (int i = 0; i < s->enlocal; i++) {
    double m = s->emass[s->etype[i]] / NPE;
    for (int q = 0; q < NPE; q++) {
      const double *v = s->nodev + 24 * i + 3 * q;
      out[3] += 0.5 * m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]) * mvv2e;
      double t6[6] = {v[0] * v[0], v[1] * v[1], v[2] * v[2], v[0] * v[1], v[0] * v[2], v[1] * v[2]};
      for (int k = 0; k < 6; k++) out[10 + k] += m * t6[k] * mvv2e;
    }
  }
  out[16] = (s->boxhi[0] - s->boxlo[0]) * (s->boxhi[1] - s->boxlo[1]) * (s->boxhi[2] - s->boxlo[2]);
  return 0;
}

/* ---- centro-symmetry, Output::centro_atom (output.cpp:352-447) ----
   The k smallest of n values land in the first k slots by the partial
   quickselect of Numerical Recipes (select / select2, output.cpp:458-554):
   median-of-three pivot at l+1, Hoare partition, narrow to the side holding
   k.  The same steps are kept so that the same neighbors are chosen among
   equal distances and the pair sums add in the same order. */

static void nr_select(int k, int n, double *arr, int *iarr) {
  /* 1-based positions, as the published routine states them */
#define A(p) arr[(p) - 1]
#define IA(p) iarr[(p) - 1]
#define SWAP_AT(p, q)                                          \
  {                                                            \
    double t_ = A(p); A(p) = A(q); A(q) = t_;                  \
    if (iarr) { int u_ = IA(p); IA(p) = IA(q); IA(q) = u_; }   \
  }
  int l = 1, ir = n;
  for (;;) {
    if (ir <= l + 1) {
      if (ir == l + 1 && A(ir) < A(l)) SWAP_AT(l, ir);
      return;
    }
    int mid = (l + ir) >> 1;
    SWAP_AT(mid, l + 1);
    if (A(l) > A(ir)) SWAP_AT(l, ir);
    if (A(l + 1) > A(ir)) SWAP_AT(l + 1, ir);
    if (A(l) > A(l + 1)) SWAP_AT(l, l + 1);
    int i = l + 1, j = ir;
    double piv = A(l + 1);
    int ipiv = iarr ? IA(l + 1) : 0;
    for (;;) {
      do i++; while (A(i) < piv);
      do j--; while (A(j) > piv);
      if (j < i) break;
      SWAP_AT(i, j);
    }
    A(l + 1) = A(j);
    A(j) = piv;
    if (iarr) {
      IA(l + 1) = IA(j);
      IA(j) = ipiv;
    }
    if (j >= k) ir = j - 1;
    if (j <= k) l = i;
  }
#undef A
#undef IA
#undef SWAP_AT
}

/* centro[i] for the local atoms over the full atom list: the 12 nearest
   neighbors within the list cutoff, the 66 pair vectors R_j + R_k - 2 R_i,
   the sum of the 6 smallest |.|^2; 0 with fewer than 12 neighbors */
int orc_centro(orc_sys *s, double *out) {
  if (!s->have_list) return fail(s, "atom neighbor list not built");
  const int nnn = 12, nhalf = nnn / 2, npairs = nnn * (nnn - 1) / 2;
  double pairs[66];
  int maxn = 1;
  for (int i = 0; i < s->nlocal; i++) maxn = s->numneigh[i] > maxn ? s->numneigh[i] : maxn;
  double *dsq = (double *) malloc(sizeof(double) * maxn);
  int *near = (int *) malloc(sizeof(int) * maxn);
  for (int i = 0; i < s->nlocal; i++) {
    const double *xi = s->x + 3 * i;
    const int *jl = s->neigh.v + s->firstneigh[i];
    int n = 0;
    for (int jj = 0; jj < s->numneigh[i]; jj++) {
      int j = jl[jj];
      double dx = xi[0] - s->x[3 * j], dy = xi[1] - s->x[3 * j + 1], dz = xi[2] - s->x[3 * j + 2];
      double rsq = dx * dx + dy * dy + dz * dz;
      if (rsq < s->cutneighmaxsq) {
        dsq[n] = rsq;
        near[n++] = j;
      }
    }
    if (n < nnn) {
      out[i] = 0.0;
      continue;
    }
    nr_select(nnn, n, dsq, near);
    int m = 0;
    for (int a = 0; a < nnn; a++) {
      const double *xa = s->x + 3 * near[a];
      for (int b = a + 1; b < nnn; b++) {
        const double *xb = s->x + 3 * near[b];
        double dx = xa[0] + xb[0] - 2.0 * xi[0];
        double dy = xa[1] + xb[1] - 2.0 * xi[1];
        double dz = xa[2] + xb[2] - 2.0 * xi[2];
        pairs[m++] = dx * dx + dy * dy + dz * dz;
      }
    }
    nr_select(nhalf, npairs, pairs, NULL);
    double v = 0.0;
    for (int a = 0; a < nhalf; a++) v += pairs[a];
    out[i] = v;
  }
  free(dsq);
  free(near);
  return 0;
}

/* FixNVE, fix_nve.cpp:54-157 */
static void nve_initial(orc_sys *s) {
  double dtv = s->dt, dtf = 0.5 * s->dt * s->ftm2v;
  for (int i = 0; i < s->nlocal; i++) {
    double dtfm = dtf / s->amass[s->type[i]];
    for (int d = 0; d < 3; d++) s->v[3 * i + d] += dtfm * s->f[3 * i + d];
    for (int d = 0; d < 3; d++) s->x[3 * i + d] += dtv * s->v[3 * i + d];
  }
  double inv_npe = 1 / (double) NPE;
  for (int i = 0; i < s->enlocal; i++) {
    double dtfm = dtf / (inv_npe * s->emass[s->etype[i]]);
    for (int j = 0; j < NPE; j++) {
      double *nv = s->nodev + 24 * i + 3 * j, *nx = s->nodex + 24 * i + 3 * j;
      const double *nf = s->nodef + 24 * i + 3 * j;
      for (int d = 0; d < 3; d++) nv[d] += dtfm * nf[d];
      for (int d = 0; d < 3; d++) nx[d] += dtv * nv[d];
    }
  }
  for (int i = 0; i < s->enlocal; i++) {
    double c[3] = {0.0, 0.0, 0.0};
    for (int j = 0; j < NPE; j++)
      for (int d = 0; d < 3; d++) c[d] += s->nodex[24 * i + 3 * j + d];
    for (int d = 0; d < 3; d++) s->ex[3 * i + d] = c[d] / NPE;
  }
}

/* FixNVE::final_integrate / efinal_integrate, fix_nve.cpp:181-242 */
static void nve_final(orc_sys *s) {
  double dtf = 0.5 * s->dt * s->ftm2v;
  for (int i = 0; i < s->nlocal; i++) {
    double dtfm = dtf / s->amass[s->type[i]];
    for (int d = 0; d < 3; d++) s->v[3 * i + d] += dtfm * s->f[3 * i + d];
  }
  double inv_npe = 1 / (double) NPE;
  for (int i = 0; i < s->enlocal; i++) {
    double dtfm = dtf / (inv_npe * s->emass[s->etype[i]]);
    for (int k = 0; k < 24; k++) s->nodev[24 * i + k] += dtfm * s->nodef[24 * i + k];
  }
}

/* Neighbor::decide + check_distance, neighbor.cpp:1150-1217; the atom branch
   uses a hold copy taken at each atom list build */
static int decide(orc_sys *s) {
  s->ago++;
  if (s->ago >= s->delay && s->ago % s->every == 0) {
    if (s->dist_check == 0) return 1;
    int flag = 0;
    for (int i = 0; i < s->nlocal; i++) {
      double dx = s->x[3 * i] - s->xhold[3 * i];
      double dy = s->x[3 * i + 1] - s->xhold[3 * i + 1];
      double dz = s->x[3 * i + 2] - s->xhold[3 * i + 2];
      if (dx * dx + dy * dy + dz * dz > s->triggersq) flag = 1;
    }
    for (int i = 0; i < s->enlocal; i++)
      for (int j = 0; j < NPE; j++) {
        const double *a = s->nodex + 24 * i + 3 * j, *b = s->nodexhold + 24 * i + 3 * j;
        double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        if (dx * dx + dy * dy + dz * dz > s->triggersq) flag = 1;
      }
    return flag;
  }
  return 0;
}

/* Domain::pbc / elepbc, domain.cpp:535-745.  Periodic dims only; the element
   +x wrap here subtracts the period from the nodes (the reference adds it,
   domain.cpp:682), so parity cases avoid elements crossing the +x face. */
static void pbc(orc_sys *s) {
  for (int i = 0; i < s->nlocal; i++)
    for (int d = 0; d < 3; d++) {
      if (!s->periodic[d]) continue;
      double *x = s->x + 3 * i + d;
      if (*x < s->boxlo[d]) *x += s->prd[d];
      if (*x >= s->boxhi[d]) {
        *x -= s->prd[d];
        *x = *x > s->boxlo[d] ? *x : s->boxlo[d];
      }
    }
  for (int i = 0; i < s->enlocal; i++)
    for (int d = 0; d < 3; d++) {
      if (!s->periodic[d]) continue;
      double *x = s->ex + 3 * i + d;
      if (*x < s->boxlo[d]) {
        *x += s->prd[d];
        for (int m = 0; m < NPE; m++) s->nodex[24 * i + 3 * m + d] += s->prd[d];
      }
      if (*x >= s->boxhi[d]) {
        *x -= s->prd[d];
        for (int m = 0; m < NPE; m++) s->nodex[24 * i + 3 * m + d] -= s->prd[d];
        *x = *x > s->boxlo[d] ? *x : s->boxlo[d];
      }
    }
}

/* Verlet::run order (verlet.cpp:163-218), with Pair::compute for atoms */
/* group bits of the local atoms and elements (NULL: every item in "all" only) */
int orc_set_masks(orc_sys *s, const int *amask, const int *emask) {
  free(s->amask);
  free(s->emask);
  s->amask = (int *) malloc(sizeof(int) * (s->nlocal + 1));
  s->emask = (int *) malloc(sizeof(int) * (s->enlocal + 1));
  for (int i = 0; i < s->nlocal; i++) s->amask[i] = amask ? amask[i] : 1;
  for (int i = 0; i < s->enlocal; i++) s->emask[i] = emask ? emask[i] : 1;
  return 0;
}

/* FixSetForce (fix_setforce.cpp:18-60): set[d] != 0 assigns val[d] */
int orc_add_setforce(orc_sys *s, int bit, const int *set, const double *val) {
  if (s->nfix == 16) return fail(s, "too many fixes");
  s->fixes[s->nfix].viscous = 0;
  s->fixes[s->nfix].bit = bit;
  for (int d = 0; d < 3; d++) {
    s->fixes[s->nfix].set[d] = set[d];
    s->fixes[s->nfix].val[d] = val[d];
  }
  s->nfix++;
  return 0;
}

/* FixViscous (fix_viscous.cpp:14-30) */
int orc_add_viscous(orc_sys *s, int bit, double gamma) {
  if (s->nfix == 16) return fail(s, "too many fixes");
  s->fixes[s->nfix].viscous = 1;
  s->fixes[s->nfix].bit = bit;
  s->fixes[s->nfix].gamma = gamma;
  s->nfix++;
  return 0;
}

/* Modify::post_force (modify.cpp:663-669): each fix on the atoms
   (FixSetForce::post_force 107-134, FixViscous::post_force 73-95), then on
   the element nodes (epost_force 136-161, 97-123) */
int orc_post_force(orc_sys *s) {
  for (int k = 0; k < s->nfix; k++) {
    const int bit = s->fixes[k].bit;
    for (int pass = 0; pass < 2; pass++) {
      const int n = pass ? s->enlocal : s->nlocal, per = pass ? NPE : 1;
      const int *mask = pass ? s->emask : s->amask;
      double *f = pass ? s->nodef : s->f;
      const double *v = pass ? s->nodev : s->v;
      for (int i = 0; i < n; i++) {
        int m = mask ? mask[i] : 1;
        if (!(m & bit)) continue;
        for (int q = 0; q < per; q++) {
          double *fi = f + 3 * (per * i + q);
          const double *vi = v + 3 * (per * i + q);
          if (s->fixes[k].viscous) {
            double drag = s->fixes[k].gamma;
            fi[0] -= drag * vi[0];
            fi[1] -= drag * vi[1];
            fi[2] -= drag * vi[2];
          } else {
            for (int d = 0; d < 3; d++)
              if (s->fixes[k].set[d]) fi[d] = s->fixes[k].val[d];
          }
        }
      }
    }
  }
  return 0;
}

/* L(t) = L0 (1 + erate t) about the box centre from now on; positions of
   atoms, nodes and element centres remapped affinely at the end of each step
   (no reference counterpart) */
int orc_get_box(orc_sys *s, double *lo, double *hi) {
  for (int d = 0; d < 3; d++) {
    lo[d] = s->boxlo[d];
    hi[d] = s->boxhi[d];
  }
  return 0;
}

int orc_set_deform(orc_sys *s, const double *erate) {
  s->deform = 0;
  for (int d = 0; d < 3; d++) {
    s->erate[d] = erate[d];
    s->dL0[d] = s->boxhi[d] - s->boxlo[d];
    s->dc0[d] = 0.5 * (s->boxlo[d] + s->boxhi[d]);
    s->deform |= erate[d] != 0.0;
  }
  s->deform_t0 = s->ntimestep;
  return 0;
}

static void deform_step(orc_sys *s) {
  if (!s->deform) return;
  double t = (double) (s->ntimestep - s->deform_t0) * s->dt;
  for (int d = 0; d < 3; d++) {
    if (s->erate[d] == 0.0) continue;
    double L = s->dL0[d] * (1.0 + s->erate[d] * t);
    double nlo = s->dc0[d] - 0.5 * L, olo = s->boxlo[d];
    double f = L / s->prd[d];
    for (int i = 0; i < s->nlocal; i++) s->x[3 * i + d] = nlo + (s->x[3 * i + d] - olo) * f;
    for (int i = 0; i < NPE * s->enlocal; i++) s->nodex[3 * i + d] = nlo + (s->nodex[3 * i + d] - olo) * f;
    for (int i = 0; i < s->enlocal; i++) s->ex[3 * i + d] = nlo + (s->ex[3 * i + d] - olo) * f;
    s->boxlo[d] = nlo;
    s->boxhi[d] = s->dc0[d] + 0.5 * L;
    s->prd[d] = L;
  }
}

int orc_run(orc_sys *s, int nsteps) {
  for (int step = 0; step < nsteps; step++) {
    s->ntimestep++;
    nve_initial(s);
    int nflag = decide(s);
    if (nflag == 0) {
      if (s->nlocal) forward_comm(s);
      if (s->enlocal) eforward_comm(s);
    } else {
      s->nrebuild++;
      pbc(s);
      if (s->enlocal && element_size(s)) return -1;
      setup_cut(s);
      comm_setup(s);
      if (setup_bins(s)) return -1;
      borders(s);
      if (s->nlocal && orc_atom_list(s)) return -1;
      if (s->enlocal && orc_elem_lists(s)) return -1;
    }
    if (s->enlocal)
      for (int i = 0; i < 24 * s->enlocal; i++) s->nodef[i] = 0.0;
    if (s->nlocal && orc_atom_forces(s)) return -1;
    if (s->enlocal && orc_elem_forces(s)) return -1;
    orc_post_force(s); /* verlet.cpp:206 */
    nve_final(s);
    deform_step(s);
  }
  return 0;
}

long long orc_size(orc_sys *s, int what) {
  switch (what) {
    case 0: return s->nlocal;
    case 1: return s->nghost;
    case 2: return s->neigh.n;
    case 3: return s->enlocal;
    case 4: return s->enghost;
    case 5: return s->eneigh.n;
    case 6: return s->ninum;
    case 7: return s->ip_j.n;
    case 8: return s->nrebuild;
    case 9: return s->nstencil;
    default: return -1;
  }
}

int orc_get_atom_list(orc_sys *s, int *numneigh, int *neigh) {
  if (numneigh) memcpy(numneigh, s->numneigh, (size_t) s->nlocal * sizeof(int));
  if (neigh) memcpy(neigh, s->neigh.v, (size_t) s->neigh.n * sizeof(int));
  return 0;
}

int orc_get_atoms(orc_sys *s, int all, double *x, double *v, double *f, int *tag) {
  int n = all ? s->nlocal + s->nghost : s->nlocal;
  if (x) memcpy(x, s->x, (size_t) n * 3 * sizeof(double));
  if (v) memcpy(v, s->v, (size_t) s->nlocal * 3 * sizeof(double));
  if (f) memcpy(f, s->f, (size_t) s->nlocal * 3 * sizeof(double));
  if (tag) memcpy(tag, s->tag, (size_t) n * sizeof(int));
  return 0;
}

int orc_get_elem_list(orc_sys *s, int *numneigh, int *neigh) {
  if (numneigh) memcpy(numneigh, s->enumneigh, (size_t) s->enlocal * sizeof(int));
  if (neigh) memcpy(neigh, s->eneigh.v, (size_t) s->eneigh.n * sizeof(int));
  return 0;
}

int orc_get_ip_list(orc_sys *s, int *numneigh, int *jelem, int *jsite) {
  if (numneigh) memcpy(numneigh, s->ip_num.v, (size_t) s->ninum * sizeof(int));
  if (jelem) memcpy(jelem, s->ip_j.v, (size_t) s->ip_j.n * sizeof(int));
  if (jsite) memcpy(jsite, s->ip_nj.v, (size_t) s->ip_nj.n * sizeof(int));
  return 0;
}

int orc_get_elements(orc_sys *s, int all, double *centre, double *nodex, double *nodev,
                     double *nodef, int *tag) {
  int n = all ? s->enlocal + s->enghost : s->enlocal;
  if (centre) memcpy(centre, s->ex, (size_t) n * 3 * sizeof(double));
  if (nodex) memcpy(nodex, s->nodex, (size_t) n * 24 * sizeof(double));
  if (nodev) memcpy(nodev, s->nodev, (size_t) s->enlocal * 24 * sizeof(double));
  if (nodef) memcpy(nodef, s->nodef, (size_t) s->enlocal * 24 * sizeof(double));
  if (tag) memcpy(tag, s->etag, (size_t) n * sizeof(int));
  return 0;
}

double orc_get_cut(orc_sys *s, int what) {
  switch (what) {
    case 0: return s->cutneighmax;
    case 1: return s->cut_all;
    case 2: return s->cut_ele;
    case 3: return s->cut_subele;
    case 4: return s->max_size;
    case 5: return (double) s->nsubele;
    default: return 0.0;
  }
}

int orc_get_eam_scratch(orc_sys *s, double *rho, double *fp, double *erho) {
  if (rho) memcpy(rho, s->rho, (size_t) s->nlocal * sizeof(double));
  if (fp) memcpy(fp, s->fp, (size_t) (s->nlocal + s->nghost) * sizeof(double));
  if (erho) memcpy(erho, s->erho, (size_t) (s->enlocal + s->enghost) * NPE * sizeof(double));
  return 0;
}
