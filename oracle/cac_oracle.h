/*
 * CPU restatement of the reference CAC per-step force path -- TEST
 * INFRASTRUCTURE ONLY.  Nothing in the product links or calls this; only the
 * tests, the fixture generator and bench.py's CPU-baseline leg do.  Each
 * routine follows the reference file:line named beside it.  It is pinned
 * against the unmodified reference (oracle/_ref, built from the reference tree
 * by oracle/Makefile) by tests/test_oracle_vs_ref.py and against the committed
 * fixtures in tests/golden/.
 */
#ifndef CAC_ORACLE_H
#define CAC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_sys orc_sys;

orc_sys *orc_create(void);
void orc_destroy(orc_sys *s);
const char *orc_error(orc_sys *s);

/* units: 0 = lj, 1 = metal (update.cpp:83-132) */
int orc_set_units(orc_sys *s, int metal);
int orc_set_timestep(orc_sys *s, double dt);
int orc_set_box(orc_sys *s, const double *lo, const double *hi, const int *periodic);
/* neighbor X bin; neigh_modify every/delay/check/binsize (neighbor.cpp:180-262) */
int orc_set_neighbor(orc_sys *s, double skin, int every, int delay, int check,
                     double binsize_user);
int orc_set_elementsplit(orc_sys *s, int nsplit);
int orc_set_atom_types(orc_sys *s, int ntypes, const double *mass /* [ntypes] */);
int orc_set_atoms(orc_sys *s, int n, const double *x, const double *v, const int *type);
int orc_set_element_types(orc_sys *s, int ntypes, const int *nae /* [t][3] */,
                          const int *numint /* [t] */, const int *intp /* [sum][3] */,
                          const double *weight /* [sum] */);
int orc_set_elements(orc_sys *s, int n, const int *etype, const double *centre,
                     const double *nodex, const double *nodev);
/* pair_style lj/cut: per type-pair eps/sigma/cut, row-major [ntypes][ntypes] */
int orc_set_lj(orc_sys *s, int ntypes, const double *eps, const double *sigma,
               const double *cut);
/* pair_style eam + pair_coeff * * file (pair_eam.cpp:197-580) */
int orc_set_eam_file(orc_sys *s, const char *path);

/* CAC::init + Verlet::setup up to and including comm->borders */
int orc_setup(orc_sys *s);
int orc_atom_list(orc_sys *s);   /* Neighbor::build */
int orc_elem_lists(orc_sys *s);  /* setup_cut + ebuild + nbuild */
int orc_atom_forces(orc_sys *s); /* Pair::compute */
int orc_elem_forces(orc_sys *s); /* Pair::ecompute */
/* group masks and the post-force fixes setforce / viscous */
int orc_set_masks(orc_sys *s, const int *amask, const int *emask);
int orc_add_setforce(orc_sys *s, int bit, const int *set, const double *val);
int orc_add_viscous(orc_sys *s, int bit, double gamma);
int orc_post_force(orc_sys *s);
/* box deformation at engineering strain rates erate[3] (per time unit) */
int orc_set_deform(orc_sys *s, const double *erate);
int orc_get_box(orc_sys *s, double *lo, double *hi);
/* centro-symmetry of the local atoms over the atom list (Output::centro_atom) */
int orc_centro(orc_sys *s, double *out);
/* energies, virial and kinetic tensors at the current state (17 values) */
int orc_thermo(orc_sys *s, double *out);
int orc_run(orc_sys *s, int nsteps); /* Verlet::run loop with atom forces */

/* sizes: 0 nlocal, 1 nghost, 2 atom list entries, 3 elem nlocal, 4 elem nghost,
   5 elem list entries, 6 ip rows, 7 ip list entries, 8 rebuilds, 9 nstencil */
long long orc_size(orc_sys *s, int what);
int orc_get_atom_list(orc_sys *s, int *numneigh, int *neigh);
int orc_get_atoms(orc_sys *s, int all, double *x, double *v, double *f, int *tag);
int orc_get_elem_list(orc_sys *s, int *numneigh, int *neigh);
int orc_get_ip_list(orc_sys *s, int *numneigh, int *jelem, int *jsite);
int orc_get_elements(orc_sys *s, int all, double *centre, double *nodex, double *nodev,
                     double *nodef, int *tag);
/* 0 cutneighmax 1 cut_all 2 cut_ele 3 cut_subele 4 max_size 5 nsubele */
double orc_get_cut(orc_sys *s, int what);
int orc_get_eam_scratch(orc_sys *s, double *rho, double *fp, double *erho);

#ifdef __cplusplus
}
#endif

#endif
