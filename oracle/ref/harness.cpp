// Test-only oracle harness: drives the UNMODIFIED reference CAC sources
// (compiled from the reference tree by oracle/Makefile) through the per-step
// force path that the reference's own driver never reaches.
//
// The reference's run command stops in Verlet::setup (verlet.cpp:97), never
// allocates the integration-point tables (element.h:27-45), never creates the
// node neighbor list (neighbor.h:50), never allocates the element bin heads
// (neighbor.cpp:635 writes ebinhead, which nothing allocates) and grows only x
// in AtomVecAtomic::grow (atom_vec_atomic.cpp:33-42).  This harness supplies
// those allocations and the call order of Verlet::run (verlet.cpp:149-219),
// and dumps neighbor lists, forces and state as raw binary arrays.
//
// Usage: cacref <input-script> <directives> <outdir>
//   The input script holds reference commands (units, boundary, read_data,
//   pair_style, pair_coeff, neighbor, neigh_modify, timestep, fix, elementsplit).
//   The directives file holds one harness action per line:
//     capacity N     atom array capacity (read before the input script runs)
//     setup          CAC::init + element tables + comm setup, bins, exchange, borders
//     atom_list      Neighbor::build, dump the full atom list
//     atom_forces    Pair::compute on atoms, dump f
//     elem_lists     Neighbor::setup_cut/ebuild/nbuild, dump both element lists
//     elem_forces    Pair::ecompute, dump nodef
//     step N         N steps in Verlet::run order (atoms get Pair::compute too)
//     state TAG      dump x, v, f, nodex, nodev, nodef with file prefix TAG
//     eam_tables     after setup: PairEAM's splines of type 1 (frho, rhor, z2r,
//                    [n + 1][7] each, pair_eam.cpp:527-580) and nr, dr, nrho,
//                    drho, cutforcesq, mass of type 1
//     lj_tables      after setup: PairLJCut's lj1, lj2 and cutsq,
//                    [ntypes + 1][ntypes + 1] each (pair_lj_cut.cpp:140-198)
//     velocities F   set atom velocities from raw float64 file F (3 per atom, in
//                    tag order); the data file format has no atom velocities
//                    (atom_vec_atomic.cpp:70-72 zero them, and ReadData has no
//                    Velocities section handler)
#include "mpi.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "atom.h"
#include "atom_vec.h"
#include "atom_vec_atomic.h"
#include "cac.h"
#include "comm.h"
#include "domain.h"
#include "element.h"
#include "error.h"
#include "fix.h"
#include "force.h"
#include "input.h"
#include "memory.h"
#include "modify.h"
#include "neigh_list.h"
#include "neighbor.h"
#include "output.h"
#include "node_neigh_list.h"
#include "pair.h"
#include "pair_eam.h"
#include "pair_lj_cut.h"
#include "update.h"

using namespace CAC_NS;

static std::string g_out;

static void write_raw(const char *name, const void *data, size_t bytes) {
  std::string path = g_out + "/" + name;
  FILE *f = fopen(path.c_str(), "wb");
  if (!f) {
    fprintf(stderr, "cacref: cannot write %s\n", path.c_str());
    exit(2);
  }
  if (bytes) fwrite(data, 1, bytes, f);
  fclose(f);
}

static void write_i32(const char *name, const std::vector<int> &v) {
  write_raw(name, v.empty() ? NULL : &v[0], v.size() * sizeof(int));
}

static void write_f64(const char *name, const std::vector<double> &v) {
  write_raw(name, v.empty() ? NULL : &v[0], v.size() * sizeof(double));
}

struct Harness {
  CAC *cac;
  int capacity;
  int tables_ready;
  int eam;

  Harness() : cac(NULL), capacity(0), tables_ready(0), eam(0) {}

  // AtomVecAtomic::grow only grows x; give every other per-atom array a fixed
  // capacity up front and point the AtomVec at them.
  void prealloc_atoms() {
    if (capacity <= 0) return;
    Atom *atom = cac->atom;
    AtomVecAtomic *avec = (AtomVecAtomic *) atom->avec;
    Memory *memory = cac->memory;
    memory->create(atom->tag, capacity, "harness:tag");
    memory->create(atom->type, capacity, "harness:type");
    memory->create(atom->mask, capacity, "harness:mask");
    memory->create(atom->image, capacity, "harness:image");
    memory->create(atom->v, capacity, 3, "harness:v");
    memory->create(atom->f, capacity, 3, "harness:f");
    for (int i = 0; i < capacity; i++) {
      atom->v[i][0] = atom->v[i][1] = atom->v[i][2] = 0.0;
      atom->f[i][0] = atom->f[i][1] = atom->f[i][2] = 0.0;
    }
    avec->tag = atom->tag;
    avec->type = atom->type;
    avec->mask = atom->mask;
    avec->image = atom->image;
    avec->v = atom->v;
    avec->f = atom->f;
    avec->grow(capacity);
  }

  void refresh_avec_x() {
    AtomVecAtomic *avec = (AtomVecAtomic *) cac->atom->avec;
    avec->x = cac->atom->x;
  }

  void check_capacity() {
    Atom *atom = cac->atom;
    if (atom->nlocal + atom->nghost > capacity && atom->nlocal + atom->nghost > 0) {
      fprintf(stderr, "cacref: capacity %d too small for %d atoms+ghosts\n", capacity,
              atom->nlocal + atom->nghost);
      exit(2);
    }
  }

  // ebinhead is written by Neighbor::bin_elements but never allocated.
  void ensure_ebinhead() {
    Neighbor *nb = cac->neighbor;
    cac->memory->destroy(nb->ebinhead);
    cac->memory->create(nb->ebinhead, nb->maxhead > 0 ? nb->maxhead : 1, "harness:ebinhead");
  }

  void build_element_tables() {
    Element *e = cac->element;
    Memory *memory = cac->memory;
    int nt = e->ntypes;
    int npe = e->npe;
    e->nsubele = e->nsplit_ele * e->nsplit_ele * e->nsplit_ele;
    int nsub = e->nsubele;
    e->Spa_int = new double **[nt];
    e->list_int = new int *[nt];
    for (int it = 0; it < nt; it++) {
      memory->create(e->Spa_int[it], e->numint[it + 1], npe, "harness:Spa_int");
      memory->create(e->list_int[it], e->numint[it + 1], "harness:list_int");
    }
    memory->create(e->node_list, nt + 1, npe, "harness:node_list");
    memory->create(e->sub_ele_pc, nsub, npe, 3, "harness:sub_ele_pc");
    memory->create(e->center_subele_pc, nsub, 3, "harness:center_subele_pc");
    memory->create(e->Spa_center_subele, nsub, npe, "harness:Spa_center_subele");
    memory->create(e->natom_subele, nsub, "harness:natom_subele");
    e->intp_pcoord();
    e->shape_array_int();
    e->specify_sub_ele_pc(0);
    e->count_sub_element();
    e->Spa_inter_subele = new double **[nsub];
    e->list_inter_subele = new int *[nsub];
    for (int s = 0; s < nsub; s++) {
      int n = e->natom_subele[s] > 0 ? e->natom_subele[s] : 1;
      memory->create(e->Spa_inter_subele[s], n, npe, "harness:Spa_inter_subele");
      memory->create(e->list_inter_subele[s], n, "harness:list_inter_subele");
    }
    e->shape_array_inter_subele();
    for (int it = 0; it < nt; it++) {
      int ny = e->nae[it + 1][1], nz = e->nae[it + 1][2];
      for (int jj = 0; jj < e->numint[it + 1]; jj++)
        e->list_int[it][jj] = (e->intp[it][jj][0] * ny + e->intp[it][jj][1]) * nz +
                              e->intp[it][jj][2];
    }
    if (eam) e->find_node_list();

    Neighbor *nb = cac->neighbor;
    nb->nilist = new NodeNeighList(cac);
    nb->nilist->setup_pages(nb->pgsize, nb->oneatom, 0);
    int maxint = 0;
    for (int it = 1; it <= nt; it++) maxint = e->numint[it] > maxint ? e->numint[it] : maxint;
    int emax = e->nmax > 1 ? e->nmax : 1;
    nb->nilist->grow(emax, emax * (maxint > 27 ? maxint : 27));
    tables_ready = 1;
  }

  void setup() {
    cac->init();
    eam = strcmp(cac->force->pair_style, "eam") == 0;
    if (cac->element_flag) build_element_tables();
    if (cac->atom->nlocal > 0 || capacity > 0) {
      Neighbor *nb = cac->neighbor;
      cac->memory->create(nb->xhold, capacity > 0 ? capacity : 1, 3, "harness:xhold");
      nb->maxhold = capacity;
    }
    cac->comm->setup();
    cac->neighbor->setup_bins();
    ensure_ebinhead();
    cac->comm->exchange();
    cac->comm->borders();
    refresh_avec_x();
    check_capacity();
    cac->neighbor->ago = 0;
  }

  void hold_atoms() {
    Neighbor *nb = cac->neighbor;
    Atom *atom = cac->atom;
    for (int i = 0; i < atom->nlocal; i++) {
      nb->xhold[i][0] = atom->x[i][0];
      nb->xhold[i][1] = atom->x[i][1];
      nb->xhold[i][2] = atom->x[i][2];
    }
  }

  void atom_build() {
    cac->neighbor->build();
    cac->force->pair->init_list(0, cac->neighbor->lists[0]);
    hold_atoms();
  }

  void elem_build() {
    cac->neighbor->setup_cut();
    cac->neighbor->ebuild();
    cac->neighbor->nbuild();
    cac->force->pair->init_nilist(cac->neighbor->nilist);
  }

  void dump_atom_list() {
    Atom *atom = cac->atom;
    NeighList *list = cac->neighbor->lists[0];
    int nall = atom->nlocal + atom->nghost;
    std::vector<int> counts, entries, tags;
    std::vector<double> xall;
    for (int ii = 0; ii < list->inum; ii++) {
      int i = list->ilist[ii];
      counts.push_back(list->numneigh[i]);
      for (int k = 0; k < list->numneigh[i]; k++) entries.push_back(list->firstneigh[i][k]);
    }
    for (int i = 0; i < nall; i++) {
      tags.push_back(atom->tag[i]);
      xall.push_back(atom->x[i][0]);
      xall.push_back(atom->x[i][1]);
      xall.push_back(atom->x[i][2]);
    }
    std::vector<int> meta(2);
    meta[0] = atom->nlocal;
    meta[1] = atom->nghost;
    write_i32("atom_meta.i32", meta);
    write_i32("atom_numneigh.i32", counts);
    write_i32("atom_neigh.i32", entries);
    write_i32("atom_tag_all.i32", tags);
    write_f64("atom_x_all.f64", xall);
  }

  void dump_elem_lists() {
    Element *e = cac->element;
    NeighList *list = cac->neighbor->lists[0];
    NodeNeighList *nl = cac->neighbor->nilist;
    int nall = e->nlocal + e->nghost;
    std::vector<int> ecounts, eentries, tags, ncounts, nj, nnj, meta(4);
    std::vector<double> xall, nodeall;
    for (int ii = 0; ii < list->einum; ii++) {
      int i = list->eilist[ii];
      ecounts.push_back(list->enumneigh[i]);
      for (int k = 0; k < list->enumneigh[i]; k++) eentries.push_back(list->efirstneigh[i][k]);
    }
    for (int r = 0; r < nl->ninum; r++) {
      ncounts.push_back(nl->numneigh[r]);
      for (int k = 0; k < nl->numneigh[r]; k++) {
        nj.push_back(nl->firstneigh[r][k]);
        nnj.push_back(nl->nfirstneigh[r][k]);
      }
    }
    for (int i = 0; i < nall; i++) {
      tags.push_back(e->tag[i]);
      for (int d = 0; d < 3; d++) xall.push_back(e->x[i][d]);
      for (int k = 0; k < e->npe; k++)
        for (int d = 0; d < 3; d++) nodeall.push_back(e->nodex[i][k][d]);
    }
    meta[0] = e->nlocal;
    meta[1] = e->nghost;
    meta[2] = nl->ninum;
    meta[3] = nl->neinum;
    write_i32("elem_meta.i32", meta);
    write_i32("elem_numneigh.i32", ecounts);
    write_i32("elem_neigh.i32", eentries);
    write_i32("elem_tag_all.i32", tags);
    write_f64("elem_x_all.f64", xall);
    write_f64("elem_nodex_all.f64", nodeall);
    write_i32("ip_numneigh.i32", ncounts);
    write_i32("ip_neigh_elem.i32", nj);
    write_i32("ip_neigh_site.i32", nnj);
    std::vector<double> cut(6);
    Neighbor *nb = cac->neighbor;
    cut[0] = nb->cutneighmax;
    cut[1] = nb->cut_all;
    cut[2] = nb->cut_ele;
    cut[3] = nb->cut_subele;
    cut[4] = e->max_size;
    cut[5] = (double) e->nsubele;
    write_f64("elem_cuts.f64", cut);
  }

  void atom_forces() {
    Atom *atom = cac->atom;
    for (int i = 0; i < atom->nlocal; i++) atom->f[i][0] = atom->f[i][1] = atom->f[i][2] = 0.0;
    cac->force->pair->compute(0, 0);
  }

  void elem_forces() {
    // PairEAM::ecompute aborts on purpose once ntimestep > 334
    // (pair_eam.cpp:826-925); the step number is not otherwise used there.
    bigint saved = cac->update->ntimestep;
    if (saved > 334) cac->update->ntimestep = 334;
    Element *e = cac->element;
    for (int i = 0; i < e->nlocal; i++)
      for (int k = 0; k < e->npe; k++) e->nodef[i][k][0] = e->nodef[i][k][1] = e->nodef[i][k][2] = 0.0;
    cac->force->pair->ecompute();
    cac->update->ntimestep = saved;
  }

  void dump_atom_forces(const char *name) {
    Atom *atom = cac->atom;
    std::vector<double> f;
    for (int i = 0; i < atom->nlocal; i++)
      for (int d = 0; d < 3; d++) f.push_back(atom->f[i][d]);
    write_f64(name, f);
  }

  void dump_nodef(const char *name) {
    Element *e = cac->element;
    std::vector<double> f;
    for (int i = 0; i < e->nlocal; i++)
      for (int k = 0; k < e->npe; k++)
        for (int d = 0; d < 3; d++) f.push_back(e->nodef[i][k][d]);
    write_f64(name, f);
  }

  void dump_state(const std::string &tag) {
    Atom *atom = cac->atom;
    Element *e = cac->element;
    std::vector<double> x, v, f, nx, nv, nf, ex;
    std::vector<int> at, et;
    for (int i = 0; i < atom->nlocal; i++) {
      at.push_back(atom->tag[i]);
      for (int d = 0; d < 3; d++) {
        x.push_back(atom->x[i][d]);
        v.push_back(atom->v[i][d]);
        f.push_back(atom->f[i][d]);
      }
    }
    for (int i = 0; i < e->nlocal; i++) {
      et.push_back(e->tag[i]);
      for (int d = 0; d < 3; d++) ex.push_back(e->x[i][d]);
      for (int k = 0; k < e->npe; k++)
        for (int d = 0; d < 3; d++) {
          nx.push_back(e->nodex[i][k][d]);
          nv.push_back(e->nodev[i][k][d]);
          nf.push_back(e->nodef[i][k][d]);
        }
    }
    write_i32((tag + "_atom_tag.i32").c_str(), at);
    write_f64((tag + "_x.f64").c_str(), x);
    write_f64((tag + "_v.f64").c_str(), v);
    write_f64((tag + "_f.f64").c_str(), f);
    write_i32((tag + "_elem_tag.i32").c_str(), et);
    write_f64((tag + "_elem_x.f64").c_str(), ex);
    write_f64((tag + "_nodex.f64").c_str(), nx);
    write_f64((tag + "_nodev.f64").c_str(), nv);
    write_f64((tag + "_nodef.f64").c_str(), nf);
  }

  // One Verlet::run iteration (verlet.cpp:163-218) with Pair::compute added
  // for atoms, which the reference's loop never calls.
  void step(int nrebuild_count[1]) {
    Update *update = cac->update;
    Atom *atom = cac->atom;
    Neighbor *nb = cac->neighbor;
    update->ntimestep++;
    cac->modify->initial_integrate(0);
    int nflag = nb->decide();
    if (nflag == 0) {
      if (atom->nlocal) cac->comm->forward_comm();
      if (cac->element_flag) cac->comm->eforward_comm();
    } else {
      nrebuild_count[0]++;
      if (atom->nlocal) cac->domain->pbc();
      if (cac->element_flag) cac->domain->elepbc();
      if (cac->element_flag) cac->element->element_size();
      nb->setup_cut();
      cac->comm->setup();
      nb->setup_bins();
      ensure_ebinhead();
      cac->comm->exchange();
      cac->comm->borders();
      refresh_avec_x();
      check_capacity();
      if (atom->nlocal) atom_build();
      if (cac->element_flag) {
        nb->ebuild();
        nb->nbuild();
      }
    }
    if (cac->element_flag) {
      Element *e = cac->element;
      for (int i = 0; i < e->nlocal; i++)
        for (int k = 0; k < e->npe; k++)
          e->nodef[i][k][0] = e->nodef[i][k][1] = e->nodef[i][k][2] = 0.0;
    }
    if (atom->nlocal) atom_forces();
    if (cac->element_flag) elem_forces();
    if (cac->modify->n_post_force) cac->modify->post_force(0);  // verlet.cpp:206
    cac->modify->final_integrate();
  }

  // Output::centro_atom over the atom list (output.cpp:352-447)
  void dump_centro() {
    cac->output->centro_atom(cac->neighbor->lists[0]);
    std::vector<double> c(cac->output->centro, cac->output->centro + cac->atom->nlocal);
    write_f64("centro.f64", c);
  }
};

int main(int argc, char **argv) {
  if (argc != 4) {
    fprintf(stderr, "usage: cacref <input-script> <directives> <outdir>\n");
    return 2;
  }
  g_out = argv[3];
  MPI_Init(&argc, &argv);

  std::vector<std::string> directives;
  {
    FILE *df = fopen(argv[2], "r");
    if (!df) {
      fprintf(stderr, "cacref: cannot open %s\n", argv[2]);
      return 2;
    }
    char line[1024];
    while (fgets(line, sizeof(line), df)) {
      std::string s(line);
      while (!s.empty() && (s[s.size() - 1] == '\n' || s[s.size() - 1] == ' ')) s.erase(s.size() - 1);
      if (!s.empty() && s[0] != '#') directives.push_back(s);
    }
    fclose(df);
  }

  char *cargv[4];
  cargv[0] = (char *) "cacref";
  cargv[1] = (char *) "-in";
  cargv[2] = argv[1];
  cargv[3] = NULL;
  Harness h;
  h.cac = new CAC(3, cargv, MPI_COMM_WORLD);
  // Element's constructor leaves image uninitialised (element.cpp:24-97) and
  // Element::grow reallocates it (element.cpp:172).
  h.cac->element->image = NULL;
  // FixNVE prints one line per atom per step to screen (fix_nve.cpp:89).
  h.cac->screen = fopen("/dev/null", "w");

  size_t first = 0;
  if (!directives.empty() && directives[0].compare(0, 9, "capacity ") == 0) {
    h.capacity = atoi(directives[0].c_str() + 9);
    first = 1;
  }
  h.prealloc_atoms();
  h.cac->input->file();
  h.refresh_avec_x();

  int nrebuild[1] = {0};
  for (size_t d = first; d < directives.size(); d++) {
    const std::string &cmd = directives[d];
    if (cmd == "setup") {
      h.setup();
    } else if (cmd == "atom_list") {
      h.atom_build();
      h.dump_atom_list();
    } else if (cmd == "centro") {
      h.dump_centro();
    } else if (cmd == "atom_forces") {
      h.atom_forces();
      h.dump_atom_forces("atom_f.f64");
    } else if (cmd == "elem_lists") {
      h.elem_build();
      h.dump_elem_lists();
    } else if (cmd == "elem_forces") {
      h.elem_forces();
      h.dump_nodef("nodef.f64");
    } else if (cmd.compare(0, 5, "step ") == 0) {
      int n = atoi(cmd.c_str() + 5);
      for (int s = 0; s < n; s++) h.step(nrebuild);
      std::vector<int> r(1, nrebuild[0]);
      write_i32("rebuilds.i32", r);
    } else if (cmd.compare(0, 11, "velocities ") == 0) {
      FILE *vf = fopen(cmd.c_str() + 11, "rb");
      if (!vf) {
        fprintf(stderr, "cacref: cannot open %s\n", cmd.c_str() + 11);
        return 2;
      }
      std::vector<double> vin;
      double buf[3];
      while (fread(buf, sizeof(double), 3, vf) == 3) vin.insert(vin.end(), buf, buf + 3);
      fclose(vf);
      Atom *atom = h.cac->atom;
      for (int i = 0; i < atom->nlocal; i++) {
        int t = atom->tag[i] - 1;
        if (t < 0 || 3 * (size_t) t + 2 >= vin.size()) {
          fprintf(stderr, "cacref: velocity file too short\n");
          return 2;
        }
        for (int d = 0; d < 3; d++) atom->v[i][d] = vin[3 * t + d];
      }
    } else if (cmd.compare(0, 6, "state ") == 0) {
      h.dump_state(cmd.substr(6));
    } else if (cmd == "eam_tables") {
      PairEAM *p = (PairEAM *) h.cac->force->pair;
      const int f1 = p->type2frho[1], r1 = p->type2rhor[1][1], z1 = p->type2z2r[1][1];
      std::vector<double> fr, rr, zr;
      for (int m = 0; m <= p->nrho; m++)
        for (int k = 0; k < 7; k++) fr.push_back(p->frho_spline[f1][m][k]);
      for (int m = 0; m <= p->nr; m++)
        for (int k = 0; k < 7; k++) {
          rr.push_back(p->rhor_spline[r1][m][k]);
          zr.push_back(p->z2r_spline[z1][m][k]);
        }
      write_f64("eam_frho.f64", fr);
      write_f64("eam_rhor.f64", rr);
      write_f64("eam_z2r.f64", zr);
      std::vector<double> sc(6);
      sc[0] = p->nr;
      sc[1] = p->dr;
      sc[2] = p->nrho;
      sc[3] = p->drho;
      sc[4] = p->cutforcesq;
      sc[5] = h.cac->atom->mass[1];
      write_f64("eam_scalars.f64", sc);
    } else if (cmd == "lj_tables") {
      PairLJCut *p = (PairLJCut *) h.cac->force->pair;
      const int nt = h.cac->atom->ntypes;
      std::vector<double> l1, l2, cs;
      for (int i = 0; i <= nt; i++)
        for (int j = 0; j <= nt; j++) {
          const bool set = i >= 1 && j >= 1;
          l1.push_back(set ? p->lj1[i][j] : 0.0);
          l2.push_back(set ? p->lj2[i][j] : 0.0);
          cs.push_back(set ? p->cutsq[i][j] : 0.0);
        }
      write_f64("lj_lj1.f64", l1);
      write_f64("lj_lj2.f64", l2);
      write_f64("lj_cutsq.f64", cs);
    } else {
      fprintf(stderr, "cacref: unknown directive '%s'\n", cmd.c_str());
      return 2;
    }
  }
  fflush(stdout);
  // The reference destructors free tables the harness allocated with its own
  // layout; the process exits instead of deleting the CAC instance.
  return 0;
}
