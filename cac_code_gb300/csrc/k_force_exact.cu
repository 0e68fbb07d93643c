// FP64 pair kernels, reference operation order without contraction (bit-identical to the CPU reference).
// Build flag: -fmad=false.  Kernel bodies live in force_fp64.cuh.
#define FP64NS fp64_exact
#include "force_fp64.cuh"

namespace cacg {
namespace fp64_exact {

namespace {
inline int nblk(long long n, int t) { return (int) ((n + t - 1) / t); }
}

void lj_atoms(const double4 *x, const int *type, const int *num, const int *list, int stride,
              int nlocal, const void *tab, double *f, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_lj_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(x, type, num, list, stride, nlocal,
                                              (const LJTab *) tab, f);
  check(cudaGetLastError(), "lj_atoms");
}

void eam_rho_atoms(const double4 *x, const int *num, const int *list, int stride, int nlocal,
                   EamTables e, double *rho, double *fp, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_eam_rho_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(x, num, list, stride, nlocal, e, rho, fp);
  check(cudaGetLastError(), "eam_rho_atoms");
}

void eam_force_atoms(const double4 *x, const int *num, const int *list, int stride, int nlocal,
                     EamTables e, const double *fp, double *f, cudaStream_t s) {
  if (nlocal <= 0) return;
  k_eam_force_atoms<<<nblk(nlocal, 128), 128, 0, s>>>(x, num, list, stride, nlocal, e, fp, f);
  check(cudaGetLastError(), "eam_force_atoms");
}

void lj_ip(const double *nodex, const int *etype, const int *row_elem, const int *row_jj,
           int nrows, const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,
           ElemTables t, double lj1, double lj2, double cutsq, double *fip, cudaStream_t s) {
  if (nrows <= 0) return;
  k_lj_ip<<<nblk(nrows, 128), 128, 0, s>>>(nodex, etype, row_elem, row_jj, nrows, ipnum, ipent,
                                          rowstride, site_x, t, lj1, lj2, cutsq, fip);
  check(cudaGetLastError(), "lj_ip");
}

void eam_erho(const double *nodex, const int *etype, const int *row_first, int nlocal_e,
              const int *ipnum, const int *ipent, int rowstride, const double4 *site_x,
              ElemTables t, EamTables e, double *erho, cudaStream_t s) {
  if (nlocal_e <= 0) return;
  k_eam_erho<<<nblk((long long) nlocal_e * NPE, 128), 128, 0, s>>>(
      nodex, etype, row_first, nlocal_e, ipnum, ipent, rowstride, site_x, t, e, erho);
  check(cudaGetLastError(), "eam_erho");
}

void eam_site_fp(const double *erho, const int *etype, const int *site_base, int nelem,
                 ElemTables t, EamTables e, double *site_fp, cudaStream_t s) {
  if (nelem <= 0) return;
  k_eam_site_fp<<<nelem, 128, 0, s>>>(erho, etype, site_base, t, e, site_fp);
  check(cudaGetLastError(), "eam_site_fp");
}

void eam_ip(const double *nodex, const double *erho, const int *etype, const int *row_elem,
            const int *row_jj, int nrows, const int *ipnum, const int *ipent, int rowstride,
            const double4 *site_x, const double *site_fp, ElemTables t, EamTables e, double *fip,
            cudaStream_t s) {
  if (nrows <= 0) return;
  k_eam_ip<<<nblk(nrows, 128), 128, 0, s>>>(nodex, erho, etype, row_elem, row_jj, nrows, ipnum,
                                           ipent, rowstride, site_x, site_fp, t, e, fip);
  check(cudaGetLastError(), "eam_ip");
}

void gather_nodef(const double *fip, const int *etype, const int *row_first, int nlocal_e,
                  ElemTables t, double *nodef, cudaStream_t s) {
  if (nlocal_e <= 0) return;
  k_gather_nodef<<<nblk((long long) nlocal_e * 24, 128), 128, 0, s>>>(fip, etype, row_first,
                                                                     nlocal_e, t, nodef);
  check(cudaGetLastError(), "gather_nodef");
}

}  // namespace fp64_exact
}  // namespace cacg
