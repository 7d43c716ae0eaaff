/*
 * CPU oracle of DISCUS's Fourier path -- TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py (cpu_baseline leg and the
 * --impl reference arm) may load this library, and only as the reference for
 * comparisons or the timed CPU baseline.  The product path (diffusecode_gb300) never calls it.
 *
 * PARITY UNPINNED: the reference (Fortran) cannot be compiled in this
 * environment (no Fortran compiler) and ships no tests, golden vectors or
 * fixtures for this path.  This restatement is pinned instead to
 * closed-form known answers (tests/golden/make_golden.py) and to its own
 * exact-FP64 mode within the reference's documented lookup-table floor.
 *
 * Two modes:
 *   REF22   -- the reference's arithmetic: 2^22 fixed-point increments, the
 *              2^16-entry FP64 cos/sin table with truncating index, istl
 *              quantised form factors, FP64 accumulation in the reference's
 *              summation order.
 *   EXACT64 -- h.r mod 1 formed with error-free FP64 products, FP64 sin/cos,
 *              optionally the form factor at the exact sin(theta)/lambda.
 */
#ifndef DISCUS_ORACLE_H
#define DISCUS_ORACLE_H

#include <stdint.h>
#include "../include/discus_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

int  oc_fourier_lmn(const double eck[12], const double vi[9], const int32_t inc[3],
                    int32_t lmn[6], double off[9]);
void oc_cexpt(double *cex);
int  oc_stltab(const double eck[12], const double vi[9], const int32_t num[3],
               const double rten[9], int32_t *istl);
void oc_formtab(const dgpu_crystal *cr, const dgpu_opts *op, double *cfact);
void oc_increments(const double *xat, int64_t nxat, const double uin[3],
                   const double vin[3], const double win[3], const double off[9],
                   int64_t *inc6);
void oc_strucf_ref(const double *xat, const float *w, int64_t nxat,
                   const double uin[3], const double vin[3], const double win[3],
                   const double off[9], const int32_t lmn[6], const int32_t num[3],
                   const int32_t fnum[3], const double *cex, int32_t row_lo,
                   int32_t row_hi, int nthreads, double *tcsf);
int  oc_four_strucf(const double *xat, int64_t nxat, const double uin[3],
                    const double vin[3], const double win[3], const double off[9],
                    const int32_t lmn[6], const int32_t num[3], const int32_t fnum[3],
                    const double *cfact, const int32_t *istl, double *tcsf);
int  oc_four_run(const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op,
                 double *csf, double *acsf, double *dsi, dgpu_info *info, int nthreads);
int  oc_chi2_grad(const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op,
                  const double *i_target, const double *weight, double *chi2,
                  double *grad_pos, double *grad_occ, int nthreads);
int  oc_four_weight(const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op,
                    const double *dsi, double *dsi3d, double *scalef);
void oc_fill_bragg(const dgpu_grid *grid, double *a, int comp);
void oc_four_symm(const dgpu_grid *grid, int32_t nops, const double *mats, double *a, int comp);
int  oc_qval(const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op, int value, int laver,
             const double *csf, const double *acsf, const double *dsi, const double *rnd, double *out);
int  oc_calc_hkl(const dgpu_crystal *cr, const dgpu_opts *op, const int32_t *hkl, int64_t nrefl, double scale,
                 double exti, double rlambda, double *icalc, double *sigi, double *phase, int nthreads);
int  oc_powder_npkt(const dgpu_powder *pw);
int  oc_powder_complete(const dgpu_crystal *cr, const dgpu_powder *pw, const dgpu_opts *op, int64_t rod_lo,
                        int64_t rod_hi, double *qsp, int64_t *nrods, int64_t *npoints, int nthreads);
double oc_time_ref_rows(const dgpu_crystal *cr, const dgpu_grid *grid, int32_t row_lo,
                        int32_t row_hi, int nthreads, int64_t *pairs_out);

#ifdef __cplusplus
}
#endif
#endif
