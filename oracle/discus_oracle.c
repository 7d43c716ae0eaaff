/*
 * CPU oracle of DISCUS's Fourier path -- TEST INFRASTRUCTURE ONLY.
 * See discus_oracle.h: parity unpinned (no Fortran compiler, no reference
 * tests); only tests/, smoke() and bench.py's CPU legs may use this file.
 *
 * Every function cites the reference routine it restates (paths relative to
 * the DiffuseCode source tree).  Build: oracle/build_oracle.sh (gcc, OpenMP,
 * -ffp-contract=off so that a*b+c is never fused: the reference's own
 * rounding under -ffast-math is compiler dependent, this file fixes one).
 */
#include "discus_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CFPKT DGPU_CFPKT
#define NTAB  (CFPKT + 1)

/* ---------------------------------------------------------------------- */
/* quad precision for fourier_lmn (PREC_QP, lib_f90/precision_mod.f90:13)  */
#if defined(__aarch64__)
typedef long double qreal;           /* IEEE binary128 on aarch64 */
#else
typedef __float128 qreal;            /* IEEE binary128 on x86_64 */
#endif

static qreal q_abs(qreal x) { return x < 0 ? -x : x; }
static qreal q_sqrt(qreal x)
{
    if (x <= 0) return 0;
    qreal y = (qreal)sqrt((double)x);
    y = 0.5 * (y + x / y);           /* two Newton steps from a double seed */
    y = 0.5 * (y + x / y);
    return y;
}
/* Fortran NINT: round half away from zero */
static int64_t q_nint(qreal x)
{
    return x >= 0 ? (int64_t)(x + (qreal)0.5) : -(int64_t)(-x + (qreal)0.5);
}

#define M3(a, r, c) (a)[3 * (c) + (r)]          /* column-major 3x3, 0-based */

/* matinv3_q / det3_q, lib_f90/matrix_mod.f90:81-92,271-300 */
static int q_matinv3(const qreal *a, qreal *b)
{
    qreal det = M3(a,0,0)*M3(a,1,1)*M3(a,2,2) - M3(a,0,0)*M3(a,1,2)*M3(a,2,1)
              - M3(a,0,1)*M3(a,1,0)*M3(a,2,2) + M3(a,0,1)*M3(a,1,2)*M3(a,2,0)
              + M3(a,0,2)*M3(a,1,0)*M3(a,2,1) - M3(a,0,2)*M3(a,1,1)*M3(a,2,0);
    for (int i = 0; i < 9; i++) b[i] = 0;
    if (det == 0) return -1;
    qreal di = (qreal)1 / det;
    M3(b,0,0) = +di * (M3(a,1,1)*M3(a,2,2) - M3(a,1,2)*M3(a,2,1));
    M3(b,1,0) = -di * (M3(a,1,0)*M3(a,2,2) - M3(a,1,2)*M3(a,2,0));
    M3(b,2,0) = +di * (M3(a,1,0)*M3(a,2,1) - M3(a,1,1)*M3(a,2,0));
    M3(b,0,1) = -di * (M3(a,0,1)*M3(a,2,2) - M3(a,0,2)*M3(a,2,1));
    M3(b,1,1) = +di * (M3(a,0,0)*M3(a,2,2) - M3(a,0,2)*M3(a,2,0));
    M3(b,2,1) = -di * (M3(a,0,0)*M3(a,2,1) - M3(a,0,1)*M3(a,2,0));
    M3(b,0,2) = +di * (M3(a,0,1)*M3(a,1,2) - M3(a,0,2)*M3(a,1,1));
    M3(b,1,2) = -di * (M3(a,0,0)*M3(a,1,2) - M3(a,0,2)*M3(a,1,0));
    M3(b,2,2) = +di * (M3(a,0,0)*M3(a,1,1) - M3(a,0,1)*M3(a,1,0));
    return 0;
}

/* fourier_lmn, discus/prog/fourier_lmn_mod.f90:4-279.
 * The ran1 draws of the "line through the origin" branch (:185-195) only
 * feed offset directions whose lmn multiplier is zero, so fixed values are
 * used here. */
int oc_fourier_lmn(const double eck_in[12], const double vi_in[9], const int32_t inc[3],
                   int32_t lmn[6], double off_out[9])
{
    const qreal big = 10000000;
    const qreal eps7 = (qreal)1.0e-7f;               /* 1.0E-7 default real */
    const qreal tiny = (qreal)1.0e-9;                /* 1.0D-9 */
    qreal eck[12], vi[9], off[9], mat_a[9], mat_i[9], vec_r[3], vec_t[3];
    int direc[3] = {0, 0, 0}, nooff[3] = {0, 0, 0}, dimen = 0, need_work = 1;
    static const double ranv[6] = {0.3141592, 0.2718281, 0.5772156,
                                   0.6931471, 0.4142135, 0.7320508};

    for (int i = 0; i < 12; i++) eck[i] = (qreal)q_nint((qreal)eck_in[i] * big) / big;
    for (int i = 0; i < 9; i++)  vi[i]  = (qreal)q_nint((qreal)vi_in[i] * big) / big;
    for (int i = 0; i < 9; i++) { mat_a[i] = 0; mat_i[i] = 0; off[i] = 0; }
    for (int i = 0; i < 6; i++) lmn[i] = 0;

    for (int i = 0; i < 3; i++) {
        if (inc[i] > 1) {
            qreal d = q_sqrt(q_abs(M3(vi,0,i)*M3(vi,0,i) + M3(vi,1,i)*M3(vi,1,i)
                                   + M3(vi,2,i)*M3(vi,2,i)));
            if (d > eps7) {
                direc[dimen++] = i;
                nooff[i] = 1;
                for (int j = 0; j < 3; j++) M3(mat_a,j,i) = M3(vi,j,i);
            } else {
                return DGPU_ERR_ZERO_INC;              /* ier_num = -132 */
            }
        }
    }

    if (dimen == 0) {
        M3(off,0,0) = 1; M3(off,1,1) = 1; M3(off,2,2) = 1;
        for (int i = 0; i < 9; i++) mat_a[i] = off[i];
    } else if (dimen == 1) {
        int j = direc[0], j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        /* axis-parallel rows (:103-169) read vi(:,1) and set everything */
        if (M3(vi,1,j) == 0 && M3(vi,2,j) == 0) {            /* parallel a* */
            if (M3(vi,0,0) == 0) return DGPU_ERR_ARG;
            qreal r = M3(eck,0,0) / M3(vi,0,0);
            lmn[0] = (int32_t)q_nint(r);
            if (q_abs(r - (qreal)q_nint(r)) > tiny) { lmn[3] = 1; M3(off,0,0) = r - (qreal)q_nint(r); }
            lmn[4] = 1; lmn[5] = 1;
            M3(off,1,1) = M3(eck,1,0);
            M3(off,2,2) = M3(eck,2,0);
            need_work = 0;
        } else if (M3(vi,0,j) == 0 && M3(vi,2,j) == 0) {     /* parallel b* */
            if (M3(vi,1,0) == 0) return DGPU_ERR_ARG;
            qreal r = M3(eck,1,0) / M3(vi,1,0);
            lmn[0] = (int32_t)q_nint(r);
            if (q_abs(r - (qreal)q_nint(r)) > tiny) { lmn[3] = 1; M3(off,1,0) = r - (qreal)q_nint(r); }
            lmn[4] = 1; lmn[5] = 1;
            M3(off,0,1) = M3(eck,0,0);
            M3(off,2,2) = M3(eck,2,0);
            need_work = 0;
        } else if (M3(vi,0,j) == 0 && M3(vi,1,j) == 0) {     /* parallel c* */
            if (M3(vi,2,0) == 0) return DGPU_ERR_ARG;
            qreal r = M3(eck,2,0) / M3(vi,2,0);
            lmn[0] = (int32_t)q_nint(r);
            if (q_abs(r - (qreal)q_nint(r)) > tiny) { lmn[3] = 1; M3(off,2,0) = r - (qreal)q_nint(r); }
            lmn[4] = 1; lmn[5] = 1;
            M3(off,0,1) = M3(eck,0,0);
            M3(off,1,2) = M3(eck,1,0);
            need_work = 0;
        } else {
            const qreal s001 = (qreal)0.001f;          /* 0.001 default real */
            M3(off,0,j2) = M3(eck,1,0)*M3(vi,2,j) - M3(eck,2,0)*M3(vi,1,j);
            M3(off,1,j2) = M3(eck,2,0)*M3(vi,0,j) - M3(eck,0,0)*M3(vi,2,j);
            M3(off,2,j2) = M3(eck,0,0)*M3(vi,1,j) - M3(eck,1,0)*M3(vi,0,j);
            qreal d = q_sqrt(q_abs(M3(off,0,j2)*M3(off,0,j2) + M3(off,1,j2)*M3(off,1,j2)
                                   + M3(off,2,j2)*M3(off,2,j2)));
            if (d > eps7) {
                for (int k = 0; k < 3; k++) M3(off,k,j2) = M3(off,k,j2) * s001 / d;
                M3(off,0,j1) = M3(off,1,j2)*M3(vi,2,j) - M3(off,2,j2)*M3(vi,1,j);
                M3(off,1,j1) = M3(off,2,j2)*M3(vi,0,j) - M3(off,0,j2)*M3(vi,2,j);
                M3(off,2,j1) = M3(off,0,j2)*M3(vi,1,j) - M3(off,1,j2)*M3(vi,0,j);
                d = q_sqrt(q_abs(M3(off,0,j1)*M3(off,0,j1) + M3(off,1,j1)*M3(off,1,j1)
                                 + M3(off,2,j1)*M3(off,2,j1)));
                if (d > eps7) {
                    for (int k = 0; k < 3; k++) M3(off,k,j1) = M3(off,k,j1) * s001 / d;
                } else {
                    for (int k = 0; k < 3; k++) M3(off,k,j1) = ranv[k];
                }
            } else {
                for (int k = 0; k < 3; k++) { M3(off,k,j1) = ranv[k]; M3(off,k,j2) = ranv[3 + k]; }
            }
            for (int k = 0; k < 3; k++) { M3(mat_a,k,j1) = M3(off,k,j1); M3(mat_a,k,j2) = M3(off,k,j2); }
        }
    } else if (dimen == 2) {
        int j = direc[0], j1 = direc[1], j2 = 3 - j - j1;
        M3(off,0,j2) = M3(vi,1,j)*M3(vi,2,j1) - M3(vi,2,j)*M3(vi,1,j1);
        M3(off,1,j2) = M3(vi,2,j)*M3(vi,0,j1) - M3(vi,0,j)*M3(vi,2,j1);
        M3(off,2,j2) = M3(vi,0,j)*M3(vi,1,j1) - M3(vi,1,j)*M3(vi,0,j1);
        qreal d = q_sqrt(M3(off,0,j2)*M3(off,0,j2) + M3(off,1,j2)*M3(off,1,j2)
                         + M3(off,2,j2)*M3(off,2,j2));
        for (int k = 0; k < 3; k++) M3(off,k,j2) = M3(off,k,j2) * (qreal)0.001 / d;
        for (int k = 0; k < 3; k++) M3(mat_a,k,j2) = M3(off,k,j2);
    }

    if (need_work) {
        if (q_matinv3(mat_a, mat_i) != 0) return DGPU_ERR_ARG;
        for (int a = 0; a < 3; a++) {
            vec_r[a] = 0;
            for (int b = 0; b < 3; b++) vec_r[a] += M3(mat_i,a,b) * M3(eck,b,0);
        }
        for (int a = 0; a < 3; a++)
            if (q_abs(vec_r[a] - (qreal)q_nint(vec_r[a])) < tiny) vec_r[a] = (qreal)q_nint(vec_r[a]);
        qreal fr[3];
        for (int a = 0; a < 3; a++) { lmn[a] = (int32_t)q_nint(vec_r[a]); fr[a] = vec_r[a] - (qreal)q_nint(vec_r[a]); }
        for (int a = 0; a < 3; a++) {
            vec_t[a] = 0;
            for (int b = 0; b < 3; b++) vec_t[a] += M3(mat_a,a,b) * fr[b];
        }
        for (int j = 0; j < 3; j++) {
            if (!nooff[j]) {
                lmn[j + 3] = lmn[j];
                lmn[j] = 0;
            } else {
                M3(off,j,j) = M3(off,j,j) + vec_t[j];
                lmn[3 + j] = 1;
                if (q_abs(M3(off,j,j)) < tiny) { M3(off,j,j) = 0; lmn[3 + j] = 0; }
            }
        }
    }
    for (int i = 0; i < 9; i++) off_out[i] = (double)off[i];
    return DGPU_OK;
}

/* four_cexpt, fourier_sup.f90:2602-2632: cex(k) = exp(2 pi i k / 2^16) */
void oc_cexpt(double *cex)
{
    const double zpi = 2.0 * 3.1415926535897932384626433832795028841971693993751;
    for (int i = 0; i < DGPU_I2PI; i++) {
        double xarg = zpi * ((double)i * 1.0 / (double)DGPU_I2PI);
        cex[2 * i] = cos(xarg);
        cex[2 * i + 1] = sin(xarg);
    }
}

/* four_stltab, fourier_sup.f90:2637-2687.  h is rounded to default REAL
 * (single precision) before the metric, as REAL() does there; the metric
 * is skalpro = dot_product(h, matmul(rten,h)) (discus/prog/metric.f90:90-105). */
int oc_stltab(const double eck[12], const double vi[9], const int32_t num[3],
              const double rten[9], int32_t *istl)
{
    int err = 0;
    for (int l = 0; l < num[2]; l++)
        for (int j = 0; j < num[1]; j++)
            for (int i = 0; i < num[0]; i++) {
                double h[3], t[3];
                for (int k = 0; k < 3; k++)
                    h[k] = (double)(float)(eck[k] + vi[k] * (double)i + vi[3 + k] * (double)j
                                           + vi[6 + k] * (double)l);
                for (int a = 0; a < 3; a++)
                    t[a] = M3(rten,a,0) * h[0] + M3(rten,a,1) * h[1] + M3(rten,a,2) * h[2];
                double q2 = (h[0] * t[0] + h[1] * t[1] + h[2] * t[2]) / 4.0;
                long v = lround(sqrt(q2) * 1000.0);
                istl[i + (int64_t)num[0] * (j + (int64_t)num[1] * l)] = (int32_t)v;
                if (v > CFPKT) err = DGPU_ERR_STL_RANGE;
            }
    return err;
}

/* form, fourier_sup.f90:2947-2971 */
static double oc_form(const double *scat, int t, int lxray, double h2, int power)
{
    double f = scat[11 * t + 0];
    if (lxray)
        for (int i = 1; i <= power; i++)
            f = f + scat[11 * t + 2 * i - 1] * exp(-scat[11 * t + 2 * i] * h2);
    return f;
}

/* cfact for one type at sin(theta)/lambda squared q2, four_formtab body
 * (fourier_sup.f90:2716-2736): the isotropic Debye-Waller term only when all
 * ADPs are isotropic (:2729) */
static void oc_cfact_at(const dgpu_crystal *cr, const dgpu_opts *op, int t, double q2,
                        double *re, double *im)
{
    double sf = oc_form(cr->scat, t, op->lxray, q2, op->power);
    double sfp = 0, sfpp = 0, sb;
    if (op->ano) { sfp = cr->delfr ? cr->delfr[t] : 0; sfpp = cr->delfi ? cr->delfi[t] : 0; }
    if (op->ldbw && !cr->is_anis) sb = exp(-(cr->dw[t] * q2)) * cr->occ[t];
    else sb = 1.0 * cr->occ[t];
    *re = sb * (sf + sfp);
    *im = sb * sfpp;
}

/* four_formtab, fourier_sup.f90:2691-2743: cfact(0:CFPKT, 1:nscat) */
void oc_formtab(const dgpu_crystal *cr, const dgpu_opts *op, double *cfact)
{
    for (int t = 1; t <= cr->nscat; t++)
        for (int iq = 0; iq <= CFPKT; iq++) {
            double s = (double)iq * DGPU_CFINC;
            double q2 = s * s;
            double *c = cfact + 2 * ((int64_t)(t - 1) * NTAB + iq);
            oc_cfact_at(cr, op, t, q2, &c[0], &c[1]);
        }
}

/* Per-atom increments, four_strucf_OMP_mod.f90:135-149.
 * INT truncates toward zero, NINT rounds half away from zero. */
static int64_t oc_inc1(double x)
{
    double fr = x - (double)(int64_t)x + 0.0;
    return (int64_t)lround(4194304.0 * fr);          /* 64 * I2PI = 2^22 */
}
void oc_increments(const double *xat, int64_t nxat, const double uin[3],
                   const double vin[3], const double win[3], const double off[9],
                   int64_t *inc6)
{
    for (int64_t k = 0; k < nxat; k++) {
        double x0 = xat[k], x1 = xat[nxat + k], x2 = xat[2 * nxat + k];
        double xu = uin[0] * x0 + uin[1] * x1 + uin[2] * x2;
        double xv = vin[0] * x0 + vin[1] * x1 + vin[2] * x2;
        double xw = win[0] * x0 + win[1] * x1 + win[2] * x2;
        double ou = off[0] * x0 + off[1] * x1 + off[2] * x2;   /* off_shift(:,1) */
        double ov = off[3] * x0 + off[4] * x1 + off[5] * x2;
        double ow = off[6] * x0 + off[7] * x1 + off[8] * x2;
        inc6[0 * nxat + k] = oc_inc1(xu);
        inc6[1 * nxat + k] = oc_inc1(xv);
        inc6[2 * nxat + k] = oc_inc1(xw);
        inc6[3 * nxat + k] = oc_inc1(ou);
        inc6[4 * nxat + k] = oc_inc1(ov);
        inc6[5 * nxat + k] = oc_inc1(ow);
    }
}

/* four_strucf_omp, four_strucf_OMP_mod.f90:72-188 (without the form factor):
 * tcsf(j,i,h) = sum_k w_k cex(IAND(ISHFT(iarg,-6),MASK)) over rows
 * j in [row_lo,row_hi) of fnum(1); atoms summed in order for each point.   */
void oc_strucf_ref(const double *xat, const float *w, int64_t nxat,
                   const double uin[3], const double vin[3], const double win[3],
                   const double off[9], const int32_t lmn[6], const int32_t num[3],
                   const int32_t fnum[3], const double *cex, int32_t row_lo,
                   int32_t row_hi, int nthreads, double *tcsf)
{
    int64_t *inc = (int64_t *)malloc(sizeof(int64_t) * 6 * (nxat > 0 ? nxat : 1));
    oc_increments(xat, nxat, uin, vin, win, off, inc);
    const int64_t *iu = inc, *iv = inc + nxat, *iw = inc + 2 * nxat;
    const int64_t *ju = inc + 3 * nxat, *jv = inc + 4 * nxat, *jw = inc + 5 * nxat;
    int64_t n1 = num[0], n12 = (int64_t)num[0] * num[1];
    int32_t f2 = fnum[1], f3 = fnum[2];
    (void)nthreads;
#pragma omp parallel num_threads(nthreads > 0 ? nthreads : 1)
    {
        double *part = (double *)malloc(sizeof(double) * 2 * (size_t)f2 * f3);
#pragma omp for schedule(static)
        for (int32_t j = row_lo; j < row_hi; j++) {
            memset(part, 0, sizeof(double) * 2 * (size_t)f2 * f3);
            for (int64_t k = 0; k < nxat; k++) {
                int64_t iarg0 = (int64_t)lmn[0] * iu[k] + (int64_t)lmn[1] * iv[k]
                              + (int64_t)lmn[2] * iw[k] + (int64_t)lmn[3] * ju[k]
                              + (int64_t)lmn[4] * jv[k] + (int64_t)lmn[5] * jw[k]
                              + (int64_t)j * iu[k];
                double wk = w ? (double)w[k] : 1.0;
                for (int32_t i = 0; i < f2; i++) {
                    int64_t iarg = iarg0 + iv[k] * i;
                    double *p = part + 2 * (size_t)i;
                    for (int32_t h = 0; h < f3; h++) {
                        int64_t idx = (int64_t)(((uint64_t)iarg >> 6) & 0xFFFF);
                        if (w) {
                            p[2 * (size_t)h * f2]     += wk * cex[2 * idx];
                            p[2 * (size_t)h * f2 + 1] += wk * cex[2 * idx + 1];
                        } else {
                            p[2 * (size_t)h * f2]     += cex[2 * idx];
                            p[2 * (size_t)h * f2 + 1] += cex[2 * idx + 1];
                        }
                        iarg += iw[k];
                    }
                }
            }
            for (int32_t i = 0; i < f2; i++)
                for (int32_t h = 0; h < f3; h++) {
                    int64_t o = 2 * (j + n1 * i + n12 * h);
                    tcsf[o]     += part[2 * ((size_t)h * f2 + i)];
                    tcsf[o + 1] += part[2 * ((size_t)h * f2 + i) + 1];
                }
        }
        free(part);
    }
    free(inc);
}

/* four_strucf + tcsf_form_iso as one call (four_strucf_OMP_mod.f90:72-188,
 * fourier_form.f90:147-177). tcsf is zeroed over num first. */
int oc_four_strucf(const double *xat, int64_t nxat, const double uin[3],
                   const double vin[3], const double win[3], const double off[9],
                   const int32_t lmn[6], const int32_t num[3], const int32_t fnum[3],
                   const double *cfact, const int32_t *istl, double *tcsf)
{
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    double *cex = (double *)malloc(sizeof(double) * 2 * DGPU_I2PI);
    oc_cexpt(cex);
    memset(tcsf, 0, sizeof(double) * 2 * np);
    oc_strucf_ref(xat, NULL, nxat, uin, vin, win, off, lmn, num, fnum, cex, 0, fnum[0], 1, tcsf);
    if (cfact) {
        for (int32_t h = 0; h < fnum[2]; h++)
            for (int32_t j = 0; j < fnum[1]; j++)
                for (int32_t i = 0; i < fnum[0]; i++) {
                    int64_t p = i + (int64_t)num[0] * (j + (int64_t)num[1] * h);
                    int32_t q = istl[p];
                    double ar = tcsf[2 * p], ai = tcsf[2 * p + 1];
                    double br = cfact[2 * q], bi = cfact[2 * q + 1];
                    tcsf[2 * p] = ar * br - ai * bi;
                    tcsf[2 * p + 1] = ar * bi + ai * br;
                }
    }
    free(cex);
    return DGPU_OK;
}

/* ---------------------------------------------------------------------- */
/* EXACT64: h.r mod 1 with error-free products (fma) and FP64 sin/cos.     */
static double oc_frac_dot(const double h[3], double x0, double x1, double x2)
{
    double p0 = h[0] * x0, e0 = fma(h[0], x0, -p0);
    double p1 = h[1] * x1, e1 = fma(h[1], x1, -p1);
    double p2 = h[2] * x2, e2 = fma(h[2], x2, -p2);
    double s = p0 + p1, z = s - p0, es = (p0 - (s - z)) + (p1 - z);   /* TwoSum */
    double t = s + p2;  z = t - s;  double et = (s - (t - z)) + (p2 - z);
    double hi = t - nearbyint(t);
    return hi + (es + et + e0 + e1 + e2);
}

static void oc_hvec(const double eck[12], const double vi[9], int32_t i, int32_t j,
                    int32_t l, double h[3])
{
    for (int k = 0; k < 3; k++)
        h[k] = eck[k] + vi[k] * (double)i + vi[3 + k] * (double)j + vi[6 + k] * (double)l;
}

/* sum_k w_k exp(2 pi i h.x_k) on the points of fnum, exact FP64 phase */
static void oc_strucf_exact(const double *xat, const float *w, int64_t nxat,
                            const double eck[12], const double vi[9],
                            const int32_t num[3], const int32_t fnum[3], int nthreads,
                            double *tcsf)
{
    const double zpi = 6.283185307179586476925286766559;
    int64_t nf = (int64_t)fnum[0] * fnum[1] * fnum[2];
    (void)nthreads;
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t p = 0; p < nf; p++) {
        int32_t i = (int32_t)(p % fnum[0]);
        int32_t j = (int32_t)((p / fnum[0]) % fnum[1]);
        int32_t l = (int32_t)(p / ((int64_t)fnum[0] * fnum[1]));
        double h[3];
        oc_hvec(eck, vi, i, j, l, h);
        double sr = 0, si = 0;
        for (int64_t k = 0; k < nxat; k++) {
            double ph = oc_frac_dot(h, xat[k], xat[nxat + k], xat[2 * nxat + k]);
            double wk = w ? (double)w[k] : 1.0;
            sr += wk * cos(zpi * ph);
            si += wk * sin(zpi * ph);
        }
        int64_t o = i + (int64_t)num[0] * (j + (int64_t)num[1] * l);
        tcsf[2 * o] += sr;
        tcsf[2 * o + 1] += si;
    }
}

/* ---------------------------------------------------------------------- */
/* Friedel reduction, fourier_sup.f90:3645-3722 */
static int oc_test_friedel(const dgpu_grid *g, const dgpu_opts *op, int32_t fnum[3])
{
    const double EPS = (double)1.0e-6f;
    for (int k = 0; k < 3; k++) fnum[k] = g->inc[k];
    if (!op->friedel || op->ano) return 0;
    double rut[3], point[3];
    for (int k = 0; k < 3; k++) {
        rut[k] = g->eck[k] + g->vi[k] * (fnum[0] - 1) + g->vi[3 + k] * (fnum[1] - 1)
               + g->vi[6 + k] * (fnum[2] - 1);
        point[k] = g->eck[k] + rut[k];
    }
    int all_odd = (fnum[0] % 2) && (fnum[1] % 2) && (fnum[2] % 2);
    if (!all_odd) return 0;
    if (!(fabs(point[0]) < EPS && fabs(point[2]) < EPS && fabs(point[1]) < EPS)) return 0;
    if (fnum[0] > 1) { fnum[0] = (fnum[0] + 1) / 2; return 1; }
    if (fnum[1] > 1) { fnum[1] = (fnum[1] + 1) / 2; return 2; }
    if (fnum[2] > 1) { fnum[2] = (fnum[2] + 1) / 2; return 3; }
    return 0;
}

/* four_apply_friedel, fourier_sup.f90:3726-3757, in its sequential order */
static void oc_apply_friedel(const int32_t num[3], const int32_t fnum[3], double *acsf,
                             double *csf, double *dsi)
{
    for (int32_t i = 0; i < fnum[0]; i++)
        for (int32_t j = 0; j < fnum[1]; j++)
            for (int32_t k = 0; k < fnum[2]; k++) {
                int64_t s = i + (int64_t)num[0] * (j + (int64_t)num[1] * k);
                int64_t m = (num[0] - 1 - i) + (int64_t)num[0] * ((num[1] - 1 - j)
                          + (int64_t)num[1] * (num[2] - 1 - k));
                if (acsf) { acsf[2 * m] = acsf[2 * s]; acsf[2 * m + 1] = -acsf[2 * s + 1]; }
                csf[2 * m] = csf[2 * s]; csf[2 * m + 1] = -csf[2 * s + 1];
                dsi[m] = dsi[s];
            }
}

/* four_qinfo, fourier_sup.f90:2859-2942 */
static void oc_qinfo(const dgpu_grid *g, const double *dsi, double res[7])
{
    double bmax = -9999.0, bmin = (double)1e19f, dmax = -9999.0, dmin = (double)1e19f;
    double dsum = 0, dsum2 = 0;
    int64_t nd = 0;
    const int32_t *num = g->inc;
    for (int32_t l = 0; l < num[2]; l++)
        for (int32_t j = 0; j < num[1]; j++)
            for (int32_t i = 0; i < num[0]; i++) {
                int bragg = 1;
                for (int k = 0; k < 3; k++) {
                    double h = g->eck[k] + g->vi[k] * (double)(float)i
                             + g->vi[3 + k] * (double)(float)j + g->vi[6 + k] * (double)(float)l;
                    bragg = bragg && (fmod(h, 1.0) == 0.0);
                }
                double v = dsi[i + (int64_t)num[0] * (j + (int64_t)num[1] * l)];
                if (bragg) { if (v > bmax) bmax = v; if (v < bmin) bmin = v; }
                else {
                    if (v > dmax) dmax = v;
                    if (v < dmin) dmin = v;
                    dsum += v; dsum2 += v * v; nd++;
                }
            }
    double ave = 0, sig = 0;
    if (nd) { ave = dsum / (double)nd; sig = sqrt(dsum2 / (double)nd - ave * ave); }
    res[0] = 6; res[1] = dmin; res[2] = dmax; res[3] = ave; res[4] = sig;
    res[5] = bmin; res[6] = bmax;
}

/* four_csize, fourier_sup.f90:2533-2555: origins available to a lot */
static void oc_csize(const dgpu_crystal *cr, const dgpu_opts *op, int32_t cs[3])
{
    for (int k = 0; k < 3; k++) {
        int32_t c = cr->icc[k] - op->ls_xyz[k] + 1;
        cs[k] = op->lperiod ? cr->icc[k] : (c > 1 ? c : 1);
    }
}

static int oc_lots_on(const dgpu_opts *op)
{
    return op->ilots == DGPU_LOT_BOX || op->ilots == DGPU_LOT_ELI;
}

/* Cell (ii,jj,kk) of the ls_xyz box belongs to the lot: always for a box,
 * inside the inscribed ellipsoid for LOT_ELI (fourier_sup.f90:1908-1937,
 * four_getav :2488-2500), summed in the reference's order x1 + x2 + x3. */
static int oc_in_lot(const dgpu_opts *op, int32_t ii, int32_t jj, int32_t kk)
{
    if (op->ilots != DGPU_LOT_ELI) return 1;
    double x0[3], xt[3];
    int32_t d[3] = {ii, jj, kk};
    for (int k = 0; k < 3; k++) {
        x0[k] = (double)op->ls_xyz[k] / 2.0;
        double u = (double)d[k] - x0[k] + 0.5;
        xt[k] = u * u / (x0[k] * x0[k]);
    }
    return (xt[0] + xt[1] + xt[2]) <= 1.0;
}

/* Atom i is of type t and, when a > 0, of ADP type a. */
/* Atom i is of type t, ADP type a (any when a <= 0) and, with DISCAMB,
 * generated by symmetry operation y (any when y < 0): four_getatm_anis /
 * four_getatm_discamb (fourier_sup.f90:2012, 2246-2247). */
static int oc_match(const dgpu_crystal *cr, int64_t i, int t, int a, int y)
{
    if (cr->iscat[i] != t) return 0;
    if (y >= 0 && cr->isym[i] != y) return 0;
    return a <= 0 || cr->ianis[i] == a;
}

/* Gather the atoms of type t (ADP a, or any when a == 0) of one lot:
 * four_getatm / four_getatm_anis (fourier_sup.f90:1806-1970, 1975-2140).
 * LOT_OFF takes every atom at its position; a box or ellipsoid lot walks
 * its cells from lbeg (1-based, wrapped once at icc), takes the ncatoms
 * sites of each cell (celltoindex, celltoindex.f90:21-23) and the atoms
 * stored after the periodic block whose INT(pos) is that cell, all shifted
 * by the lot origin.  xat == NULL counts only; xat is SoA with stride n.
 * *ncell receives the cells of the lot. */
static int64_t oc_getatm_lot(const dgpu_crystal *cr, const dgpu_opts *op, int t, int a, int y,
                             const int32_t lbeg[3], double *xat, float *w, int64_t n,
                             int32_t *ncell, int64_t *src)
{
    int64_t m = 0;
    if (!oc_lots_on(op)) {
        *ncell = cr->icc[0] * cr->icc[1] * cr->icc[2];
        for (int64_t i = 0; i < cr->natoms; i++)
            if (oc_match(cr, i, t, a, y)) {
                if (xat) {
                    for (int k = 0; k < 3; k++) xat[k * n + m] = cr->pos[3 * i + k];
                    if (w) w[m] = cr->atom_occ ? cr->atom_occ[i] : 1.0f;
                    if (src) src[m] = i;
                }
                m++;
            }
        return m;
    }
    const int64_t cr_end = (int64_t)cr->ncatoms * cr->icc[0] * cr->icc[1] * cr->icc[2];
    int32_t nc = 0;
    for (int32_t kk = 0; kk < op->ls_xyz[2]; kk++)
        for (int32_t jj = 0; jj < op->ls_xyz[1]; jj++)
            for (int32_t ii = 0; ii < op->ls_xyz[0]; ii++) {
                int32_t d[3] = {ii, jj, kk}, icell[3];
                double off[3];
                for (int k = 0; k < 3; k++) {
                    icell[k] = d[k] + lbeg[k];
                    off[k] = cr->dim0[k] + lbeg[k] - 1;
                    if (icell[k] > cr->icc[k]) {
                        icell[k] -= cr->icc[k];
                        off[k] -= (double)cr->icc[k];
                    }
                }
                if (!oc_in_lot(op, ii, jj, kk)) continue;
                nc++;
                int64_t c = (icell[2] - 1) * (int64_t)cr->icc[0] * cr->icc[1]
                          + (icell[1] - 1) * (int64_t)cr->icc[0] + (icell[0] - 1);
                for (int32_t is = 0; is < cr->ncatoms; is++) {
                    int64_t ia = c * cr->ncatoms + is;
                    if (ia >= cr->natoms || !oc_match(cr, ia, t, a, y)) continue;
                    if (xat) {
                        for (int k = 0; k < 3; k++) xat[k * n + m] = cr->pos[3 * ia + k] - off[k];
                        if (w) w[m] = cr->atom_occ ? cr->atom_occ[ia] : 1.0f;
                        if (src) src[m] = ia;
                    }
                    m++;
                }
                int64_t jc[3];
                for (int k = 0; k < 3; k++) jc[k] = icell[k] + lround(cr->dim_lo[k]) - 1;
                for (int64_t ir = cr_end; ir < cr->natoms; ir++) {
                    if ((int64_t)cr->pos[3 * ir] != jc[0] || (int64_t)cr->pos[3 * ir + 1] != jc[1] ||
                        (int64_t)cr->pos[3 * ir + 2] != jc[2] || !oc_match(cr, ir, t, a, y))
                        continue;
                    if (xat) {
                        for (int k = 0; k < 3; k++) xat[k * n + m] = cr->pos[3 * ir + k] - off[k];
                        if (w) w[m] = cr->atom_occ ? cr->atom_occ[ir] : 1.0f;
                        if (src) src[m] = ir;
                    }
                    m++;
                }
            }
    *ncell = nc;
    return m;
}

/* four_nanis, fourier_sup.f90:4294-4326: the ADP types met among the atoms
 * of type t, in order of first appearance. */
static int oc_anis_list(const dgpu_crystal *cr, int t, int32_t *list)
{
    int n = 0;
    for (int64_t i = 0; i < cr->natoms; i++) {
        if (cr->iscat[i] != t) continue;
        int seen = 0;
        for (int j = 0; j < n && !seen; j++) seen = list[j] == cr->ianis[i];
        if (!seen) list[n++] = cr->ianis[i];
    }
    return n;
}

/* four_dbw of ADP type a at h, four_dbwtab (fourier_sup.f90:2809-2831),
 * zpi*pi = 2 pi^2 (lib_f90/wink_mod.f90:10-11). */
static double oc_dbw(const dgpu_crystal *cr, int a, const double h[3])
{
    const double pi = 3.1415926535897932384626433832795028841971693993751;
    const double *u = cr->anis_full + 6 * (int64_t)(a - 1), *r = cr->ar;
    double arg = ((h[0] * h[0] * r[0] * r[0] * u[0]) +
                  (h[1] * h[1] * r[1] * r[1] * u[1]) +
                  (h[2] * h[2] * r[2] * r[2] * u[2]) +
                  (h[1] * h[2] * r[1] * r[2] * u[3]) * 2.0 +
                  (h[0] * h[2] * r[0] * r[2] * u[4]) * 2.0 +
                  (h[0] * h[1] * r[0] * r[1] * u[5]) * 2.0) * (2.0 * pi) * pi;
    return exp(-arg);
}

/* Multiply by the form factor on fnum, by table (istl) or at the exact
 * sin(theta)/lambda: tcsf_form_iso (fourier_form.f90:147-177), or, for ADP
 * type a > 0, tcsf_form_aniso (fourier_form.f90:106-143) with four_dbw = 1
 * unless ldbw (fourier_sup.f90:2797-2800). */
static void oc_apply_form(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op,
                          int t, int a, const double *cfact, const int32_t *istl,
                          const int32_t fnum[3], double *tcsf)
{
    const int32_t *num = g->inc;
    for (int32_t l = 0; l < fnum[2]; l++)
        for (int32_t j = 0; j < fnum[1]; j++)
            for (int32_t i = 0; i < fnum[0]; i++) {
                int64_t p = i + (int64_t)num[0] * (j + (int64_t)num[1] * l);
                double br, bi, h[3];
                oc_hvec(g->eck, g->vi, i, j, l, h);
                if (op->form == DGPU_FORM_TABLE) {
                    const double *c = cfact + 2 * ((int64_t)(t - 1) * NTAB + istl[p]);
                    br = c[0]; bi = c[1];
                } else {
                    double tt[3];
                    for (int k = 0; k < 3; k++)
                        tt[k] = M3(cr->rten,k,0) * h[0] + M3(cr->rten,k,1) * h[1] + M3(cr->rten,k,2) * h[2];
                    double q2 = (h[0] * tt[0] + h[1] * tt[1] + h[2] * tt[2]) / 4.0;
                    oc_cfact_at(cr, op, t, q2, &br, &bi);
                }
                double ar = tcsf[2 * p], ai = tcsf[2 * p + 1];
                double xr = ar * br - ai * bi, xi = ar * bi + ai * br;
                if (a > 0 && op->ldbw) {
                    double d = oc_dbw(cr, a, h);
                    xr *= d;
                    xi *= d;
                }
                tcsf[2 * p] = xr;
                tcsf[2 * p + 1] = xi;
            }
}

/* tcsf_form_discamb (fourier_form.f90:63-102): the sum of the atoms of type
 * t, symmetry slot k (0-based) and ADP type a times the caller's table at
 * nint(h), then times four_dbw(a) (1 without ldbw).  Returns 1 when a point
 * maps outside the table. */
static int oc_apply_discamb(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op, int t,
                            int k, int a, const int32_t fnum[3], double *tcsf)
{
    const dgpu_discamb *dc = op->discamb;
    const int32_t *num = g->inc, *mh = dc->maxhkl;
    const int64_t n0 = 2 * mh[0] + 1, n1 = 2 * mh[1] + 1, tsz = n0 * n1 * (2 * mh[2] + 1);
    int64_t m = k;
    for (int u = 1; u < t; u++) m += dc->nsymm[u - 1];
    const double *tab = dc->form_tsc + 2 * m * tsz;
    for (int32_t l = 0; l < fnum[2]; l++)
        for (int32_t j = 0; j < fnum[1]; j++)
            for (int32_t i = 0; i < fnum[0]; i++) {
                int64_t p = i + (int64_t)num[0] * (j + (int64_t)num[1] * l);
                double h[3];
                int64_t ii[3];
                oc_hvec(g->eck, g->vi, i, j, l, h);
                for (int c = 0; c < 3; c++) {
                    ii[c] = lround(h[c]);
                    if (ii[c] < -mh[c] || ii[c] > mh[c]) return 1;
                }
                const double *f = tab + 2 * ((ii[0] + mh[0]) + n0 * ((ii[1] + mh[1]) + n1 * (ii[2] + mh[2])));
                double ar = tcsf[2 * p], ai = tcsf[2 * p + 1];
                double xr = ar * f[0] - ai * f[1], xi = ar * f[1] + ai * f[0];
                if (op->ldbw) {
                    double d = oc_dbw(cr, a, h);
                    xr *= d;
                    xi *= d;
                }
                tcsf[2 * p] = xr;
                tcsf[2 * p + 1] = xi;
            }
    return 0;
}

/* One type's (or the lattice's) sum into tcsf (zeroed over num first). */
static void oc_strucf_mode(const dgpu_grid *g, const dgpu_opts *op, const double *xat,
                           const float *w, int64_t nxat, const int32_t lmn[6],
                           const double off[9], const int32_t fnum[3], const double *cex,
                           int nthreads, double *tcsf)
{
    const int32_t *num = g->inc;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    memset(tcsf, 0, sizeof(double) * 2 * np);
    if (op->phase == DGPU_PHASE_REF22)
        oc_strucf_ref(xat, w, nxat, g->vi, g->vi + 3, g->vi + 6, off, lmn, num, fnum, cex,
                      0, fnum[0], nthreads, tcsf);
    else
        oc_strucf_exact(xat, w, nxat, g->eck, g->vi, num, fnum, nthreads, tcsf);
}

/* Checks of the lot options, the lots command's own (fourier.f90:490-497)
 * plus the range of the caller's origins. */
static int oc_check_lots(const dgpu_crystal *cr, const dgpu_opts *op, const int32_t cs[3])
{
    int lots = oc_lots_on(op);
    if (op->ilots != 0 && op->ilots != DGPU_LOT_OFF && !lots) return DGPU_ERR_ARG;
    if (!lots && op->lperiod) return 0;
    for (int k = 0; k < 3; k++)
        if (op->ls_xyz[k] < 1 || op->ls_xyz[k] > cr->icc[k]) return DGPU_ERR_ARG;
    if (!lots) return 0;
    if (!op->lot_all) {
        if (op->nlots < 1 || !op->lot_origins) return DGPU_ERR_ARG;
        for (int64_t l = 0; l < op->nlots; l++)
            for (int k = 0; k < 3; k++)
                if (op->lot_origins[3 * l + k] < 1 || op->lot_origins[3 * l + k] > cs[k]) return DGPU_ERR_ARG;
    }
    return 0;
}

/* four_run for the independent atom model, fourier_sup.f90:11-323: lots
 * (LOT_OFF, box, ellipsoid) and isotropic or anisotropic ADPs. */
int oc_four_run(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op,
                double *csf, double *acsf_out, double *dsi, dgpu_info *info, int nthreads)
{
    const int32_t *num = g->inc;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    int32_t lmn[6], fnum[3], cs[3];
    double off[9];
    int rc, warn = 0;
    if (cr->natoms < 1) return DGPU_ERR_NO_ATOMS;
    if (cr->is_anis && (cr->nanis < 1 || !cr->ianis || !cr->anis_full)) return DGPU_ERR_ARG;
    if (op->discamb) {
        if (!cr->isym || !op->discamb->nsymm || !op->discamb->isymm || !op->discamb->form_tsc) return DGPU_ERR_ARG;
        if (op->fave != 0.0) return DGPU_ERR_UNSUPPORTED;   /* four_aver would read disc_list(0) */
        if (op->ldbw && (cr->nanis < 1 || !cr->ianis || !cr->anis_full)) return DGPU_ERR_ARG;
    }
    oc_csize(cr, op, cs);
    rc = oc_check_lots(cr, op, cs);
    if (rc) return rc;
    const int lots = oc_lots_on(op);
    const int64_t nlots = !lots ? 1 : op->lot_all ? (int64_t)cs[0] * cs[1] * cs[2] : op->nlots;

    memset(csf, 0, sizeof(double) * 2 * np);
    memset(dsi, 0, sizeof(double) * np);
    double *acsf = (double *)calloc(2 * np, sizeof(double));
    double *tcsf = (double *)malloc(sizeof(double) * 2 * np);
    int32_t *istl = (int32_t *)malloc(sizeof(int32_t) * np);
    double *cfact = (double *)malloc(sizeof(double) * 2 * NTAB * (cr->nscat > 0 ? cr->nscat : 1));
    double *cex = (double *)malloc(sizeof(double) * 2 * DGPU_I2PI);
    double *xat = (double *)malloc(sizeof(double) * 3 * cr->natoms);
    float *w = (float *)malloc(sizeof(float) * cr->natoms);
    int32_t *alist = (int32_t *)malloc(sizeof(int32_t) * (cr->ianis ? cr->natoms : 1));
    int64_t pairs = 0;

    rc = oc_fourier_lmn(g->eck, g->vi, g->inc, lmn, off);
    if (rc) goto done;
    oc_cexpt(cex);
    rc = oc_stltab(g->eck, g->vi, num, cr->rten, istl);
    if (rc && op->form == DGPU_FORM_TABLE) goto done;
    rc = 0;
    oc_formtab(cr, op, cfact);
    int idim = oc_test_friedel(g, op, fnum);

    /* four_aver, fourier_sup.f90:1194-1357: cells drawn over csize */
    int32_t ncell = 0;
    if (op->fave != 0.0) {
        for (int t = 1; t <= cr->nscat; t++) {
            int64_t nx = 0;
            for (int pass = 0; pass < 2; pass++) {
                int64_t m = 0;
                double *xa = pass ? xat : NULL;
                for (int32_t ii = 0; ii < cs[0]; ii++)
                    for (int32_t jj = 0; jj < cs[1]; jj++)
                        for (int32_t kk = 0; kk < cs[2]; kk++) {
                            int64_t s = ii + (int64_t)cs[0] * (jj + (int64_t)cs[1] * kk);
                            int sel = op->fave >= 1.0 ? 1 : (op->aver_cells ? op->aver_cells[s] != 0 : 0);
                            if (!sel) continue;
                            if (pass) ncell++;
                            int32_t icell[3] = {ii, jj, kk};
                            int64_t c = ii + (int64_t)cr->icc[0] * (jj + (int64_t)cr->icc[1] * kk);
                            for (int32_t is = 0; is < cr->ncatoms; is++) {
                                int64_t ia = c * cr->ncatoms + is;              /* celltoindex */
                                if (ia >= cr->natoms || cr->iscat[ia] != t) continue;
                                if (xa) {
                                    for (int k = 0; k < 3; k++)
                                        xa[k * nx + m] = cr->pos[3 * ia + k] - (double)icell[k] - cr->dim0[k];
                                    w[m] = cr->atom_occ ? cr->atom_occ[ia] : 1.0f;
                                }
                                m++;
                            }
                        }
                nx = m;
            }
            oc_strucf_mode(g, op, xat, cr->atom_occ ? w : NULL, nx, lmn, off, fnum, cex, nthreads, tcsf);
            oc_apply_form(cr, g, op, t, 0, cfact, istl, fnum, tcsf);
            for (int64_t p = 0; p < 2 * np; p++) acsf[p] += tcsf[p];
        }
        ncell = ncell / cr->nscat;
        /* four_getav (fourier_sup.f90:2440-2510): the lattice of the whole
         * crystal or of one lot, summed on the full num */
        int64_t nl = 0;
        double *xl = (double *)malloc(sizeof(double) * 3 * ((int64_t)cr->icc[0] * cr->icc[1] * cr->icc[2] + 1));
        int64_t cap = (int64_t)cr->icc[0] * cr->icc[1] * cr->icc[2];
        double *xs = (double *)malloc(sizeof(double) * 3 * (cap > 0 ? cap : 1));
        if (!lots) {
            for (int32_t ii = 0; ii < cr->icc[0]; ii++)
                for (int32_t jj = 0; jj < cr->icc[1]; jj++)
                    for (int32_t kk = 0; kk < cr->icc[2]; kk++) {
                        xs[3 * nl] = (double)ii + cr->dim0[0];
                        xs[3 * nl + 1] = (double)jj + cr->dim0[1];
                        xs[3 * nl + 2] = (double)kk + cr->dim0[2];
                        nl++;
                    }
        } else {
            for (int32_t kk = 0; kk < op->ls_xyz[2]; kk++)
                for (int32_t jj = 0; jj < op->ls_xyz[1]; jj++)
                    for (int32_t ii = 0; ii < op->ls_xyz[0]; ii++) {
                        if (!oc_in_lot(op, ii, jj, kk)) continue;
                        xs[3 * nl] = ii;
                        xs[3 * nl + 1] = jj;
                        xs[3 * nl + 2] = kk;
                        nl++;
                    }
        }
        for (int64_t m = 0; m < nl; m++)
            for (int k = 0; k < 3; k++) xl[k * nl + m] = xs[3 * m + k];
        oc_strucf_mode(g, op, xl, NULL, nl, lmn, off, num, cex, nthreads, tcsf);
        free(xl);
        free(xs);
        double norm = 0.0;
        if (ncell > 0) norm = 1.0 / ncell; else warn = DGPU_WARN_NO_CELL;
        for (int64_t p = 0; p < np; p++) {
            double ar = acsf[2 * p], ai = acsf[2 * p + 1];
            double br = tcsf[2 * p], bi = tcsf[2 * p + 1];
            double cr_ = ar * br - ai * bi, ci = ar * bi + ai * br;
            acsf[2 * p] = cr_ * norm;
            acsf[2 * p + 1] = ci * norm;
        }
    }

    /* loop over lots and atom types (fourier_sup.f90:136-257) */
    int32_t lcell = 0;
    for (int64_t lot = 0; lot < nlots; lot++) {
        int32_t lbeg[3] = {1, 1, 1};
        if (lots && op->lot_all) {
            int64_t ii = lot;
            lbeg[2] = (int32_t)(ii / ((int64_t)cs[0] * cs[1])) + 1;
            ii -= (int64_t)(lbeg[2] - 1) * cs[0] * cs[1];
            lbeg[1] = (int32_t)(ii / cs[0]) + 1;
            ii -= (int64_t)(lbeg[1] - 1) * cs[0];
            lbeg[0] = (int32_t)(ii % cs[0]) + 1;
        } else if (lots) {
            for (int k = 0; k < 3; k++) lbeg[k] = op->lot_origins[3 * lot + k];
        }
        memset(csf, 0, sizeof(double) * 2 * np);
        /* DISCAMB: (type, symmetry, ADP) groups (fourier_sup.f90:166-193) */
        const dgpu_discamb *dc = op->discamb;
        const int by_adp = cr->is_anis || (dc && cr->ianis && cr->nanis >= 1);
        for (int t = 1, ks = 0; t <= cr->nscat; ks += dc ? dc->nsymm[t - 1] : 0, t++) {
            int na = 1;
            if (by_adp) na = oc_anis_list(cr, t, alist);
            const int nk = dc ? dc->nsymm[t - 1] : 1;
            for (int k = 0; k < nk; k++)
            for (int j = 0; j < na; j++) {
                int a = by_adp ? alist[j] : 0;
                int y = dc ? dc->isymm[ks + k] : -1;
                int64_t nx = oc_getatm_lot(cr, op, t, a, y, lbeg, NULL, NULL, 0, &lcell, NULL);
                if (nx <= 0) continue;
                oc_getatm_lot(cr, op, t, a, y, lbeg, xat, w, nx, &lcell, NULL);
                pairs += nx * np;
                oc_strucf_mode(g, op, xat, cr->atom_occ ? w : NULL, nx, lmn, off, fnum, cex, nthreads, tcsf);
                if (dc) {
                    if (oc_apply_discamb(cr, g, op, t, k, a > 0 ? a : 1, fnum, tcsf)) { rc = DGPU_ERR_ARG; goto done; }
                } else {
                    oc_apply_form(cr, g, op, t, a, cfact, istl, fnum, tcsf);
                }
                for (int64_t p = 0; p < 2 * np; p++) csf[p] += tcsf[p];
                if (op->cancel && *op->cancel) { rc = DGPU_ERR_CANCELLED; goto done; }
            }
        }
        for (int64_t p = 0; p < np; p++) {
            csf[2 * p] -= acsf[2 * p];
            csf[2 * p + 1] -= acsf[2 * p + 1];
            dsi[p] = dsi[p] + (csf[2 * p] * csf[2 * p] + csf[2 * p + 1] * csf[2 * p + 1]);
        }
        if (idim) oc_apply_friedel(num, fnum, acsf, csf, dsi);
    }
    if (nlots != 1) {
        /* fourier_sup.f90:273-277 */
        double dnorm = (double)((int64_t)cr->icc[0] * cr->icc[1] * cr->icc[2]) / (double)(lcell * nlots);
        for (int64_t p = 0; p < np; p++) dsi[p] = dnorm * dsi[p];
    }
    {
        double sq = sqrt(op->diff_scale);
        for (int64_t p = 0; p < 2 * np; p++) csf[p] *= sq;
        for (int64_t p = 0; p < np; p++) dsi[p] *= op->diff_scale;
    }
    if (info) {
        memset(info, 0, sizeof(*info));
        for (int k = 0; k < 3; k++) info->fnum[k] = fnum[k];
        info->friedel_dim = idim;
        for (int k = 0; k < 6; k++) info->lmn[k] = lmn[k];
        for (int k = 0; k < 9; k++) info->off_shift[k] = off[k];
        info->ncell = ncell;
        info->pairs = pairs;
        oc_qinfo(g, dsi, info->res);
    }
    if (acsf_out) memcpy(acsf_out, acsf, sizeof(double) * 2 * np);
    rc = warn;
done:
    free(acsf); free(tcsf); free(istl); free(cfact); free(cex); free(xat); free(w); free(alist);
    return rc;
}
/* ---------------------------------------------------------------------- */
/* chi^2 = sum_h wt(h) (I(h) - It(h))^2 and its gradient, exact FP64, full
 * grid, no Friedel reduction.  I = diff_scale |F|^2 with
 * F = sum_j cf_t(j)(h) D_a(j)(h) w_j exp(2 pi i h.r_j) - A(h), D the
 * anisotropic Debye-Waller term of atom j's ADP type (1 for an isotropic
 * crystal).  A = 0 unless fave > 0; then (four_aver, fourier_sup.f90:
 * 1194-1357, with the lattice of four_getav :2440-2510) the atoms of the
 * cells selected over csize are moved into one cell,
 *   A(h) = L(h)/ncell sum_{j selected} cf_t(j)(h) w_j exp(2 pi i h.(r_j - cell_j - dim0)),
 *   L(h) = sum over all icc cells of exp(2 pi i h.(cell + dim0)),
 * and every selected atom gets a second term with Q^A = -L/ncell Q.        */
/* The same with lots (fourier_sup.f90:136-277): I = ds dnorm sum_L |F_L|^2,
 * F_L the sum over lot L's atoms at their positions shifted by the lot
 * origin (oc_getatm_lot) less <F>, dnorm = icc1 icc2 icc3 / (ncell nlots)
 * when nlots != 1.  <F> (fave > 0) takes the lot's lattice: the cells of the
 * lot shape at the origin (four_getav).  An atom's gradient adds its terms
 * over every lot that holds it; a folded atom of <F> gets
 * Q^A = -L/ncell 2 ds dnorm G conj(sum_L F_L) cf.                          */
static int oc_chi2_grad_lots(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op,
                             const double *it, const double *wt, double *chi2, double *grad_pos,
                             double *grad_occ, int nthreads)
{
    const double zpi = 6.283185307179586476925286766559;
    const int32_t *num = g->inc;
    const int64_t np = (int64_t)num[0] * num[1] * num[2];
    const int ns = cr->nscat, na = (int)cr->natoms;
    const int anis = cr->is_anis && op->ldbw;
    int32_t cs[3];
    oc_csize(cr, op, cs);
    int rc = oc_check_lots(cr, op, cs);
    if (rc) return rc;
    const int64_t nlots = op->lot_all ? (int64_t)cs[0] * cs[1] * cs[2] : op->nlots;
    double *cf = (double *)malloc(sizeof(double) * 2 * np * ns);
    double *H = (double *)malloc(sizeof(double) * 3 * np);
    double *D = (double *)malloc(sizeof(double) * np * (anis ? cr->nanis : 1));
    int32_t *istl = (int32_t *)malloc(sizeof(int32_t) * np);
    double *cfact = (double *)malloc(sizeof(double) * 2 * NTAB * ns);
    oc_stltab(g->eck, g->vi, num, cr->rten, istl);
    oc_formtab(cr, op, cfact);
    for (int64_t p = 0; p < np; p++) {
        int32_t i = (int32_t)(p % num[0]), j = (int32_t)((p / num[0]) % num[1]), l = (int32_t)(p / ((int64_t)num[0] * num[1]));
        double h[3], tt[3];
        oc_hvec(g->eck, g->vi, i, j, l, h);
        for (int k = 0; k < 3; k++) H[3 * p + k] = h[k];
        if (anis)
            for (int a = 1; a <= cr->nanis; a++) D[(int64_t)(a - 1) * np + p] = oc_dbw(cr, a, h);
        for (int a = 0; a < 3; a++)
            tt[a] = M3(cr->rten,a,0) * h[0] + M3(cr->rten,a,1) * h[1] + M3(cr->rten,a,2) * h[2];
        double q2 = (h[0] * tt[0] + h[1] * tt[1] + h[2] * tt[2]) / 4.0;
        for (int t = 1; t <= ns; t++) {
            double br, bi;
            if (op->form == DGPU_FORM_TABLE) {
                const double *c = cfact + 2 * ((int64_t)(t - 1) * NTAB + istl[p]);
                br = c[0]; bi = c[1];
            } else {
                oc_cfact_at(cr, op, t, q2, &br, &bi);
            }
            cf[2 * ((int64_t)(t - 1) * np + p)] = br;
            cf[2 * ((int64_t)(t - 1) * np + p) + 1] = bi;
        }
    }
    /* the lots' atoms: positions, types, ADP types, weights, sources */
    int64_t *lstart = (int64_t *)calloc(nlots + 1, sizeof(int64_t));
    int64_t cap = 0;
    int32_t lcell = 0;
    for (int pass = 0; pass < 2; pass++) {
        int64_t tot = 0;
        for (int64_t L = 0; L < nlots; L++) {
            int32_t lbeg[3];
            if (op->lot_all) {
                int64_t ii = L;
                lbeg[2] = (int32_t)(ii / ((int64_t)cs[0] * cs[1])) + 1;
                ii -= (int64_t)(lbeg[2] - 1) * cs[0] * cs[1];
                lbeg[1] = (int32_t)(ii / cs[0]) + 1;
                lbeg[0] = (int32_t)(ii % cs[0]) + 1;
            } else {
                for (int k = 0; k < 3; k++) lbeg[k] = op->lot_origins[3 * L + k];
            }
            if (pass == 0) lstart[L] = tot;
            for (int t = 1; t <= ns; t++) {
                int64_t nx = oc_getatm_lot(cr, op, t, 0, -1, lbeg, NULL, NULL, 0, &lcell, NULL);
                tot += nx;
            }
        }
        if (pass == 0) { lstart[nlots] = tot; cap = tot; }
    }
    double *lx = (double *)malloc(sizeof(double) * 3 * (cap > 0 ? cap : 1));
    float *lw = (float *)malloc(sizeof(float) * (cap > 0 ? cap : 1));
    int64_t *lsrc = (int64_t *)malloc(sizeof(int64_t) * (cap > 0 ? cap : 1));
    int32_t *lt = (int32_t *)malloc(sizeof(int32_t) * (cap > 0 ? cap : 1));
    {
        double *xt = (double *)malloc(sizeof(double) * 3 * (na > 0 ? na : 1));
        float *wt1 = (float *)malloc(sizeof(float) * (na > 0 ? na : 1));
        int64_t *st1 = (int64_t *)malloc(sizeof(int64_t) * (na > 0 ? na : 1));
        for (int64_t L = 0; L < nlots; L++) {
            int32_t lbeg[3];
            if (op->lot_all) {
                int64_t ii = L;
                lbeg[2] = (int32_t)(ii / ((int64_t)cs[0] * cs[1])) + 1;
                ii -= (int64_t)(lbeg[2] - 1) * cs[0] * cs[1];
                lbeg[1] = (int32_t)(ii / cs[0]) + 1;
                lbeg[0] = (int32_t)(ii % cs[0]) + 1;
            } else {
                for (int k = 0; k < 3; k++) lbeg[k] = op->lot_origins[3 * L + k];
            }
            int64_t m = lstart[L];
            for (int t = 1; t <= ns; t++) {
                int64_t nx = oc_getatm_lot(cr, op, t, 0, -1, lbeg, NULL, NULL, 0, &lcell, NULL);
                oc_getatm_lot(cr, op, t, 0, -1, lbeg, xt, wt1, nx, &lcell, st1);
                for (int64_t q = 0; q < nx; q++, m++) {
                    for (int k = 0; k < 3; k++) lx[3 * m + k] = xt[k * nx + q];
                    lw[m] = cr->atom_occ ? wt1[q] : 1.0f;
                    lsrc[m] = st1[q];
                    lt[m] = t;
                }
            }
        }
        free(xt); free(wt1); free(st1);
    }
    /* <F>: the folded atoms of the cells selected over csize, the lot lattice */
    unsigned char *insel = (unsigned char *)calloc(na > 0 ? na : 1, 1);
    double *xf = (double *)malloc(sizeof(double) * 3 * (na > 0 ? na : 1));
    int32_t ncell = 0;
    if (op->fave > 0.0)
        for (int32_t kk = 0; kk < cs[2]; kk++)
            for (int32_t jj = 0; jj < cs[1]; jj++)
                for (int32_t ii = 0; ii < cs[0]; ii++) {
                    int64_t sidx = ii + (int64_t)cs[0] * (jj + (int64_t)cs[1] * kk);
                    if (!(op->fave >= 1.0 || (op->aver_cells && op->aver_cells[sidx] != 0))) continue;
                    ncell++;
                    int32_t icell[3] = {ii, jj, kk};
                    int64_t c = ii + (int64_t)cr->icc[0] * (jj + (int64_t)cr->icc[1] * kk);
                    for (int32_t is = 0; is < cr->ncatoms; is++) {
                        int64_t ia = c * cr->ncatoms + is;
                        if (ia >= na) continue;
                        insel[ia] = 1;
                        for (int k = 0; k < 3; k++) xf[3 * ia + k] = cr->pos[3 * ia + k] - (double)icell[k] - cr->dim0[k];
                    }
                }
    const double anorm = ncell > 0 ? 1.0 / ncell : 0.0;
    double *A = (double *)calloc(2 * np, sizeof(double));
    double *Lh = (double *)calloc(2 * np, sizeof(double));
    if (ncell > 0) {
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
        for (int64_t p = 0; p < np; p++) {
            double lr = 0, li = 0, ar = 0, ai = 0;
            for (int32_t kk = 0; kk < op->ls_xyz[2]; kk++)
                for (int32_t jj = 0; jj < op->ls_xyz[1]; jj++)
                    for (int32_t ii = 0; ii < op->ls_xyz[0]; ii++) {
                        if (!oc_in_lot(op, ii, jj, kk)) continue;
                        double ph = oc_frac_dot(H + 3 * p, ii, jj, kk);
                        lr += cos(zpi * ph);
                        li += sin(zpi * ph);
                    }
            for (int64_t a = 0; a < na; a++) {
                int t = cr->iscat[a];
                if (!insel[a] || t < 1 || t > ns) continue;
                double ph = oc_frac_dot(H + 3 * p, xf[3 * a], xf[3 * a + 1], xf[3 * a + 2]);
                double wa = cr->atom_occ ? (double)cr->atom_occ[a] : 1.0;
                double c = cos(zpi * ph) * wa, sn = sin(zpi * ph) * wa;
                double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
                ar += br * c - bi * sn;
                ai += br * sn + bi * c;
            }
            Lh[2 * p] = lr;
            Lh[2 * p + 1] = li;
            A[2 * p] = anorm * (lr * ar - li * ai);
            A[2 * p + 1] = anorm * (lr * ai + li * ar);
        }
    }
    /* F_L at every point */
    double *F = (double *)malloc(sizeof(double) * 2 * np * (nlots > 0 ? nlots : 1));
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t p = 0; p < np; p++)
        for (int64_t L = 0; L < nlots; L++) {
            double fr = -A[2 * p], fi = -A[2 * p + 1];
            for (int64_t m = lstart[L]; m < lstart[L + 1]; m++) {
                int t = lt[m];
                double ph = oc_frac_dot(H + 3 * p, lx[3 * m], lx[3 * m + 1], lx[3 * m + 2]);
                double wa = (double)lw[m];
                if (anis) wa *= D[(int64_t)(cr->ianis[lsrc[m]] - 1) * np + p];
                double c = cos(zpi * ph) * wa, sn = sin(zpi * ph) * wa;
                double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
                fr += br * c - bi * sn;
                fi += br * sn + bi * c;
            }
            F[2 * (L * np + p)] = fr;
            F[2 * (L * np + p) + 1] = fi;
        }
    const double dnorm = nlots != 1 ? (double)((int64_t)cr->icc[0] * cr->icc[1] * cr->icc[2]) / (double)(lcell * nlots)
                                     : 1.0;
    double *G = (double *)malloc(sizeof(double) * np);
    double x2 = 0;
    for (int64_t p = 0; p < np; p++) {
        double s = 0;
        for (int64_t L = 0; L < nlots; L++) s += F[2 * (L * np + p)] * F[2 * (L * np + p)] + F[2 * (L * np + p) + 1] * F[2 * (L * np + p) + 1];
        double I = op->diff_scale * dnorm * s;
        double d = I - it[p];
        double wp = wt ? wt[p] : 1.0;
        x2 += wp * d * d;
        G[p] = 2.0 * wp * d * 2.0 * op->diff_scale * dnorm;    /* 2 ds dnorm dchi2/dI */
    }
    if (chi2) *chi2 = x2;
    if (grad_pos) memset(grad_pos, 0, sizeof(double) * 3 * na);
    if (grad_occ) memset(grad_occ, 0, sizeof(double) * na);
    /* per lot atom: T = sum_p G conj(F_L) cf D e^{2 pi i h.x} */
    for (int64_t L = 0; L < nlots; L++)
        for (int64_t m = lstart[L]; m < lstart[L + 1]; m++) {
            int t = lt[m];
            int64_t a = lsrc[m];
            double go = 0, gx[3] = {0, 0, 0};
            for (int64_t p = 0; p < np; p++) {
                double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
                if (anis) {
                    double d = D[(int64_t)(cr->ianis[a] - 1) * np + p];
                    br *= d;
                    bi *= d;
                }
                double fr = F[2 * (L * np + p)], fi = -F[2 * (L * np + p) + 1];
                double qr = G[p] * (fr * br - fi * bi), qi = G[p] * (fr * bi + fi * br);
                double ph = oc_frac_dot(H + 3 * p, lx[3 * m], lx[3 * m + 1], lx[3 * m + 2]);
                double c = cos(zpi * ph), sn = sin(zpi * ph);
                double zr = qr * c - qi * sn, zi = qr * sn + qi * c;
                go += zr;
                for (int k = 0; k < 3; k++) gx[k] += H[3 * p + k] * zi;
            }
            double wa = (double)lw[m];
            if (grad_occ) grad_occ[a] += go;
            if (grad_pos) for (int k = 0; k < 3; k++) grad_pos[3 * a + k] += -zpi * wa * gx[k];
        }
    /* folded atoms of <F> */
    if (ncell > 0)
        for (int64_t a = 0; a < na; a++) {
            int t = cr->iscat[a];
            if (!insel[a] || t < 1 || t > ns) continue;
            double go = 0, gx[3] = {0, 0, 0};
            for (int64_t p = 0; p < np; p++) {
                double sr = 0, si = 0;
                for (int64_t L = 0; L < nlots; L++) { sr += F[2 * (L * np + p)]; si += F[2 * (L * np + p) + 1]; }
                double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
                /* Q^A = -anorm L G conj(sum F) cf */
                double ur = sr * br + si * bi, ui = sr * bi - si * br;          /* conj(sum F) cf */
                double lr = -anorm * Lh[2 * p], li = -anorm * Lh[2 * p + 1];
                double qr = G[p] * (lr * ur - li * ui), qi = G[p] * (lr * ui + li * ur);
                double ph = oc_frac_dot(H + 3 * p, xf[3 * a], xf[3 * a + 1], xf[3 * a + 2]);
                double c = cos(zpi * ph), sn = sin(zpi * ph);
                double zr = qr * c - qi * sn, zi = qr * sn + qi * c;
                go += zr;
                for (int k = 0; k < 3; k++) gx[k] += H[3 * p + k] * zi;
            }
            double wa = cr->atom_occ ? (double)cr->atom_occ[a] : 1.0;
            if (grad_occ) grad_occ[a] += go;
            if (grad_pos) for (int k = 0; k < 3; k++) grad_pos[3 * a + k] += -zpi * wa * gx[k];
        }
    free(cf); free(H); free(D); free(istl); free(cfact); free(lstart); free(lx); free(lw); free(lsrc); free(lt);
    free(insel); free(xf); free(A); free(Lh); free(F); free(G);
    return DGPU_OK;
}

int oc_chi2_grad(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op,
                 const double *it, const double *wt, double *chi2, double *grad_pos,
                 double *grad_occ, int nthreads)
{
    if (oc_lots_on(op)) return oc_chi2_grad_lots(cr, g, op, it, wt, chi2, grad_pos, grad_occ, nthreads);
    const double zpi = 6.283185307179586476925286766559;
    const int32_t *num = g->inc;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    int ns = cr->nscat;
    double *cf = (double *)malloc(sizeof(double) * 2 * np * (ns > 0 ? ns : 1));
    double *F = (double *)calloc(2 * np, sizeof(double));
    double *Q = (double *)malloc(sizeof(double) * 2 * np * (ns > 0 ? ns : 1));
    double *H = (double *)malloc(sizeof(double) * 3 * np);
    int32_t *istl = (int32_t *)malloc(sizeof(int32_t) * np);
    double *cfact = (double *)malloc(sizeof(double) * 2 * NTAB * (ns > 0 ? ns : 1));
    const int anis = cr->is_anis && op->ldbw;
    double *D = (double *)malloc(sizeof(double) * np * (anis ? cr->nanis : 1));
    (void)nthreads;
    /* <F>: selected atoms, their folded positions, the lattice sum */
    const int64_t na = cr->natoms;
    unsigned char *insel = (unsigned char *)calloc(na > 0 ? na : 1, 1);
    double *xf = (double *)malloc(sizeof(double) * 3 * (na > 0 ? na : 1));
    double *Lh = (double *)calloc(2 * np, sizeof(double));
    int32_t ncell = 0;
    if (op->fave > 0.0) {
        int32_t cs[3];
        oc_csize(cr, op, cs);
        for (int32_t kk = 0; kk < cs[2]; kk++)
            for (int32_t jj = 0; jj < cs[1]; jj++)
                for (int32_t ii = 0; ii < cs[0]; ii++) {
                    int64_t s = ii + (int64_t)cs[0] * (jj + (int64_t)cs[1] * kk);
                    if (!(op->fave >= 1.0 || (op->aver_cells && op->aver_cells[s] != 0))) continue;
                    ncell++;
                    int32_t icell[3] = {ii, jj, kk};
                    int64_t c = ii + (int64_t)cr->icc[0] * (jj + (int64_t)cr->icc[1] * kk);
                    for (int32_t is = 0; is < cr->ncatoms; is++) {
                        int64_t ia = c * cr->ncatoms + is;
                        if (ia >= na) continue;
                        insel[ia] = 1;
                        for (int k = 0; k < 3; k++)
                            xf[3 * ia + k] = cr->pos[3 * ia + k] - (double)icell[k] - cr->dim0[k];
                    }
                }
    }
    const double anorm = ncell > 0 ? 1.0 / ncell : 0.0;
    oc_stltab(g->eck, g->vi, num, cr->rten, istl);
    oc_formtab(cr, op, cfact);
    for (int32_t l = 0; l < num[2]; l++)
        for (int32_t j = 0; j < num[1]; j++)
            for (int32_t i = 0; i < num[0]; i++) {
                int64_t p = i + (int64_t)num[0] * (j + (int64_t)num[1] * l);
                double h[3], tt[3];
                oc_hvec(g->eck, g->vi, i, j, l, h);
                for (int k = 0; k < 3; k++) H[3 * p + k] = h[k];
                if (anis)
                    for (int a = 1; a <= cr->nanis; a++) D[(int64_t)(a - 1) * np + p] = oc_dbw(cr, a, h);
                for (int a = 0; a < 3; a++)
                    tt[a] = M3(cr->rten,a,0) * h[0] + M3(cr->rten,a,1) * h[1] + M3(cr->rten,a,2) * h[2];
                double q2 = (h[0] * tt[0] + h[1] * tt[1] + h[2] * tt[2]) / 4.0;
                for (int t = 1; t <= ns; t++) {
                    double br, bi;
                    if (op->form == DGPU_FORM_TABLE) {
                        const double *c = cfact + 2 * ((int64_t)(t - 1) * NTAB + istl[p]);
                        br = c[0]; bi = c[1];
                    } else {
                        oc_cfact_at(cr, op, t, q2, &br, &bi);
                    }
                    cf[2 * ((int64_t)(t - 1) * np + p)] = br;
                    cf[2 * ((int64_t)(t - 1) * np + p) + 1] = bi;
                }
            }
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t p = 0; p < np; p++) {
        double fr = 0, fi = 0;
        for (int64_t a = 0; a < cr->natoms; a++) {
            int t = cr->iscat[a];
            if (t < 1 || t > ns) continue;
            double ph = oc_frac_dot(H + 3 * p, cr->pos[3 * a], cr->pos[3 * a + 1], cr->pos[3 * a + 2]);
            double wa = cr->atom_occ ? (double)cr->atom_occ[a] : 1.0;
            if (anis) wa *= D[(int64_t)(cr->ianis[a] - 1) * np + p];
            double c = cos(zpi * ph) * wa, s = sin(zpi * ph) * wa;
            double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
            fr += br * c - bi * s;
            fi += br * s + bi * c;
        }
        if (ncell > 0) {
            double lr = 0, li = 0, ar = 0, ai = 0;
            for (int32_t kk = 0; kk < cr->icc[2]; kk++)
                for (int32_t jj = 0; jj < cr->icc[1]; jj++)
                    for (int32_t ii = 0; ii < cr->icc[0]; ii++) {
                        double ph = oc_frac_dot(H + 3 * p, ii + cr->dim0[0], jj + cr->dim0[1], kk + cr->dim0[2]);
                        lr += cos(zpi * ph);
                        li += sin(zpi * ph);
                    }
            for (int64_t a = 0; a < na; a++) {
                int t = cr->iscat[a];
                if (!insel[a] || t < 1 || t > ns) continue;
                double ph = oc_frac_dot(H + 3 * p, xf[3 * a], xf[3 * a + 1], xf[3 * a + 2]);
                double wa = cr->atom_occ ? (double)cr->atom_occ[a] : 1.0;
                double c = cos(zpi * ph) * wa, s = sin(zpi * ph) * wa;
                double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
                ar += br * c - bi * s;
                ai += br * s + bi * c;
            }
            Lh[2 * p] = lr;
            Lh[2 * p + 1] = li;
            fr -= anorm * (lr * ar - li * ai);
            fi -= anorm * (lr * ai + li * ar);
        }
        F[2 * p] = fr; F[2 * p + 1] = fi;
    }
    double x2 = 0;
    for (int64_t p = 0; p < np; p++) {
        double I = op->diff_scale * (F[2 * p] * F[2 * p] + F[2 * p + 1] * F[2 * p + 1]);
        double d = I - it[p];
        double wp = wt ? wt[p] : 1.0;
        x2 += wp * d * d;
        double gsc = 2.0 * wp * d * op->diff_scale;       /* d chi2 / d|F|^2 */
        for (int t = 1; t <= ns; t++) {
            /* Q_t = 2 g conj(F) cf_t */
            double br = cf[2 * ((int64_t)(t - 1) * np + p)], bi = cf[2 * ((int64_t)(t - 1) * np + p) + 1];
            double fr = F[2 * p], fi = -F[2 * p + 1];
            Q[2 * ((int64_t)(t - 1) * np + p)] = 2.0 * gsc * (fr * br - fi * bi);
            Q[2 * ((int64_t)(t - 1) * np + p) + 1] = 2.0 * gsc * (fr * bi + fi * br);
        }
    }
    if (chi2) *chi2 = x2;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t a = 0; a < cr->natoms; a++) {
        int t = cr->iscat[a];
        double go = 0, gx[3] = {0, 0, 0};
        if (t >= 1 && t <= ns) {
            for (int64_t p = 0; p < np; p++) {
                double ph = oc_frac_dot(H + 3 * p, cr->pos[3 * a], cr->pos[3 * a + 1], cr->pos[3 * a + 2]);
                double c = cos(zpi * ph), s = sin(zpi * ph);
                double qr = Q[2 * ((int64_t)(t - 1) * np + p)], qi = Q[2 * ((int64_t)(t - 1) * np + p) + 1];
                if (anis) {
                    double d = D[(int64_t)(cr->ianis[a] - 1) * np + p];
                    qr *= d;
                    qi *= d;
                }
                double zr = qr * c - qi * s, zi = qr * s + qi * c;
                go += zr;
                for (int k = 0; k < 3; k++) gx[k] += H[3 * p + k] * zi;
            }
        }
        if (t >= 1 && t <= ns && insel[a]) {
            /* the atom's folded copy in <F>: Q^A = -L/ncell Q, no ADP term */
            for (int64_t p = 0; p < np; p++) {
                double ph = oc_frac_dot(H + 3 * p, xf[3 * a], xf[3 * a + 1], xf[3 * a + 2]);
                double c = cos(zpi * ph), s = sin(zpi * ph);
                double qr = Q[2 * ((int64_t)(t - 1) * np + p)], qi = Q[2 * ((int64_t)(t - 1) * np + p) + 1];
                double lr = -anorm * Lh[2 * p], li = -anorm * Lh[2 * p + 1];
                double ur = lr * qr - li * qi, ui = lr * qi + li * qr;
                double zr = ur * c - ui * s, zi = ur * s + ui * c;
                go += zr;
                for (int k = 0; k < 3; k++) gx[k] += H[3 * p + k] * zi;
            }
        }
        double wa = cr->atom_occ ? (double)cr->atom_occ[a] : 1.0;
        if (grad_occ) grad_occ[a] = go;
        if (grad_pos) for (int k = 0; k < 3; k++) grad_pos[3 * a + k] = -zpi * wa * gx[k];
    }
    free(cf); free(F); free(Q); free(H); free(istl); free(cfact); free(D);
    free(insel); free(xf); free(Lh);
    return DGPU_OK;
}

/* Time the REF22 type sums of four_run on rows [row_lo,row_hi) of the
 * abscissa (the reference's OMP loop is uniform per row), all types.
 * Returns seconds; *pairs_out = atoms x points covered.                   */
double oc_time_ref_rows(const dgpu_crystal *cr, const dgpu_grid *g, int32_t row_lo,
                        int32_t row_hi, int nthreads, int64_t *pairs_out)
{
    const int32_t *num = g->inc;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    int32_t lmn[6], fnum[3] = {num[0], num[1], num[2]};
    double off[9];
    oc_fourier_lmn(g->eck, g->vi, g->inc, lmn, off);
    double *cex = (double *)malloc(sizeof(double) * 2 * DGPU_I2PI);
    oc_cexpt(cex);
    double *tcsf = (double *)calloc(2 * np, sizeof(double));
    double *xat = (double *)malloc(sizeof(double) * 3 * cr->natoms);
    int64_t pairs = 0;
    double t0 = 0, t1 = 0;
#ifdef _OPENMP
    t0 = omp_get_wtime();
#endif
    for (int t = 1; t <= cr->nscat; t++) {
        dgpu_opts whole;
        memset(&whole, 0, sizeof(whole));
        whole.ilots = DGPU_LOT_OFF;
        int32_t nc;
        int64_t nx = oc_getatm_lot(cr, &whole, t, 0, -1, NULL, NULL, NULL, 0, &nc, NULL);
        if (nx <= 0) continue;
        oc_getatm_lot(cr, &whole, t, 0, -1, NULL, xat, NULL, nx, &nc, NULL);
        oc_strucf_ref(xat, NULL, nx, g->vi, g->vi + 3, g->vi + 6, off, lmn, num, fnum, cex,
                      row_lo, row_hi, nthreads, tcsf);
        pairs += nx * (int64_t)(row_hi - row_lo) * num[1] * num[2];
    }
#ifdef _OPENMP
    t1 = omp_get_wtime();
#endif
    free(cex); free(tcsf); free(xat);
    if (pairs_out) *pairs_out = pairs;
    return t1 - t0;
}

/* ---------------------------------------------------------------------- */
/* four_weight, fourier_sup.f90:1428-1643, with do_volume / do_bang /
 * do_blen (discus/prog/metric.f90:6-60, 576-605) in the reciprocal metric. */
static double oc_skal(const double *u, const double *v, const double *g)
{
    double s = 0;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) s += u[i] * M3(g, i, j) * v[j];
    return s;
}

static double oc_bang(const double *u, const double *w, const double *g)
{
    double xx = sqrt(oc_skal(u, u, g)), yy = sqrt(oc_skal(w, w, g)), xy = oc_skal(u, w, g);
    if (!(xx > 0 && yy > 0)) return 0.0;
    double arg = xy / (xx * yy);
    const float rad_sp = (float)(3.1415926535897932384626433832795028841971693993751 / 180.0);
    if (fabs(arg) < 1.0) return acos(arg) / (double)rad_sp;
    return arg >= 1.0 ? 0.0 : 180.0;
}

static double oc_volume(const double *u, const double *v, const double *w, const double *g)
{
    const double rad = 3.1415926535897932384626433832795028841971693993751 / 180.0;
    double l1 = sqrt(oc_skal(u, u, g)), l2 = sqrt(oc_skal(v, v, g)), l3 = sqrt(oc_skal(w, w, g));
    double c1 = cos(oc_bang(v, w, g) * rad), c2 = cos(oc_bang(u, w, g) * rad), c3 = cos(oc_bang(u, v, g) * rad);
    return l1 * l2 * l3 * sqrt(1.0 - c1 * c1 - c2 * c2 - c3 * c3 + 2.0 * c1 * c2 * c3);
}

int oc_four_weight(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op, const double *dsi,
                   double *dsi3d, double *scalef_out)
{
    const int32_t *num = g->inc;
    const double *uin = g->vi, *vin = g->vi + 3, *win = g->vi + 6;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    double scalef = 1.0;
    if (op->fave == 0.0) {
        int isdim = 3;
        for (int k = 0; k < 3; k++) if (num[k] == 1) isdim--;
        int32_t cs[3];
        oc_csize(cr, op, cs);
        int64_t nlots = !oc_lots_on(op) ? 1 : op->lot_all ? (int64_t)cs[0] * cs[1] * cs[2] : op->nlots;
        const int32_t *n = nlots == 1 ? cr->icc : op->ls_xyz;
        double B[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};     /* bases(3,3), column-major */
        int64_t ncells = 1;
        if (isdim == 1) {
            if (num[0] != 1) {
                for (int k = 0; k < 3; k++) B[k] = uin[k];
                if (B[0] != 0) { B[3 + 1] = 1; B[6 + 2] = 1; }
                else if (B[1] != 0) { B[3 + 2] = 1; B[6 + 0] = 1; }
                else if (B[2] != 0) { B[3 + 0] = 1; B[6 + 1] = 1; }
                ncells = n[0];
            } else if (num[1] == 1) {
                for (int k = 0; k < 3; k++) B[3 + k] = vin[k];
                if (B[3] != 0) { B[0 + 1] = 1; B[6 + 2] = 1; }
                else if (B[4] != 0) { B[0 + 2] = 1; B[6 + 0] = 1; }
                else if (B[5] != 0) { B[0 + 0] = 1; B[6 + 1] = 1; }
                ncells = n[1];
            } else if (num[2] == 1) {
                for (int k = 0; k < 3; k++) B[6 + k] = win[k];
                if (B[6] != 0) { B[0 + 1] = 1; B[3 + 2] = 1; }
                else if (B[7] != 0) { B[0 + 2] = 1; B[3 + 0] = 1; }
                else if (B[8] != 0) { B[0 + 0] = 1; B[3 + 1] = 1; }
                ncells = n[2];
            }
        } else if (isdim == 2) {
            if (num[2] == 1) {
                for (int k = 0; k < 3; k++) { B[k] = uin[k]; B[3 + k] = vin[k]; B[6 + k] = 1.0; }
                for (int k = 0; k < 3; k++) if (B[k] != 0 || B[3 + k] != 0) B[6 + k] = 0.0;
                ncells = (int64_t)n[0] * n[1];
            } else if (num[1] == 1) {
                for (int k = 0; k < 3; k++) { B[k] = uin[k]; B[3 + k] = 1.0; B[6 + k] = win[k]; }
                for (int k = 0; k < 3; k++) if (B[k] != 0 || B[6 + k] != 0) B[3 + k] = 0.0;
                ncells = (int64_t)n[0] * n[2];
            } else {
                /* the reference's third test repeats num(3)==1 and leaves
                 * bases undefined here; the evident intent: */
                for (int k = 0; k < 3; k++) { B[k] = 1.0; B[3 + k] = vin[k]; B[6 + k] = win[k]; }
                for (int k = 0; k < 3; k++) if (B[3 + k] != 0 || B[6 + k] != 0) B[k] = 0.0;
                ncells = (int64_t)n[1] * n[2];
            }
        } else if (isdim == 3) {
            for (int k = 0; k < 3; k++) { B[k] = uin[k]; B[3 + k] = vin[k]; B[6 + k] = win[k]; }
            ncells = (int64_t)n[0] * n[1] * n[2];
        }
        double voxel = oc_volume(B, B + 3, B + 6, cr->rten);
        if (voxel > 0.0) {
            const double *r = cr->rten;
            double det = M3(r,0,0) * (M3(r,1,1) * M3(r,2,2) - M3(r,1,2) * M3(r,2,1))
                       - M3(r,0,1) * (M3(r,1,0) * M3(r,2,2) - M3(r,1,2) * M3(r,2,0))
                       + M3(r,0,2) * (M3(r,1,0) * M3(r,2,1) - M3(r,1,1) * M3(r,2,0));
            scalef = (double)(float)ncells / sqrt(det) * voxel;
        }
    }
    if (scalef_out) *scalef_out = scalef;
    if (op->fave == 0.0 && fabs(scalef - 1.0) > (double)1.0e-5f) {
        int64_t ii = 0;
        for (int32_t k = 0; k < num[2]; k++)
            for (int32_t j = 0; j < num[1]; j++)
                for (int32_t i = 0; i < num[0]; i++, ii++) {
                    int bragg = 1;
                    for (int c = 0; c < 3; c++) {
                        double h = g->eck[c] + g->vi[c] * i + g->vi[3 + c] * j + g->vi[6 + c] * k;
                        bragg = bragg && fabs(h - (double)llround(h)) < (double)1.0e-4f;
                    }
                    dsi3d[ii] = bragg ? dsi[ii] / scalef : dsi[ii];
                }
    } else {
        memcpy(dsi3d, dsi, sizeof(double) * np);
    }
    return 0;
}

/* four_fill_csf / four_fill_dsi with fave < 0 (fourier_sup.f90:3844-4044):
 * in place, h slowest; comp = 2 for interleaved complex, 1 for real. */
/* four_symm_csf / four_symm_dsi (fourier_sup.f90:4048-4290): the pixel of
 * hkl = 0 from the inverted step matrix, then for every operation 2..nops
 * (spc_mat, column-major 3x3) each pixel h adds its value and a weight at
 * izero + NINT((h - izero) S) (row vector times matrix), in the reference's
 * loop order; finally value / weight / nops.  a: comp = 2 (complex, re/im
 * interleaved) or 1 values per pixel.                                      */
void oc_four_symm(const dgpu_grid *g, int32_t nops, const double *mats, double *a, int comp)
{
    const int32_t *num = g->inc;
    const int64_t np = (int64_t)num[0] * num[1] * num[2];
    double m[9], inv[9];
    for (int c = 0; c < 3; c++)
        for (int r = 0; r < 3; r++) m[r + 3 * c] = num[c] > 1 ? g->vi[r + 3 * c] : (r == c ? 1.0 : 0.0);
    double det = m[0] * (m[4] * m[8] - m[7] * m[5]) - m[3] * (m[1] * m[8] - m[7] * m[2]) + m[6] * (m[1] * m[5] - m[4] * m[2]);
    inv[0] = (m[4] * m[8] - m[7] * m[5]) / det; inv[3] = (m[6] * m[5] - m[3] * m[8]) / det;
    inv[6] = (m[3] * m[7] - m[6] * m[4]) / det; inv[1] = (m[7] * m[2] - m[1] * m[8]) / det;
    inv[4] = (m[0] * m[8] - m[6] * m[2]) / det; inv[7] = (m[6] * m[1] - m[0] * m[7]) / det;
    inv[2] = (m[1] * m[5] - m[4] * m[2]) / det; inv[5] = (m[3] * m[2] - m[0] * m[5]) / det;
    inv[8] = (m[0] * m[4] - m[3] * m[1]) / det;
    int32_t iz[3];
    for (int r = 0; r < 3; r++) {
        double u = -(inv[r] * g->eck[0] + inv[r + 3] * g->eck[1] + inv[r + 6] * g->eck[2]);
        iz[r] = num[r] > 1 ? (int32_t)lround(1.0 + u) : 1;
    }
    double *sym = (double *)malloc(sizeof(double) * comp * np);
    int32_t *w = (int32_t *)malloc(sizeof(int32_t) * np);
    memcpy(sym, a, sizeof(double) * comp * np);
    for (int64_t p = 0; p < np; p++) w[p] = 1;
    for (int i = 1; i < nops; i++) {
        const double *S = mats + 9 * i;
        for (int32_t l = 1; l <= num[2]; l++)
            for (int32_t k = 1; k <= num[1]; k++)
                for (int32_t h = 1; h <= num[0]; h++) {
                    double hkl[3] = {(double)(h - iz[0]), (double)(k - iz[1]), (double)(l - iz[2])};
                    int32_t t[3];
                    for (int c = 0; c < 3; c++) {
                        double u = hkl[0] * S[0 + 3 * c] + hkl[1] * S[1 + 3 * c] + hkl[2] * S[2 + 3 * c];
                        t[c] = iz[c] + (int32_t)lround(u);
                    }
                    if (t[0] < 1 || t[0] > num[0] || t[1] < 1 || t[1] > num[1] || t[2] < 1 || t[2] > num[2]) continue;
                    int64_t src = (h - 1) + (int64_t)num[0] * ((k - 1) + (int64_t)num[1] * (l - 1));
                    int64_t dst = (t[0] - 1) + (int64_t)num[0] * ((t[1] - 1) + (int64_t)num[1] * (t[2] - 1));
                    for (int q = 0; q < comp; q++) sym[comp * dst + q] += a[comp * src + q];
                    w[dst]++;
                }
    }
    for (int64_t p = 0; p < np; p++)
        for (int q = 0; q < comp; q++) a[comp * p + q] = sym[comp * p + q] / (double)w[p] / (double)nops;
    free(sym);
    free(w);
}

void oc_fill_bragg(const dgpu_grid *g, double *a, int comp)
{
    const int32_t *num = g->inc;
    const double *vi = g->vi;
    double step[3];
    for (int c = 0; c < 3; c++) {
        double m = vi[c];
        if (vi[3 + c] > m) m = vi[3 + c];
        if (vi[6 + c] > m) m = vi[6 + c];
        step[c] = m * (double)0.005f;
        if (num[c] == 1) step[c] = (double)0.0001f;
    }
#define AT(h, k, l) (a + comp * ((int64_t)((h) - 1) + (int64_t)num[0] * (((k) - 1) + (int64_t)num[1] * ((l) - 1))))
    for (int32_t h = 1; h <= num[0]; h++)
        for (int32_t k = 1; k <= num[1]; k++)
            for (int32_t l = 1; l <= num[2]; l++) {
                int bragg = 1;
                for (int c = 0; c < 3; c++) {
                    double x = g->eck[c] + (h - 1) * vi[c] + (k - 1) * vi[3 + c] + (l - 1) * vi[6 + c];
                    bragg = bragg && fabs(x - (double)llround(x)) < step[c];
                }
                if (!bragg) continue;
                double s[2] = {0, 0};
                int np = 0;
                const int nb[6][3] = {{h - 1, k, l}, {h + 1, k, l}, {h, k - 1, l}, {h, k + 1, l}, {h, k, l - 1}, {h, k, l + 1}};
                const int ok[6] = {h > 1, h < num[0], k > 1, k < num[1], l > 1, l < num[2]};
                for (int q = 0; q < 6; q++)
                    if (ok[q]) {
                        const double *v = AT(nb[q][0], nb[q][1], nb[q][2]);
                        for (int c = 0; c < comp; c++) s[c] += v[c];
                        np++;
                    }
                if (np > 0) {
                    double *t = AT(h, k, l);
                    for (int c = 0; c < comp; c++) t[c] = s[c] / (double)(float)np;
                }
            }
#undef AT
}

/* ---------------------------------------------------------------------- */
/* qval, discus/prog/qval.f90:65-290, with cr_amount / cr_n_real_atoms /
 * cr_u2aver of chem_aver (chem_aver_mod.f90:495-537).  Indexing as in the
 * reference: istl(i,j,1) for the form-factor sums, istl(i,1,1) for S(Q)'s
 * Q^2; the sign of <f> from cfact_pure(1,l); the <f> values keep sign 1. */
int oc_qval(const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op, int value, int laver,
            const double *csf, const double *acsf, const double *dsi, const double *rnd, double *out)
{
    const double pi = 3.1415926535897932384626433832795028841971693993751, rad = pi / 180.0;
    const int32_t *num = g->inc;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    int ns = cr->nscat;
    int tables = value == 7 || value >= 9;
    int32_t *istl = NULL;
    double *cf = NULL, *cfp = NULL, amount[64], signum[64], nreal = 0, u2 = 0;
    if (tables) {
        istl = (int32_t *)malloc(sizeof(int32_t) * np);
        if (oc_stltab(g->eck, g->vi, num, cr->rten, istl)) { free(istl); return DGPU_ERR_STL_RANGE; }
        cf = (double *)malloc(sizeof(double) * 2 * NTAB * ns);
        cfp = (double *)malloc(sizeof(double) * 2 * NTAB * ns);
        oc_formtab(cr, op, cf);
        double *ones = (double *)malloc(sizeof(double) * (ns + 1));
        for (int l = 0; l <= ns; l++) ones[l] = 1.0;
        dgpu_crystal pc = *cr;
        pc.occ = ones;
        dgpu_opts po = *op;
        po.ldbw = 0;
        oc_formtab(&pc, &po, cfp);
        free(ones);
        for (int l = 0; l <= ns; l++) amount[l] = 0;
        for (int64_t a = 0; a < cr->natoms; a++)
            if (cr->iscat[a] >= 0 && cr->iscat[a] <= ns) amount[cr->iscat[a]] += 1;
        for (int l = 0; l <= ns; l++) {
            u2 = u2 + cr->dw[l] * amount[l];
            if (l > 0) nreal += amount[l];
        }
        u2 = u2 / nreal / 8.0 / (double)(float)(pi * pi);
        for (int l = 1; l <= ns; l++) signum[l] = cfp[2 * ((int64_t)(l - 1) * NTAB + 1)] < 0.0 ? -1.0 : 1.0;
    } else if (value == 13) {
        for (int64_t a = 0; a < cr->natoms; a++)
            if (cr->iscat[a] >= 1 && cr->iscat[a] <= ns) nreal += 1;
    }
    for (int32_t k = 0; k < num[2]; k++)
        for (int32_t j = 0; j < num[1]; j++)
            for (int32_t i = 0; i < num[0]; i++) {
                int64_t p = i + (int64_t)num[0] * (j + (int64_t)num[1] * k);
                const double *fz = laver ? acsf + 2 * p : csf + 2 * p;
                double fr = fz[0], fi = fz[1], f2 = fr * fr + fi * fi, r = 0;
                double I = laver ? f2 : (dsi ? dsi[p] : 0.0);
                if (value == 1) r = I;
                else if (value == 2) r = sqrt(f2);
                else if (value == 3) r = (fr == 0 && fi == 0) ? 0.0 : atan2(fi, fr) / rad;
                else if (value == 4) r = fr;
                else if (value == 5) r = fi;
                else if (value == 6) {
                    int bragg = 1;
                    for (int l = 0; l < 3; l++) {
                        double h = g->eck[l] + g->vi[l] * (double)(float)i + g->vi[3 + l] * (double)(float)j;
                        bragg = bragg && fabs(h - (double)llround(h)) < 0.000001;
                    }
                    r = bragg ? ((fr == 0 && fi == 0) ? 0.0 : atan2(fi, fr) / rad) : (rnd[p] - 0.5) * 360.0;
                } else if (value == 13) r = I / nreal;
                else {
                    int32_t s = istl[i + (int64_t)num[0] * j];
                    int pure = value == 7 || value == 9 || value == 10 || value == 11;
                    const double *tab = pure ? cfp : cf;
                    double sum = 0;
                    for (int l = 1; l <= ns; l++) {
                        const double *c = tab + 2 * ((int64_t)(l - 1) * NTAB + s);
                        double a2 = c[0] * c[0] + c[1] * c[1];
                        if (value == 9 || value == 17) sum += a2 * amount[l];
                        else if (value == 11 || value == 19) sum += sqrt(a2) * amount[l];
                        else sum += sqrt(a2) * amount[l] * signum[l];
                    }
                    if (value == 7) {
                        double st = 2.0 * (double)istl[i] * DGPU_CFINC;
                        double q2 = (double)(float)((2 * pi) * (2 * pi) * (st * st));
                        r = I / (sum * sum) / nreal + 1.0 - exp(-q2 * u2);
                    } else if (value == 10 || value == 18) {
                        double t = sum / nreal;
                        r = t * t;
                    } else r = sum / nreal;
                }
                out[p] = r;
            }
    free(istl); free(cf); free(cfp);
    return 0;
}

/* calc_hkl (fourier_sup.f90:3230-3549), the numeric core: four_run on the
 * integer box of the listed reflections (extrema starting at 0, vi =
 * identity), then per reflection the extinction-corrected intensity, its
 * square root and the phase (:3491-3535). */
int oc_calc_hkl(const dgpu_crystal *cr, const dgpu_opts *op, const int32_t *hkl, int64_t nrefl, double scale,
                double exti, double rlambda, double *icalc, double *sigi, double *phase, int nthreads)
{
    const double pi = 3.1415926535897932384626433832795028841971693993751, rad = pi / 180.0;
    int32_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int64_t r = 0; r < nrefl; r++)
        for (int a = 0; a < 3; a++) {
            if (hkl[3 * r + a] < lo[a]) lo[a] = hkl[3 * r + a];
            if (hkl[3 * r + a] > hi[a]) hi[a] = hkl[3 * r + a];
        }
    dgpu_grid g;
    memset(&g, 0, sizeof(g));
    for (int a = 0; a < 3; a++) {
        g.inc[a] = hi[a] - lo[a] + 1;
        M3(g.vi, a, a) = 1.0;
        g.eck[a] = g.eck[3 + a] = g.eck[6 + a] = g.eck[9 + a] = lo[a];
    }
    g.eck[3 + 0] = hi[0];                        /* eck(1,2) = h_max */
    g.eck[6 + 1] = hi[1];                        /* eck(2,3) = k_max */
    g.eck[9 + 2] = hi[2];                        /* eck(3,4) = l_max */
    int64_t np = (int64_t)g.inc[0] * g.inc[1] * g.inc[2];
    double *csf = (double *)malloc(sizeof(double) * 2 * np);
    double *acsf = (double *)malloc(sizeof(double) * 2 * np);
    double *dsi = (double *)malloc(sizeof(double) * np);
    int rc = oc_four_run(cr, &g, op, csf, acsf, dsi, NULL, nthreads);
    if (rc >= 0) {
        double ncells = (double)cr->icc[0] * cr->icc[1] * cr->icc[2];
        for (int64_t r = 0; r < nrefl; r++) {
            int32_t h = hkl[3 * r], k = hkl[3 * r + 1], l = hkl[3 * r + 2];
            if (h == 0 && k == 0 && l == 0) { icalc[r] = sigi[r] = 0; if (phase) phase[r] = 0; continue; }
            int64_t p = (h - lo[0]) + (int64_t)g.inc[0] * ((k - lo[1]) + (int64_t)g.inc[1] * (l - lo[2]));
            double fr = csf[2 * p], fi = csf[2 * p + 1];
            double qq = sqrt(fr * fr + fi * fi) / ncells;
            double hv[3] = {h, k, l};
            double ds = sqrt(oc_skal(hv, hv, cr->rten));
            double tth = 2.0 * (asin(0.5 * rlambda * ds) / rad);
            double ext = pow(1.0 / (1.0 + 0.001 * exti * qq * qq * rlambda * rlambda * rlambda / sin(tth * rad)), 0.25);
            double e = qq * ext;
            icalc[r] = e * e * scale;
            sigi[r] = sqrt(fabs(icalc[r]));
            if (phase) phase[r] = atan2(fi, fr) / rad;
        }
    }
    free(csf); free(acsf); free(dsi);
    return rc;
}

/* ---- powder "complete" mode ------------------------------------------------
 * powder_complete (discus/prog/powder.f90:1829-2593) with pow_four_mode =
 * fourier: the literal rod loop, four_run_powder (:3143-3206) per rod as a
 * four_run over the rod's line of points (all atoms, no <F>, no lots; the
 * anisotropic crystal gets no Debye-Waller factor, since four_strucf is called
 * with is_anis = .false. and four_formtab leaves it out of cfact), binned by
 * powder_split (:2975-3008) in the reference's order. */

static void pw_matvec(const double *t, const double *x, double *y)   /* matmul(t, x) */
{
    for (int i = 0; i < 3; i++) y[i] = (M3(t, i, 0) * x[0] + M3(t, i, 1) * x[1]) + M3(t, i, 2) * x[2];
}

static double pw_dot(const double *a, const double *b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

static double pw_skalpro(const double *a, const double *b, const double *t)   /* metric.f90:90-105 */
{
    double m[3];
    pw_matvec(t, b, m);
    return pw_dot(a, m);
}

/* do_proj (metric.f90:337-548): res[0..2] and res[3..5] as the command
 * returns them in res_para(1:6) for the four space letters sp. */
static int pw_do_proj(const double *uin, const double *vin, const char *sp, const double *rten,
                      const double *gten, double *res)
{
    double u[3], v[3], w[3], h[3], x[3];
    memcpy(u, uin, sizeof u);
    memcpy(v, vin, sizeof v);
    if (sp[0] == 'r') { pw_matvec(rten, u, w); memcpy(u, w, sizeof u); }
    if (sp[1] == 'r') { pw_matvec(rten, v, w); memcpy(v, w, sizeof v); }
    double uv = pw_skalpro(u, v, gten);
    double vv = pw_skalpro(v, v, gten);
    if (vv == 0.0) return -1;
    for (int i = 0; i < 3; i++) w[i] = v[i] / uv / vv;
    if (sp[2] == 'r') { pw_matvec(gten, w, x); memcpy(w, x, sizeof w); }
    memcpy(res, w, sizeof w);
    pw_matvec(gten, v, h);
    double uh = pw_dot(u, h);
    double hh = pw_skalpro(h, h, rten);
    if (hh == 0.0) return -1;
    for (int i = 0; i < 3; i++) w[i] = u[i] - uh * v[i] / hh;
    if (sp[3] == 'r') { pw_matvec(gten, w, x); memcpy(w, x, sizeof w); }
    memcpy(res + 3, w, sizeof w);
    return 0;
}

/* calc_preferred (powder.f90:3332-3376) with do_bang (metric.f90:35-86):
 * lspace = .true., so the angle between hkl and pref_hkl is taken in the
 * direct metric; acos is divided by REAL(rad), rad in single precision. */
static double pw_preferred(const double *hkl, const dgpu_powder *pw)
{
    const double pi = 3.1415926535897932384626433832795028841971693993751, rad = pi / 180.0;
    double x[3], y[3];
    for (int i = 0; i < 3; i++) { x[i] = 0.0 - hkl[i]; y[i] = 0.0 - pw->pref_hkl[i]; }
    double xx = sqrt(pw_skalpro(x, x, pw->gten)), xy = pw_skalpro(x, y, pw->gten), yy = sqrt(pw_skalpro(y, y, pw->gten));
    double alpha = 0.0;
    if (xx > 0 && yy > 0) {
        double arg = xy / (xx * yy);
        if (fabs(arg) < 1.0) alpha = acos(arg) / (double)(float)rad;
        else if (arg >= 1.0) alpha = 0.0;
        else alpha = 180.0;
    }
    if (pw->pref_type == DGPU_PREF_RIETVELD) {
        double a2 = alpha <= 90.0 ? alpha * alpha : (180 - alpha) * (180 - alpha);
        return pw->pref_g2 + (1. - pw->pref_g2) * exp(pw->pref_g1 * a2);
    }
    if (pw->pref_type == DGPU_PREF_MARCH) {
        double c = pw->pref_g1 * cos(alpha * rad), s = sin(alpha * rad);
        return pw->pref_g2 + (1. - pw->pref_g2) * pow(c * c + s * s / pw->pref_g1, -1.5);
    }
    return 1.0;
}

typedef struct { int32_t ih, ik, l_start, n; double hh, kk, e31; int hreal, kreal; } pw_rod;

/* The rods of powder_complete in loop order; returns their count (rods may
 * be NULL to count only), or -1. */
static int64_t pw_rods(const dgpu_crystal *cr, const dgpu_powder *pw, int ano, pw_rod *rods)
{
    const double *del = pw->hkl_del, *sh = pw->hkl_shift, *rten = cr->rten;
    double hkl_max1 = pw->a0[0] * pw->ds_max;
    int32_t h_start = ano ? -(int32_t)(hkl_max1 / del[0]) : 0;
    int32_t h_end = (int32_t)(hkl_max1 / del[0]);
    int64_t nr = 0;
    double v[3], res[6];
    const double e1[3] = {1, 0, 0}, e2[3] = {0, 1, 0};
    for (int32_t ih = h_start; ih <= h_end; ih++) {
        double hh = ih * del[0] + sh[0];
        int hreal = fabs((round(hh) - hh) / del[0]) > 0.51;
        double u[3], u2;
        if (hh == 0.0) {
            u[0] = u[1] = u[2] = 0.0;
            u2 = 0.0;
        } else {
            double hv[3] = {hh, 0, 0};
            if (pw_do_proj(hv, e1, "rdrr", rten, pw->gten, res)) return -1;
            memcpy(u, res, sizeof u);
            u2 = pw_skalpro(u, u, rten);
        }
        if (pw_do_proj(e2, e1, "ddrr", rten, pw->gten, res)) return -1;
        memcpy(v, res + 3, sizeof v);
        double vv = sqrt(pw_skalpro(v, v, rten));
        for (int i = 0; i < 3; i++) v[i] = v[i] / vv;
        double rr = pw->ds_max * pw->ds_max - u2;
        double wmin[3], wmax[3];
        if (rr >= 0.0)
            for (int i = 0; i < 3; i++) {
                wmin[i] = u[i] - sqrt(rr) * v[i];
                wmax[i] = u[i] + sqrt(rr) * v[i];
            }
        if (!(rr > 0.0)) continue;
        int32_t k_start = (!ano && ih == 0) ? 0 : (int32_t)(wmin[1] / del[1]);
        int32_t k_end = (int32_t)(wmax[1] / del[1]);
        for (int32_t ik = k_start; ik <= k_end; ik++) {
            double kk = ik * del[1] + sh[1];
            int kreal = fabs((round(kk) - kk) / del[1]) > 0.51;
            double aaa = M3(rten, 2, 2);
            double bbb = 2.0 * (M3(rten, 0, 2) * hh + M3(rten, 1, 2) * kk);
            double ccc = M3(rten, 0, 0) * (hh * hh) + 2.0 * M3(rten, 0, 1) * hh * kk + M3(rten, 1, 1) * (kk * kk) -
                         pw->ds_max * pw->ds_max;
            double rrr = bbb * bbb - 4.0 * aaa * ccc;
            int32_t l_start = 0, l_end = 0;
            if (rrr >= 0.0) {
                double llstart = (-bbb - sqrt(rrr)) / 2. / aaa;
                double llend = (-bbb + sqrt(rrr)) / 2. / aaa;
                if (!ano && ih == 0 && ik == 0) {
                    l_start = 0;
                    l_end = (int32_t)(llend / del[2]);
                } else {
                    l_start = (int32_t)(llstart / del[2]);
                    l_end = (int32_t)(llend / del[2]);
                }
            }
            if (!(rrr > 0.0)) continue;
            double e31 = l_start * del[2] + sh[2], e32 = l_end * del[2] + sh[2];
            int32_t n = (int32_t)lround((e32 - e31) / del[2]) + 1;
            if (rods) {
                pw_rod *r = rods + nr;
                r->ih = ih; r->ik = ik; r->l_start = l_start; r->n = n;
                r->hh = hh; r->kk = kk; r->e31 = e31; r->hreal = hreal; r->kreal = kreal;
            }
            nr++;
        }
    }
    return nr;
}

int oc_powder_npkt(const dgpu_powder *pw)
{
    if (!(pw->deltaq > 0.0) || !(pw->qmax >= pw->qmin)) return -1;
    return (int)lround((pw->qmax + pw->deltaq - pw->qmin) / pw->deltaq) + 2;   /* powder.f90:1957 */
}

int oc_powder_complete(const dgpu_crystal *cr, const dgpu_powder *pw, const dgpu_opts *op, int64_t rod_lo,
                       int64_t rod_hi, double *qsp, int64_t *nrods_out, int64_t *npoints_out, int nthreads)
{
    const double pi = 3.1415926535897932384626433832795028841971693993751, zpi = 2.0 * pi;
    int n_pkt = oc_powder_npkt(pw);
    if (n_pkt < 0) return DGPU_ERR_ARG;
    if (!(pw->hkl_del[2] <= pw->hkl_del[0] && pw->hkl_del[2] <= pw->hkl_del[1])) return DGPU_ERR_UNSUPPORTED;
    int64_t nr = pw_rods(cr, pw, op->ano, NULL);
    if (nr < 0) return DGPU_ERR_ARG;
    pw_rod *rods = (pw_rod *)malloc(sizeof(pw_rod) * (nr > 0 ? nr : 1));
    pw_rods(cr, pw, op->ano, rods);
    if (rod_lo < 0) rod_lo = 0;
    if (rod_hi < 0 || rod_hi > nr) rod_hi = nr;
    if (nrods_out) *nrods_out = nr;
    int64_t *first = (int64_t *)malloc(sizeof(int64_t) * (nr + 1));
    first[0] = 0;
    for (int64_t r = 0; r < nr; r++) first[r + 1] = first[r] + (r >= rod_lo && r < rod_hi ? rods[r].n : 0);
    if (npoints_out) *npoints_out = first[nr];
    double *csf = (double *)malloc(sizeof(double) * 2 * (first[nr] > 0 ? first[nr] : 1));
    dgpu_crystal c2 = *cr;
    c2.is_anis = 0;
    dgpu_opts o2 = *op;
    o2.fave = 0.0;
    o2.aver_cells = NULL;
    o2.ilots = DGPU_LOT_OFF;
    o2.lot_all = 0;
    o2.lperiod = 1;
    o2.diff_scale = 1.0;
    o2.ldbw = (op->ldbw && !cr->is_anis) ? 1 : 0;
    int rc = 0;
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads > 0 ? nthreads : 1)
    for (int64_t r = rod_lo; r < rod_hi; r++) {
        /* four_run_powder on the rod: eck(:,1) = (hh, kk, l_start dL + shift3),
           vi(:,1) = (0, 0, dL), inc = (n, 1, 1) (powder.f90:2305-2319) */
        const pw_rod *d = rods + r;
        dgpu_grid g;
        memset(&g, 0, sizeof(g));
        for (int c = 0; c < 4; c++) { g.eck[3 * c] = d->hh; g.eck[3 * c + 1] = d->kk; g.eck[3 * c + 2] = d->e31; }
        g.eck[3 * 1 + 2] = (d->l_start + d->n - 1) * pw->hkl_del[2] + pw->hkl_shift[2];
        M3(g.vi, 2, 0) = pw->hkl_del[2];
        g.inc[0] = d->n;
        g.inc[1] = g.inc[2] = 1;
        double *acsf = (double *)malloc(sizeof(double) * 2 * d->n);
        double *dsi = (double *)malloc(sizeof(double) * d->n);
        int rr = oc_four_run(&c2, &g, &o2, csf + 2 * first[r], acsf, dsi, NULL, 1);
        if (rr < 0) {
#pragma omp critical
            rc = rr;
        }
        free(acsf);
        free(dsi);
    }
    if (rc >= 0) {
        memset(qsp, 0, sizeof(double) * (n_pkt + 1));
        for (int64_t r = rod_lo; r < rod_hi; r++) {
            const pw_rod *d = rods + r;
            for (int32_t i = 1; i <= d->n; i++) {
                double hkl[3] = {d->hh, d->kk, d->e31 + (i - 1) * pw->hkl_del[2]};
                double ll = hkl[2];
                int lreal = fabs((round(ll) - ll) / pw->hkl_del[2]) > 0.51;
                if (!(pw->l_all || d->hreal || d->kreal || lreal)) continue;
                double dstar = sqrt(pw_skalpro(hkl, hkl, cr->rten));
                double q = zpi * dstar;
                if (!(pw->qmin <= q && q <= pw->qmax + pw->deltaq)) continue;
                const double *f = csf + 2 * (first[r] + i - 1);
                double inten = (f[0] * f[0] - f[1] * (-f[1])) * 1.0;           /* DBLE(csf conjg(csf)) */
                if (pw->pref_type != DGPU_PREF_NONE) inten = inten * pw_preferred(hkl, pw);
                /* powder_split */
                int32_t it1 = (int32_t)((q - pw->qmin) / pw->deltaq);
                double frac1 = 1.0 - ((q - pw->qmin) / pw->deltaq - (int32_t)((q - pw->qmin) / pw->deltaq));
                double frac2 = ((q - pw->qmin) / pw->deltaq - (int32_t)((q - pw->qmin) / pw->deltaq));
                if (it1 < 0 || it1 + 1 > n_pkt) continue;
                qsp[it1] += inten * frac1;
                qsp[it1 + 1] += inten * frac2;
            }
        }
        if (!op->ano)
            for (int i = 0; i <= n_pkt; i++) qsp[i] = qsp[i] * 2.0;   /* half-volume correction */
    }
    free(csf);
    free(first);
    free(rods);
    return rc;
}
