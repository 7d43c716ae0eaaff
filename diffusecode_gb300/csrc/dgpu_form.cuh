// Form factors at one grid point, shared by the combine and adjoint kernels:
// h of a box point, cfact of a type (table, four_formtab fourier_sup.f90:
// 2691-2743, or the same formula at the exact sin(theta)/lambda), the
// anisotropic Debye-Waller term (four_dbwtab, fourier_sup.f90:2809-2831) and
// the factor of a partial-sum group (tcsf_form_iso / tcsf_form_aniso,
// fourier_form.f90:106-177).
#pragma once
#include "dgpu_internal.h"

// h = eck + i vi_1 + j vi_2 + l vi_3, unfused (four_dbwtab :2810-2821)
__device__ __forceinline__ void form_hvec(const FormSpec *fs, int64_t i, int64_t j, int64_t l, double h[3])
{
    for (int k = 0; k < 3; k++)
        h[k] = __dadd_rn(__dadd_rn(__dadd_rn(fs->eck[k], __dmul_rn(fs->vi[k], (double)i)),
                                   __dmul_rn(fs->vi[3 + k], (double)j)),
                         __dmul_rn(fs->vi[6 + k], (double)l));
}

// cfact of type t (1-based) at a point: table or exact sin(theta)/lambda
__device__ __forceinline__ double2 form_cfact(const FormSpec *fs, const double2 *cfact, int32_t istl,
                                              int t, const double h[3])
{
    if (fs->mode == DGPU_FORM_TABLE) return cfact[(int64_t)(t - 1) * DGPU_NTAB + istl];
    const double *r = fs->rten;
    double t0 = __dadd_rn(__dadd_rn(__dmul_rn(r[0], h[0]), __dmul_rn(r[3], h[1])), __dmul_rn(r[6], h[2]));
    double t1 = __dadd_rn(__dadd_rn(__dmul_rn(r[1], h[0]), __dmul_rn(r[4], h[1])), __dmul_rn(r[7], h[2]));
    double t2 = __dadd_rn(__dadd_rn(__dmul_rn(r[2], h[0]), __dmul_rn(r[5], h[1])), __dmul_rn(r[8], h[2]));
    double q2 = __dadd_rn(__dadd_rn(__dmul_rn(h[0], t0), __dmul_rn(h[1], t1)), __dmul_rn(h[2], t2)) / 4.0;
    const double *sc = fs->scat + 11 * t;
    double f = sc[0];
    if (fs->lxray)
        for (int i = 1; i <= fs->power; i++) f = __dadd_rn(f, __dmul_rn(sc[2 * i - 1], exp(-__dmul_rn(sc[2 * i], q2))));
    double fp = fs->ano ? fs->delfr[t] : 0.0, fpp = fs->ano ? fs->delfi[t] : 0.0;
    double sb = fs->ldbw ? __dmul_rn(exp(-__dmul_rn(fs->dw[t], q2)), fs->occ[t]) : fs->occ[t];
    return make_double2(__dmul_rn(sb, __dadd_rn(f, fp)), __dmul_rn(sb, fpp));
}

// exp(-2 pi^2 sum_ij h_i h_j a*_i a*_j U_ij) of group g, in the reference's
// order of terms: (U11 + U22 + U33 + 2 U23 + 2 U13 + 2 U12) * zpi * pi
__device__ __forceinline__ double form_anis_dbw(const FormSpec *fs, int g, const double h[3])
{
    const double pi = 3.1415926535897932384626433832795028841971693993751;
    const double *u = fs->gU + 6 * g, *a = fs->ar;
    double t11 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(h[0], h[0]), a[0]), a[0]), u[0]);
    double t22 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(h[1], h[1]), a[1]), a[1]), u[1]);
    double t33 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(h[2], h[2]), a[2]), a[2]), u[2]);
    double t23 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(h[1], h[2]), a[1]), a[2]), u[3]), 2.0);
    double t13 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(h[0], h[2]), a[0]), a[2]), u[4]), 2.0);
    double t12 = __dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(__dmul_rn(h[0], h[1]), a[0]), a[1]), u[5]), 2.0);
    double arg = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(t11, t22), t33), t23), t13), t12);
    arg = __dmul_rn(__dmul_rn(arg, 2.0 * pi), pi);
    return exp(-arg);
}

// whether the factors need h (analytic form factor, anisotropic term, DISCAMB)
__device__ __forceinline__ bool form_needs_h(const FormSpec *fs)
{
    return fs->mode != DGPU_FORM_TABLE || fs->adbw || fs->disc;
}

// DISCAMB table of group g at nint(h) (tcsf_form_discamb, fourier_form.f90:
// 90-97; nint rounds half away from zero); NaN outside the table
__device__ __forceinline__ double2 form_discamb(const FormSpec *fs, int g, const double h[3])
{
    const int32_t m0 = fs->gtab[g];
    if (m0 < 0 || m0 >= fs->dntab) return make_double2(nan(""), nan(""));
    int64_t idx = 0, stride = 1;
    for (int k = 0; k < 3; k++) {
        const double r = round(h[k]);
        const int32_t m = fs->dmax[k];
        if (!(r >= -(double)m && r <= (double)m)) return make_double2(nan(""), nan(""));
        idx += ((int64_t)r + m) * stride;
        stride *= 2 * (int64_t)m + 1;
    }
    return fs->dtab[(int64_t)m0 * stride + idx];
}

// factor of partial-sum group g (1-based)
__device__ __forceinline__ double2 form_group(const FormSpec *fs, const double2 *cfact, int32_t istl, int g,
                                              const double h[3])
{
    double2 c = fs->disc ? form_discamb(fs, g, h) : form_cfact(fs, cfact, istl, fs->gtype[g], h);
    if (fs->adbw) {
        const double d = form_anis_dbw(fs, g, h);
        c.x = __dmul_rn(c.x, d);
        c.y = __dmul_rn(c.y, d);
    }
    return c;
}

__device__ __forceinline__ double2 cmul(double2 a, double2 b)
{
    return make_double2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

// one-axis geometric series sum_{m<n} exp(2 pi i x m)
__device__ __forceinline__ double2 geom_series(double x, int32_t n)
{
    double xr = x - rint(x);
    if (xr == 0.0) return make_double2((double)n, 0.0);
    double num = sinpi((double)n * xr), den = sinpi(xr);
    double r = num / den, sp, cp;
    sincospi(xr * (double)(n - 1), &sp, &cp);
    return make_double2(r * cp, r * sp);
}

// Lattice sum of a box of c0 x c1 x c2 cells starting at d (four_strucf(0,..)
// over the lattice of four_getav, fourier_sup.f90:1315-1318) in closed form:
// a product of three geometric series times exp(2 pi i h.d), the phase
// h.d reduced exactly.
__device__ __forceinline__ double2 lattice_closed(const double h[3], int32_t c0, int32_t c1, int32_t c2, double d0,
                                                  double d1, double d2)
{
    double2 L = cmul(cmul(geom_series(h[0], c0), geom_series(h[1], c1)), geom_series(h[2], c2));
    double p0 = h[0] * d0, e0 = fma(h[0], d0, -p0);
    double p1 = h[1] * d1, e1 = fma(h[1], d1, -p1);
    double p2 = h[2] * d2, e2 = fma(h[2], d2, -p2);
    double ph = (p0 - rint(p0)) + (p1 - rint(p1)) + (p2 - rint(p2)) + (e0 + e1 + e2);
    double sp, cp;
    sincospi(2.0 * ph, &sp, &cp);
    return cmul(L, make_double2(cp, sp));
}

// box point of partial-sum layout slot r (PartLayout), false for a padding slot
__device__ __forceinline__ bool part_point(const PartLayout &L, const BoxSpec &box, int64_t r, int64_t &i,
                                           int64_t &j, int64_t &l)
{
    const int64_t c2 = r / L.m2, rem = r - c2 * L.m2, c1 = L.m1 > 0 ? rem / L.m1 : 0, c0 = rem - c1 * L.m1;
    if (c0 >= box.f[L.a0] || c1 >= box.f[L.a1] || c2 >= box.f[L.a2]) return false;
    i = L.a0 == 0 ? c0 : L.a1 == 0 ? c1 : c2;
    j = L.a0 == 1 ? c0 : L.a1 == 1 ? c1 : c2;
    l = L.a0 == 2 ? c0 : L.a1 == 2 ? c1 : c2;
    return true;
}
