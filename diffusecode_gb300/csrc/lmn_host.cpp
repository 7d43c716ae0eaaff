// fourier_lmn (discus/prog/fourier_lmn_mod.f90:4-279) on the host, in IEEE
// binary128 like the reference's PREC_QP: the integer decomposition of the
// grid corner, eck(:,1) = sum_k lmn(k) vi(:,k) + sum_k lmn(3+k) off_shift(:,k),
// that makes the REF22 phases at h and -h exact negatives of each other.
// Corners and increments are first rounded to 1e-7 (:48-49).
#include <math.h>
#include <stdint.h>

#include "../../include/discus_gpu.h"

namespace {

#if defined(__aarch64__)
typedef long double quad;
#else
typedef __float128 quad;
#endif

inline quad qabs(quad x) { return x < 0 ? -x : x; }

inline quad qsqrt(quad x)
{
    if (x <= 0) return 0;
    quad y = (quad)sqrt((double)x);
    for (int it = 0; it < 2; ++it) y = (y + x / y) / 2;   // Newton from a double seed
    return y;
}

// Fortran NINT (half away from zero)
inline int64_t qnint(quad x)
{
    quad a = qabs(x) + (quad)0.5;
    int64_t v = (int64_t)a;
    return x < 0 ? -v : v;
}

struct Mat3 {
    quad m[3][3];   // m[row][col]
    quad &operator()(int r, int c) { return m[r][c]; }
    quad operator()(int r, int c) const { return m[r][c]; }
};

// direct 3x3 inverse by cofactors (lib_f90/matrix_mod.f90:271-300)
bool inverse(const Mat3 &a, Mat3 &b)
{
    quad det = a(0,0) * a(1,1) * a(2,2) - a(0,0) * a(1,2) * a(2,1) - a(0,1) * a(1,0) * a(2,2)
             + a(0,1) * a(1,2) * a(2,0) + a(0,2) * a(1,0) * a(2,1) - a(0,2) * a(1,1) * a(2,0);
    if (det == 0) return false;
    quad di = (quad)1 / det;
    b(0,0) = +di * (a(1,1) * a(2,2) - a(1,2) * a(2,1));
    b(1,0) = -di * (a(1,0) * a(2,2) - a(1,2) * a(2,0));
    b(2,0) = +di * (a(1,0) * a(2,1) - a(1,1) * a(2,0));
    b(0,1) = -di * (a(0,1) * a(2,2) - a(0,2) * a(2,1));
    b(1,1) = +di * (a(0,0) * a(2,2) - a(0,2) * a(2,0));
    b(2,1) = -di * (a(0,0) * a(2,1) - a(0,1) * a(2,0));
    b(0,2) = +di * (a(0,1) * a(1,2) - a(0,2) * a(1,1));
    b(1,2) = -di * (a(0,0) * a(1,2) - a(0,2) * a(1,0));
    b(2,2) = +di * (a(0,0) * a(1,1) - a(0,1) * a(1,0));
    return true;
}

inline quad norm3(const quad v[3]) { return qsqrt(qabs(v[0] * v[0] + v[1] * v[1] + v[2] * v[2])); }

}  // namespace

int dgpu_lmn_host(const double eck_in[12], const double vi_in[9], const int32_t inc[3],
                  int32_t lmn[6], double off_out[9])
{
    const quad big = 10000000;
    const quad tol7 = (quad)1.0e-7f;    // single-precision literal 1.E-7 of the reference
    const quad tol9 = (quad)1.0e-9;
    // v[axis][component], c = corner ll
    quad v[3][3], c[3], off[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 3; ++k) v[a][k] = (quad)qnint((quad)vi_in[3 * a + k] * big) / big;
    for (int k = 0; k < 3; ++k) c[k] = (quad)qnint((quad)eck_in[k] * big) / big;
    for (int k = 0; k < 6; ++k) lmn[k] = 0;

    Mat3 A = {};
    int thick[3], ndim = 0;
    bool has_inc[3] = {false, false, false};
    for (int a = 0; a < 3; ++a) {
        if (inc[a] <= 1) continue;
        if (!(norm3(v[a]) > tol7)) return DGPU_ERR_ZERO_INC;
        thick[ndim++] = a;
        has_inc[a] = true;
        for (int k = 0; k < 3; ++k) A(k, a) = v[a][k];
    }

    bool solve = true;
    if (ndim == 0) {
        for (int k = 0; k < 3; ++k) { off[k][k] = 1; A(k, k) = 1; }
    } else if (ndim == 1) {
        const int j = thick[0], j1 = (j + 1) % 3, j2 = (j + 2) % 3;
        // rows parallel to a*, b* or c* (:103-169): these read vi(:,1) as the step
        int axis = -1;
        if (v[j][1] == 0 && v[j][2] == 0) axis = 0;
        else if (v[j][0] == 0 && v[j][2] == 0) axis = 1;
        else if (v[j][0] == 0 && v[j][1] == 0) axis = 2;
        if (axis >= 0) {
            if (v[0][axis] == 0) return DGPU_ERR_ARG;
            quad r = c[axis] / v[0][axis];
            lmn[0] = (int32_t)qnint(r);
            if (qabs(r - (quad)qnint(r)) > tol9) {
                lmn[3] = 1;
                off[0][axis] = r - (quad)qnint(r);
            }
            lmn[4] = 1;
            lmn[5] = 1;
            if (axis == 0) { off[1][1] = c[1]; off[2][2] = c[2]; }
            if (axis == 1) { off[1][0] = c[0]; off[2][2] = c[2]; }
            if (axis == 2) { off[1][0] = c[0]; off[2][1] = c[1]; }
            solve = false;
        } else {
            const quad s = (quad)0.001f;   // single-precision literal 0.001
            static const double fill[6] = {0.3141592, 0.2718281, 0.5772156, 0.6931471, 0.4142135, 0.7320508};
            quad *o2 = off[j2], *o1 = off[j1];
            o2[0] = c[1] * v[j][2] - c[2] * v[j][1];
            o2[1] = c[2] * v[j][0] - c[0] * v[j][2];
            o2[2] = c[0] * v[j][1] - c[1] * v[j][0];
            quad d = norm3(o2);
            if (d > tol7) {
                for (int k = 0; k < 3; ++k) o2[k] = o2[k] * s / d;
                o1[0] = o2[1] * v[j][2] - o2[2] * v[j][1];
                o1[1] = o2[2] * v[j][0] - o2[0] * v[j][2];
                o1[2] = o2[0] * v[j][1] - o2[1] * v[j][0];
                d = norm3(o1);
                if (d > tol7) for (int k = 0; k < 3; ++k) o1[k] = o1[k] * s / d;
                else for (int k = 0; k < 3; ++k) o1[k] = fill[k];
            } else {
                // a line through the origin: these directions get lmn = 0, so
                // the values (ran1 draws in the reference) never enter a phase
                for (int k = 0; k < 3; ++k) { o1[k] = fill[k]; o2[k] = fill[3 + k]; }
            }
            for (int k = 0; k < 3; ++k) { A(k, j1) = o1[k]; A(k, j2) = o2[k]; }
        }
    } else if (ndim == 2) {
        const int j = thick[0], j1 = thick[1], j2 = 3 - j - j1;
        quad *o = off[j2];
        o[0] = v[j][1] * v[j1][2] - v[j][2] * v[j1][1];
        o[1] = v[j][2] * v[j1][0] - v[j][0] * v[j1][2];
        o[2] = v[j][0] * v[j1][1] - v[j][1] * v[j1][0];
        quad d = qsqrt(o[0] * o[0] + o[1] * o[1] + o[2] * o[2]);
        for (int k = 0; k < 3; ++k) { o[k] = o[k] * (quad)0.001 / d; A(k, j2) = o[k]; }
    }

    if (solve) {
        Mat3 Ai;
        if (!inverse(A, Ai)) return DGPU_ERR_ARG;
        quad r[3], fr[3], t[3];
        for (int a = 0; a < 3; ++a) r[a] = Ai(a, 0) * c[0] + Ai(a, 1) * c[1] + Ai(a, 2) * c[2];
        for (int a = 0; a < 3; ++a)
            if (qabs(r[a] - (quad)qnint(r[a])) < tol9) r[a] = (quad)qnint(r[a]);
        for (int a = 0; a < 3; ++a) { lmn[a] = (int32_t)qnint(r[a]); fr[a] = r[a] - (quad)qnint(r[a]); }
        for (int a = 0; a < 3; ++a) t[a] = A(a, 0) * fr[0] + A(a, 1) * fr[1] + A(a, 2) * fr[2];
        for (int a = 0; a < 3; ++a) {
            if (!has_inc[a]) {
                lmn[a + 3] = lmn[a];
                lmn[a] = 0;
            } else {
                off[a][a] = off[a][a] + t[a];
                lmn[3 + a] = 1;
                if (qabs(off[a][a]) < tol9) { off[a][a] = 0; lmn[3 + a] = 0; }
            }
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int k = 0; k < 3; ++k) off_out[3 * a + k] = (double)off[a][k];
    return DGPU_OK;
}
