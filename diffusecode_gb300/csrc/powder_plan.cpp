// Host planner of powder "complete" mode: which (h, k) rods powder_complete
// (discus/prog/powder.f90:1829-2593) evaluates and over which l range, then
// the h-slabs the device evaluates them in.  Compiled without floating-point
// contraction so that the rod limits round as the reference's do.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "dgpu_powder.h"

namespace {

// column-major 3x3 times vector, each component summed j = 1, 2, 3 (matmul)
void matvec(const double t[9], const double x[3], double y[3])
{
    for (int i = 0; i < 3; i++) y[i] = (t[i] * x[0] + t[i + 3] * x[1]) + t[i + 6] * x[2];
}

double dot3(const double a[3], const double b[3]) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }

// skalpro (metric.f90:90-105): dot_product(a, matmul(t, b))
double skal(const double a[3], const double b[3], const double t[9])
{
    double m[3];
    matvec(t, b, m);
    return dot3(a, m);
}

// nint of a double as Fortran rounds it (half away from zero)
double fnint(double x) { return (double)llround(x); }

}  // namespace

int32_t dgpu_powder_npkt_host(const dgpu_powder *pw)
{
    if (!pw || !(pw->deltaq > 0.0) || !(pw->qmax >= pw->qmin)) return -1;
    const double x = (pw->qmax + pw->deltaq - pw->qmin) / pw->deltaq;
    if (!(x < 2.0e9)) return -1;
    return (int32_t)llround(x) + 2;
}

int dgpu_powder_plan(const double rten[9], const dgpu_powder *pw, int ano, int min_slabs, int64_t max_points,
                     PowderPlan &plan, char *msg, size_t msg_len)
{
    plan = PowderPlan();
    plan.n_pkt = dgpu_powder_npkt_host(pw);
    if (plan.n_pkt < 0) {
        snprintf(msg, msg_len, "invalid Q range (qmin %g, qmax %g, deltaq %g)", pw->qmin, pw->qmax, pw->deltaq);
        return DGPU_ERR_ARG;
    }
    const double *del = pw->hkl_del, *sh = pw->hkl_shift, *gten = pw->gten;
    for (int a = 0; a < 3; a++)
        if (!(del[a] > 0.0)) {
            snprintf(msg, msg_len, "hkl step %d must be > 0", a + 1);
            return DGPU_ERR_ARG;
        }
    // trans_to_short (discus_trans_to_short.f90:26-60) leaves the structure
    // alone only when dL is the smallest step; the transformed case is the caller's
    if (!(del[2] <= del[0] && del[2] <= del[1])) {
        snprintf(msg, msg_len, "dL must be the smallest hkl step (the structure transformation is not done here)");
        return DGPU_ERR_UNSUPPORTED;
    }
    if (!(pw->ds_max > 0.0) || !(rten[8] > 0.0)) {
        snprintf(msg, msg_len, "ds_max and the reciprocal metric must be positive");
        return DGPU_ERR_ARG;
    }
    const double ds2 = pw->ds_max * pw->ds_max;

    // do_proj "0,1,0, 1,0,0, ddrr" (metric.f90:337-548): the part of b normal
    // to a, in reciprocal coordinates, then normalised (powder.f90:2045-2057)
    double v[3];
    {
        const double e1[3] = {1.0, 0.0, 0.0}, e2[3] = {0.0, 1.0, 0.0};
        double h[3];
        matvec(gten, e1, h);
        const double uh = dot3(e2, h);
        const double hh = skal(h, h, rten);
        if (hh == 0.0) {
            snprintf(msg, msg_len, "degenerate metric");
            return DGPU_ERR_ARG;
        }
        double w[3];
        for (int i = 0; i < 3; i++) w[i] = e2[i] - uh * e1[i] / hh;
        matvec(gten, w, v);
        const double vv = sqrt(skal(v, v, rten));
        for (int i = 0; i < 3; i++) v[i] = v[i] / vv;
    }

    const double hmax = pw->a0[0] * pw->ds_max;
    const int32_t h_end = (int32_t)(hmax / del[0]);
    const int32_t h_start = ano ? -h_end : 0;
    for (int32_t ih = h_start; ih <= h_end; ih++) {
        const double hh = ih * del[0] + sh[0];
        double u[3] = {0.0, 0.0, 0.0}, u2 = 0.0;
        if (hh != 0.0) {
            // do_proj "hh,0,0, 1,0,0, rdrr": its parallel part is v / (u.v) / |v|^2
            const double hv[3] = {hh, 0.0, 0.0}, e1[3] = {1.0, 0.0, 0.0};
            double ud[3];
            matvec(rten, hv, ud);
            const double uv = skal(ud, e1, gten);
            const double vv = skal(e1, e1, gten);
            double w[3];
            for (int i = 0; i < 3; i++) w[i] = e1[i] / uv / vv;
            matvec(gten, w, u);
            u2 = skal(u, u, rten);
        }
        const double rr = ds2 - u2;
        if (!(rr > 0.0)) continue;
        const double sr = sqrt(rr);
        const double wmin2 = u[1] - sr * v[1], wmax2 = u[1] + sr * v[1];
        const int32_t k_start = (!ano && ih == 0) ? 0 : (int32_t)(wmin2 / del[1]);
        const int32_t k_end = (int32_t)(wmax2 / del[1]);
        for (int32_t ik = k_start; ik <= k_end; ik++) {
            const double kk = ik * del[1] + sh[1];
            const double aaa = rten[8];
            const double bbb = 2.0 * (rten[6] * hh + rten[7] * kk);
            const double ccc = ((rten[0] * (hh * hh) + 2.0 * rten[3] * hh * kk) + rten[4] * (kk * kk)) - ds2;
            const double rrr = bbb * bbb - 4.0 * aaa * ccc;
            if (!(rrr > 0.0)) continue;
            const double llstart = (-bbb - sqrt(rrr)) / 2.0 / aaa;
            const double llend = (-bbb + sqrt(rrr)) / 2.0 / aaa;
            const int32_t l_start = (!ano && ih == 0 && ik == 0) ? 0 : (int32_t)(llstart / del[2]);
            const int32_t l_end = (int32_t)(llend / del[2]);
            const double e31 = l_start * del[2] + sh[2], e32 = l_end * del[2] + sh[2];
            const int32_t n = (int32_t)fnint((e32 - e31) / del[2]) + 1;
            if (n < 1) continue;
            plan.rods.push_back({ih, ik, l_start, n});
            plan.rod_points += n;
        }
    }
    if (plan.rods.empty()) return 0;

    // ---- slabs: consecutive h planes with about equal rod points ----
    struct Plane {
        int32_t ih;
        size_t r0, r1;   // rods [r0, r1)
        int64_t pts;
    };
    std::vector<Plane> planes;
    for (size_t r = 0; r < plan.rods.size(); r++) {
        if (planes.empty() || planes.back().ih != plan.rods[r].ih) planes.push_back({plan.rods[r].ih, r, r, 0});
        planes.back().r1 = r + 1;
        planes.back().pts += plan.rods[r].n;
    }
    auto box_of = [&](size_t p0, size_t p1, int32_t kq0, int32_t kq1, PowderSlab &s) {
        // bounds of the rods of planes [p0, p1) with k in [kq0, kq1]
        int32_t k0 = INT32_MAX, k1 = INT32_MIN, l0 = INT32_MAX, l1 = INT32_MIN;
        for (size_t p = p0; p < p1; p++)
            for (size_t r = planes[p].r0; r < planes[p].r1; r++) {
                const PowderRod &d = plan.rods[r];
                if (d.ik < kq0 || d.ik > kq1) continue;
                k0 = std::min(k0, d.ik);
                k1 = std::max(k1, d.ik);
                l0 = std::min(l0, d.l0);
                l1 = std::max(l1, d.l0 + d.n - 1);
            }
        s.h0 = planes[p0].ih;
        s.nh = planes[p1 - 1].ih - planes[p0].ih + 1;
        s.k0 = k0;
        s.nk = k1 - k0 + 1;
        s.l0 = l0;
        s.nl = l1 - l0 + 1;
        return k0 <= k1;
    };
    auto points = [](const PowderSlab &s) { return (int64_t)s.nh * s.nk * s.nl; };
    const int64_t total = plan.rod_points;
    const int want = std::max(1, std::min((int)planes.size(), min_slabs));
    std::vector<std::pair<size_t, size_t>> groups;
    {
        size_t p0 = 0;
        int64_t acc = 0;
        for (size_t p = 0; p < planes.size(); p++) {
            acc += planes[p].pts;
            const int64_t target = total * (int64_t)(groups.size() + 1) / want;
            if (acc >= target || p + 1 == planes.size()) {
                groups.push_back({p0, p + 1});
                p0 = p + 1;
            }
        }
    }
    // split groups whose box exceeds max_points: by planes, then by k within a plane
    std::vector<std::pair<size_t, size_t>> work(groups.rbegin(), groups.rend());
    while (!work.empty()) {
        auto g = work.back();
        work.pop_back();
        PowderSlab s;
        box_of(g.first, g.second, INT32_MIN, INT32_MAX, s);
        if (points(s) <= max_points) {
            s.tab_off = 0;
            plan.slabs.push_back(s);
            continue;
        }
        if (g.second - g.first > 1) {
            const size_t mid = (g.first + g.second) / 2;
            work.push_back({mid, g.second});
            work.push_back({g.first, mid});
            continue;
        }
        // one plane: k pieces of at most max_points / nl rows
        const int64_t rows = max_points / std::max(1, s.nl);
        if (rows < 1) {
            snprintf(msg, msg_len, "a rod of %d points exceeds the device grid limit", s.nl);
            return DGPU_ERR_ARG;
        }
        for (int32_t k = s.k0; k < s.k0 + s.nk; k += (int32_t)rows) {
            PowderSlab q;
            if (box_of(g.first, g.second, k, (int32_t)std::min<int64_t>(k + rows - 1, s.k0 + s.nk - 1), q)) {
                q.tab_off = 0;
                plan.slabs.push_back(q);
            }
        }
    }
    // rod tables
    for (PowderSlab &s : plan.slabs) {
        s.tab_off = (int64_t)plan.tab.size() / 2;
        plan.tab.resize(plan.tab.size() + 2 * (size_t)s.nh * s.nk, 0);
        plan.grid_points += points(s);
    }
    for (const PowderRod &d : plan.rods)
        for (const PowderSlab &s : plan.slabs) {
            if (d.ih < s.h0 || d.ih >= s.h0 + s.nh || d.ik < s.k0 || d.ik >= s.k0 + s.nk) continue;
            const int64_t e = s.tab_off + (int64_t)(d.ih - s.h0) * s.nk + (d.ik - s.k0);
            plan.tab[2 * e] = d.l0;
            plan.tab[2 * e + 1] = d.n;
            break;
        }
    return 0;
}
