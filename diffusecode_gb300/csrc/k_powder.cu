// Powder "complete" mode on the device: powder_complete
// (discus/prog/powder.f90:1829-2593) with four_run_powder (:3143-3206) as the
// structure factor and powder_split (:2975-3008) as the binning.
//
// The reference evaluates F rod by rod.  Here the rods of consecutive h
// planes share one (l, k, h) box that four_run's engine evaluates in one
// call; k_powder_bin then walks the box, keeps the points that lie on a rod
// and adds |F|^2 (times the preferred-orientation factor) to the two Q bins
// with FP64 atomics.  The box coordinates, Q and the split follow the
// reference's formulas operation by operation (no contraction), so every
// point lands in the reference's bins with the reference's weights.
#include <math.h>

#include <algorithm>
#include <vector>

#include "dgpu_internal.h"
#include "dgpu_powder.h"

namespace {

struct BinSpec {
    int32_t h0, nh, k0, nk, l0, nl;
    const int2 *tab;          // (l_start, inc) per (h, k) of the slab
    double del[3], sh[3];
    double rten[9], gten[9];
    double qmin, qtop, deltaq;   // qtop = qmax + deltaq
    int32_t l_all, n_pkt;
    int32_t pref_type;
    double pref[3], g1, g2;
};

__device__ __forceinline__ double dm(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double da(double a, double b) { return __dadd_rn(a, b); }

// skalpro (metric.f90:90-105): dot_product(a, matmul(t, b)), no contraction
__device__ double skal_d(const double a[3], const double b[3], const double t[9])
{
    double m[3];
#pragma unroll
    for (int i = 0; i < 3; i++) m[i] = da(da(dm(t[i], b[0]), dm(t[i + 3], b[1])), dm(t[i + 6], b[2]));
    return da(da(dm(a[0], m[0]), dm(a[1], m[1])), dm(a[2], m[2]));
}

// calc_preferred (powder.f90:3332-3376); its angle comes from do_bang
// (metric.f90:35-86) called with lspace = .true., i.e. in the direct metric,
// and divides by rad rounded to single precision.
__device__ double preferred(const BinSpec &s, const double hkl[3])
{
    const double x[3] = {-hkl[0], -hkl[1], -hkl[2]};
    const double y[3] = {-s.pref[0], -s.pref[1], -s.pref[2]};
    const double xx = sqrt(skal_d(x, x, s.gten));
    const double xy = skal_d(x, y, s.gten);
    const double yy = sqrt(skal_d(y, y, s.gten));
    double alpha = 0.0;
    if (xx > 0.0 && yy > 0.0) {
        const double arg = xy / dm(xx, yy);
        const double rad_sp = (double)(float)(3.1415926535897932384626433832795 / 180.0);
        if (fabs(arg) < 1.0) alpha = acos(arg) / rad_sp;
        else if (arg >= 1.0) alpha = 0.0;
        else alpha = 180.0;
    }
    const double rad = 3.1415926535897932384626433832795 / 180.0;
    if (s.pref_type == DGPU_PREF_RIETVELD) {
        const double a2 = alpha <= 90.0 ? dm(alpha, alpha) : dm(180.0 - alpha, 180.0 - alpha);
        return da(s.g2, dm(1.0 - s.g2, exp(dm(s.g1, a2))));
    }
    if (s.pref_type == DGPU_PREF_MARCH) {
        const double c = dm(s.g1, cos(dm(alpha, rad)));
        const double sn = sin(dm(alpha, rad));
        return da(s.g2, dm(1.0 - s.g2, pow(da(dm(c, c), dm(sn, sn) / s.g1), -1.5)));
    }
    return 1.0;
}

// one thread per box point; points off the rods return at once
__global__ void k_powder_bin(BinSpec s, const double2 *__restrict__ csf, double *__restrict__ qsp,
                             unsigned long long *__restrict__ nbinned)
{
    const int64_t np = (int64_t)s.nl * s.nk * s.nh;
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    bool added = false;
    if (p < np) {
        const int32_t jl = (int32_t)(p % s.nl);
        const int64_t r = p / s.nl;
        const int32_t jk = (int32_t)(r % s.nk), jh = (int32_t)(r / s.nk);
        const int2 rod = s.tab[(int64_t)jh * s.nk + jk];
        const int32_t il = s.l0 + jl;
        const int32_t i = il - rod.x;                      // i - 1 of the rod's loop
        if (rod.y > 0 && i >= 0 && i < rod.y) {
            const int32_t ih = s.h0 + jh, ik = s.k0 + jk;
            double hkl[3];
            hkl[0] = da(dm((double)ih, s.del[0]), s.sh[0]);
            hkl[1] = da(dm((double)ik, s.del[1]), s.sh[1]);
            hkl[2] = da(da(dm((double)rod.x, s.del[2]), s.sh[2]), dm((double)i, s.del[2]));
            const bool hreal = fabs((round(hkl[0]) - hkl[0]) / s.del[0]) > 0.51;
            const bool kreal = fabs((round(hkl[1]) - hkl[1]) / s.del[1]) > 0.51;
            const bool lreal = fabs((round(hkl[2]) - hkl[2]) / s.del[2]) > 0.51;
            if (s.l_all || hreal || kreal || lreal) {
                const double q = dm(6.283185307179586476925286766559, sqrt(skal_d(hkl, hkl, s.rten)));
                if (s.qmin <= q && q <= s.qtop) {
                    const double2 f = csf[p];
                    double inten = da(dm(f.x, f.x), dm(f.y, f.y));
                    if (s.pref_type != DGPU_PREF_NONE) inten = dm(inten, preferred(s, hkl));
                    const double x = (q - s.qmin) / s.deltaq;
                    const int32_t it = (int32_t)x;
                    const double fr2 = x - (double)it, fr1 = 1.0 - fr2;
                    if (it >= 0 && it + 1 <= s.n_pkt) {
                        atomicAdd(qsp + it, dm(inten, fr1));
                        atomicAdd(qsp + it + 1, dm(inten, fr2));
                        added = true;
                    }
                }
            }
        }
    }
    const unsigned b = __ballot_sync(0xffffffffu, added);
    if ((threadIdx.x & 31) == 0 && b) atomicAdd(nbinned, (unsigned long long)__popc(b));
}

}  // namespace

extern "C" int32_t dgpu_powder_npkt(const dgpu_powder *pw) { return dgpu_powder_npkt_host(pw); }

extern "C" int dgpu_powder_complete(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_powder *pw,
                                    const dgpu_opts *opts, double *pow_qsp, dgpu_powder_info *info)
{
    if (!ctx || !cr || !pw || !opts || !pow_qsp) return DGPU_ERR_ARG;
    if (opts->phase != DGPU_PHASE_EXACT64)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "powder complete mode needs EXACT64 phases");
    if (pw->pref_type < DGPU_PREF_NONE || pw->pref_type > DGPU_PREF_MARCH)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "pref_type=%d", pw->pref_type);
    if (pw->pref_type == DGPU_PREF_MARCH && pw->pref_g1 == 0.0)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "March-Dollase g1 must be non-zero");
    PowderPlan plan;
    char msg[256] = {0};
    const int64_t max_points = (int64_t)1 << 26;
    if (pw->slabs < 0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "slabs=%d", pw->slabs);
    int rc = dgpu_powder_plan(cr->rten, pw, opts->ano, pw->slabs ? pw->slabs : 1, max_points, plan, msg,
                              sizeof msg);
    if (rc) return dgpu_set_error(ctx, rc, "%s", msg);
    const int32_t n_pkt = plan.n_pkt;
    if (info) {
        memset(info, 0, sizeof(*info));
        info->n_pkt = n_pkt;
        info->nslab = (int32_t)plan.slabs.size();
        info->rods = (int64_t)plan.rods.size();
        info->rod_points = plan.rod_points;
        info->grid_points = plan.grid_points;
    }
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[8], ctx->stream));
    dgpu_crystal dc;
    rc = dgpu_stage_crystal(ctx, cr, dc);
    if (rc) return rc;
    // four_run_powder: all atoms, no <F>, no lots, four_strucf with is_anis = .false.
    // and cfact from four_formtab, which drops the isotropic term of an
    // anisotropic crystal
    dc.is_anis = 0;
    dgpu_opts op = *opts;
    op.fave = 0.0;
    op.aver_cells = nullptr;
    op.ilots = DGPU_LOT_OFF;
    op.lot_all = 0;
    op.lperiod = 1;
    op.diff_scale = 1.0;
    op.ldbw = (opts->ldbw && !cr->is_anis) ? 1 : 0;

    int64_t maxnp = 1;
    for (const PowderSlab &s : plan.slabs) maxnp = std::max(maxnp, (int64_t)s.nh * s.nk * s.nl);
    const size_t tab_b = plan.tab.size() * sizeof(int32_t);
    const size_t qsp_b = ((size_t)n_pkt + 1) * sizeof(double);
    const size_t off_tab = (qsp_b + 255) / 256 * 256;
    const size_t off_cnt = off_tab + (tab_b + 255) / 256 * 256;
    DGPU_CUDA(ctx, ctx->wbuf.ensure(off_cnt + 256));
    uint8_t *base = ctx->wbuf.as<uint8_t>();
    double *d_qsp = reinterpret_cast<double *>(base);
    int2 *d_tab = reinterpret_cast<int2 *>(base + off_tab);
    unsigned long long *d_cnt = reinterpret_cast<unsigned long long *>(base + off_cnt);
    DGPU_CUDA(ctx, cudaMemsetAsync(d_qsp, 0, qsp_b, ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long), ctx->stream));
    if (tab_b)
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_tab, plan.tab.data(), tab_b, cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, ctx->csf.ensure(maxnp * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->acsf.ensure(maxnp * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->dsi.ensure(maxnp * sizeof(double)));

    BinSpec bs;
    memset(&bs, 0, sizeof(bs));
    for (int a = 0; a < 3; a++) {
        bs.del[a] = pw->hkl_del[a];
        bs.sh[a] = pw->hkl_shift[a];
        bs.pref[a] = pw->pref_hkl[a];
    }
    memcpy(bs.rten, cr->rten, sizeof(bs.rten));
    memcpy(bs.gten, pw->gten, sizeof(bs.gten));
    bs.qmin = pw->qmin;
    bs.qtop = pw->qmax + pw->deltaq;
    bs.deltaq = pw->deltaq;
    bs.l_all = pw->l_all ? 1 : 0;
    bs.n_pkt = n_pkt;
    bs.pref_type = pw->pref_type;
    bs.g1 = pw->pref_g1;
    bs.g2 = pw->pref_g2;

    double kernel_ms = 0.0;
    int64_t pairs = 0;
    int warn = 0;
    for (const PowderSlab &s : plan.slabs) {
        if (opts->cancel && *opts->cancel)
            return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
        dgpu_grid g;
        memset(&g, 0, sizeof(g));
        g.inc[0] = s.nl;
        g.inc[1] = s.nk;
        g.inc[2] = s.nh;
        g.vi[2] = pw->hkl_del[2];                       // axis 0: l
        g.vi[3 + 1] = pw->hkl_del[1];                   // axis 1: k
        g.vi[6 + 0] = pw->hkl_del[0];                   // axis 2: h
        const double e0[3] = {s.h0 * pw->hkl_del[0] + pw->hkl_shift[0], s.k0 * pw->hkl_del[1] + pw->hkl_shift[1],
                              s.l0 * pw->hkl_del[2] + pw->hkl_shift[2]};
        for (int c = 0; c < 4; c++)
            for (int a = 0; a < 3; a++) g.eck[3 * c + a] = e0[a];
        g.eck[3 * 1 + 2] += (s.nl - 1) * pw->hkl_del[2];  // lower right: last l
        g.eck[3 * 2 + 1] += (s.nk - 1) * pw->hkl_del[1];  // upper left: last k
        g.eck[3 * 3 + 0] += (s.nh - 1) * pw->hkl_del[0];  // top left: last h
        dgpu_info fi;
        rc = dgpu_four_run_dev(ctx, &dc, &g, &op, ctx->csf.as<double2>(), ctx->acsf.as<double2>(),
                               ctx->dsi.as<double>(), &fi);
        if (rc < 0) return rc;
        if (rc > 0) warn = rc;
        kernel_ms += fi.kernel_ms;
        pairs += fi.pairs;
        bs.h0 = s.h0;
        bs.nh = s.nh;
        bs.k0 = s.k0;
        bs.nk = s.nk;
        bs.l0 = s.l0;
        bs.nl = s.nl;
        bs.tab = d_tab + s.tab_off;
        const int64_t np = (int64_t)s.nh * s.nk * s.nl;
        k_powder_bin<<<(unsigned)dgpu_cdiv(np, 256), 256, 0, ctx->stream>>>(bs, ctx->csf.as<double2>(), d_qsp, d_cnt);
        DGPU_CUDA(ctx, cudaGetLastError());
    }
    unsigned long long nb = 0;
    DGPU_CUDA(ctx, cudaMemcpyAsync(pow_qsp, d_qsp, qsp_b, cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(&nb, d_cnt, sizeof(nb), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[9], ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    // half-volume correction (powder.f90:2549)
    if (!opts->ano)
        for (int32_t i = 0; i <= n_pkt; i++) pow_qsp[i] *= 2.0;
    if (info) {
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ctx->ev[8], ctx->ev[9]);
        info->total_ms = ms;
        info->kernel_ms = kernel_ms;
        info->pairs = pairs;
        info->binned = (int64_t)nb;
    }
    return warn;
}
