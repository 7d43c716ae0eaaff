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

// origin phase of the atoms for a box shifted by (sl, sk, sh) steps along the
// axes l, k, h: ph0 + sl du + sk dv + sh dw, modulo one turn (exact)
__global__ void k_slab_phase(const uint64_t *__restrict__ ph0, const uint64_t *__restrict__ du,
                             const uint64_t *__restrict__ dv, const uint64_t *__restrict__ dw, int64_t n, int64_t sl,
                             int64_t sk, int64_t sh, uint64_t *__restrict__ out)
{
    const int64_t j = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    out[j] = ph0[j] + (uint64_t)sl * du[j] + (uint64_t)sk * dv[j] + (uint64_t)sh * dw[j];
}

}  // namespace

// The (l, k, h) box of a slab as a grid: axis 0 = l, axis 1 = k, axis 2 = h.
static void slab_grid(const PowderSlab &s, const dgpu_powder *pw, dgpu_grid &g)
{
    memset(&g, 0, sizeof(g));
    g.inc[0] = s.nl;
    g.inc[1] = s.nk;
    g.inc[2] = s.nh;
    g.vi[2] = pw->hkl_del[2];
    g.vi[3 + 1] = pw->hkl_del[1];
    g.vi[6 + 0] = pw->hkl_del[0];
    const double e0[3] = {s.h0 * pw->hkl_del[0] + pw->hkl_shift[0], s.k0 * pw->hkl_del[1] + pw->hkl_shift[1],
                          s.l0 * pw->hkl_del[2] + pw->hkl_shift[2]};
    for (int c = 0; c < 4; c++)
        for (int a = 0; a < 3; a++) g.eck[3 * c + a] = e0[a];
    g.eck[3 * 1 + 2] += (s.nl - 1) * pw->hkl_del[2];  // lower right: last l
    g.eck[3 * 2 + 1] += (s.nk - 1) * pw->hkl_del[1];  // upper left: last k
    g.eck[3 * 3 + 0] += (s.nh - 1) * pw->hkl_del[0];  // top left: last h
}

// The type sums of all slabs in ONE tensor-core launch: the atoms are
// prepared once for the union box, each slab's origin phase is shifted from
// it exactly, and the slabs (same atoms, same column axis l) share one set of
// V images; then per slab the combine and the binning.
static int powder_tc_slabs(dgpu_ctx *ctx, const dgpu_crystal &dc, const dgpu_opts &op, const dgpu_powder *pw,
                           const PowderPlan &plan, BinSpec bs, const int2 *d_tab, double *d_qsp,
                           unsigned long long *d_cnt, double &kernel_ms, int64_t &pairs)
{
    const int nsl = (int)plan.slabs.size();
    if (nsl == 0) return DGPU_OK;
    PowderSlab u = plan.slabs[0];                      // union box
    int32_t h1 = u.h0 + u.nh, k1 = u.k0 + u.nk, l1 = u.l0 + u.nl;
    int64_t maxnp = 1;
    for (const PowderSlab &s : plan.slabs) {
        u.h0 = std::min(u.h0, s.h0);
        u.k0 = std::min(u.k0, s.k0);
        u.l0 = std::min(u.l0, s.l0);
        h1 = std::max(h1, s.h0 + s.nh);
        k1 = std::max(k1, s.k0 + s.nk);
        l1 = std::max(l1, s.l0 + s.nl);
        maxnp = std::max(maxnp, (int64_t)s.nh * s.nk * s.nl);
    }
    u.nh = h1 - u.h0;
    u.nk = k1 - u.k0;
    u.nl = l1 - u.l0;
    dgpu_grid gu;
    slab_grid(u, pw, gu);
    PhaseGeom geo;
    memset(&geo, 0, sizeof(geo));
    geo.mode = DGPU_PHASE_EXACT64;
    for (int k = 0; k < 3; k++) geo.eck[k] = gu.eck[k];
    memcpy(geo.vi, gu.vi, sizeof(geo.vi));
    const int32_t nscat = dc.nscat;
    int64_t ts[2 * 64 + 4];
    FoldSpec nofold = {0, dc.ncatoms, {dc.icc[0], dc.icc[1], dc.icc[2]}, {0, 0, 0}, nullptr};
    int rc = dgpu_prepare_atoms(ctx, dc.pos, dc.iscat, dc.atom_occ, dc.natoms, nscat, geo, nofold, ctx->ph0, ctx->du,
                                ctx->dv, ctx->dw, ctx->w, ts);
    if (rc) return rc;
    const int64_t npad = ts[nscat];
    int64_t natoms = 0;
    for (int t = 0; t < nscat; t++) natoms += ts[nscat + 1 + t];
    DGPU_CUDA(ctx, ctx->slab_ph0.ensure((size_t)nsl * (npad > 0 ? npad : 1) * sizeof(uint64_t)));
    DGPU_CUDA(ctx, ctx->tc_mult.ensure((size_t)TC_MULT_ARRAYS * (npad > 0 ? npad : 1) * sizeof(float2)));
    rc = dgpu_tc_mult_async(ctx, ctx->du.as<uint64_t>(), ctx->dv.as<uint64_t>(), ctx->dw.as<uint64_t>(), npad, npad,
                            ctx->tc_mult.as<float2>());
    if (rc) return rc;
    std::vector<TcInput> in((size_t)nsl);
    for (int i = 0; i < nsl; i++) {
        const PowderSlab &s = plan.slabs[i];
        uint64_t *p = ctx->slab_ph0.as<uint64_t>() + (int64_t)i * npad;
        if (npad > 0)
            k_slab_phase<<<(unsigned)dgpu_cdiv(npad, 256), 256, 0, ctx->stream>>>(
                ctx->ph0.as<uint64_t>(), ctx->du.as<uint64_t>(), ctx->dv.as<uint64_t>(), ctx->dw.as<uint64_t>(), npad,
                s.l0 - u.l0, s.k0 - u.k0, s.h0 - u.h0, p);
        TcInput &t = in[(size_t)i];
        t.ph0 = p;
        t.du = ctx->du.as<uint64_t>();
        t.dv = ctx->dv.as<uint64_t>();
        t.dw = ctx->dw.as<uint64_t>();
        t.w = ctx->w.as<float>();
        t.mult = ctx->tc_mult.as<float2>();
        t.mult_stride = npad;
        t.ts = ts;
        t.ntype = nscat;
        t.box.f[0] = t.box.num[0] = s.nl;
        t.box.f[1] = t.box.num[1] = s.nk;
        t.box.f[2] = t.box.num[2] = s.nh;
        t.axis = 0;                                    // columns along l: every slab the same, images shared
        pairs += natoms * ((int64_t)s.nh * s.nk * s.nl);
    }
    DGPU_CUDA(ctx, cudaGetLastError());
    TcPlan tp;
    const int N = op.tc_tile_n > 0 ? op.tc_tile_n : 64;
    rc = dgpu_tc_plan(ctx, nsl, in.data(), &op, N, 4, tp, ctx->part, ctx->tc_part, &ctx->tc_vimg);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
    rc = dgpu_tc_launch(ctx, tp);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
    rc = dgpu_tc_check(ctx);
    if (rc) return rc;
    float ms = 0.f;
    DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
    kernel_ms += ms;
    // tables, combine and binning, slab by slab
    DGPU_CUDA(ctx, ctx->istl.ensure(maxnp * sizeof(int32_t)));
    DGPU_CUDA(ctx, ctx->cfact.ensure((size_t)nscat * DGPU_NTAB * sizeof(double2)));
    rc = dgpu_formtab_dev(ctx, &dc, &op, ctx->cfact.as<double2>());
    if (rc) return rc;
    for (int i = 0; i < nsl; i++) {
        const PowderSlab &s = plan.slabs[i];
        dgpu_grid g;
        slab_grid(s, pw, g);
        rc = dgpu_stltab_dev(ctx, g.eck, g.vi, g.inc, dc.rten, ctx->istl.as<int32_t>());
        if (rc) return rc;
        FormSpec fs;
        dgpu_fill_formspec(ctx, &dc, &op, &g, fs);
        PartRef ref;
        dgpu_tc_partref(tp.probs[(size_t)i], ctx->part.as<float2>() + tp.part_off[(size_t)i], ref);
        BoxSpec box;
        for (int k = 0; k < 3; k++) box.f[k] = box.num[k] = g.inc[k];
        rc = dgpu_combine(ctx, fs, box, ref, ctx->istl.as<int32_t>(), ctx->cfact.as<double2>(), nullptr,
                          ctx->csf.as<double2>(), ctx->dsi.as<double>(), 1.0);
        if (rc) return rc;
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
    return DGPU_OK;
}

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
    if (cr->natoms < 1) return dgpu_set_error(ctx, DGPU_ERR_NO_ATOMS, "no atoms: no powder pattern will be calculated");
    if (!cr->pos || !cr->iscat || !cr->scat || !cr->occ || !cr->dw)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "crystal arrays missing");
    if (cr->nscat < 1 || cr->nscat > 63)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "nscat=%d outside 1..63", cr->nscat);
    if (opts->power < 0 || opts->power > 5) return dgpu_set_error(ctx, DGPU_ERR_ARG, "power=%d", opts->power);
    if (opts->form != DGPU_FORM_TABLE && opts->form != DGPU_FORM_ANALYTIC)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "form=%d", opts->form);
    // the tensor-core engine evaluates all slabs in one launch, the CUDA-core
    // engine one slab after another
    const bool tc_multi = opts->engine != DGPU_ENGINE_DIRECT && dgpu_tc_available(ctx);
    int rc = dgpu_powder_plan(cr->rten, pw, opts->ano, pw->slabs ? pw->slabs : 8, max_points, plan, msg,
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
    op.filter = DGPU_FILTER_OFF;                 // four_run_powder filters no slab
    op.fave = 0.0;
    op.aver_cells = nullptr;
    op.ilots = DGPU_LOT_OFF;
    op.lot_all = 0;
    op.lperiod = 1;
    op.diff_scale = 1.0;
    op.ldbw = (opts->ldbw && !cr->is_anis) ? 1 : 0;
    op.discamb = nullptr;           // the powder run has ldiscamb = .false. (fourier_sup.f90:507)

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
    if (opts->cancel && *opts->cancel) return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
    if (tc_multi) {
        rc = powder_tc_slabs(ctx, dc, op, pw, plan, bs, d_tab, d_qsp, d_cnt, kernel_ms, pairs);
        if (rc) return rc;
    }
    for (const PowderSlab &s : plan.slabs) {
        if (tc_multi) break;
        if (opts->cancel && *opts->cancel)
            return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
        dgpu_grid g;
        slab_grid(s, pw, g);
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
