// C-ABI entry points and the four_run orchestration on the device.
//
// dgpu_four_run replaces four_run (discus/prog/fourier_sup.f90:11-323) for
// the independent atom model.  The order of work follows it:
// four_layer/fourier_lmn (:71,:82), four_stltab (:84), four_formtab (:120),
// four_nanis (:131), four_test_friedel (:132), four_aver (:134), the loop
// over lots (:136-257) and over atom types or (type, ADP type) groups
// (:195-244), csf -= acsf and dsi += |csf|^2 (:250-254), four_apply_friedel
// (:256, once after the lots: it only copies the computed half), the lot
// normalisation (:273-277), scaling (:281-282) and four_qinfo (:294).
#include <math.h>
#include <stdarg.h>
#include <stdlib.h>

#include <vector>

#include "dgpu_internal.h"
#include "dgpu_lots.h"

int dgpu_set_error(dgpu_ctx *ctx, int code, const char *fmt, ...)
{
    if (ctx) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(ctx->err, sizeof(ctx->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

extern "C" const char *dgpu_last_error(const dgpu_ctx *ctx) { return ctx ? ctx->err : "no context"; }

extern "C" void dgpu_default_opts(dgpu_opts *o)
{
    memset(o, 0, sizeof(*o));
    o->lxray = 1;
    o->power = 4;
    o->ano = 0;
    o->ldbw = 0;
    o->friedel = 1;
    o->fave = 0.0;
    o->aver_cells = nullptr;
    o->diff_scale = 1.0;
    o->phase = DGPU_PHASE_EXACT64;
    o->form = DGPU_FORM_TABLE;
    o->engine = DGPU_ENGINE_AUTO;
    o->split = DGPU_SPLIT_F16;
    o->cancel = nullptr;
    o->ilots = DGPU_LOT_OFF;
    o->nlots = 1;
    for (int k = 0; k < 3; k++) o->ls_xyz[k] = 5;
    o->lot_all = 0;
    o->lperiod = 1;
    o->lot_origins = nullptr;
    o->tc_vimg = 0;
    o->tc_wait_us = 0;
    o->filter = DGPU_FILTER_OFF;
    o->filter_width = 4;
    o->filter_damp = 0.5;
    o->filter_scale = 1.0;
}

extern "C" int dgpu_ctx_create(int device, dgpu_ctx **out)
{
    if (!out) return DGPU_ERR_ARG;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return DGPU_ERR_CUDA;
    if (device < 0 || device >= ndev) return DGPU_ERR_ARG;
    dgpu_ctx *c = new dgpu_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess) { delete c; return DGPU_ERR_CUDA; }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) { delete c; return DGPU_ERR_CUDA; }
    c->nsm = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) { delete c; return DGPU_ERR_CUDA; }
    for (int i = 0; i < DGPU_NEV; i++)
        if (cudaEventCreate(&c->ev[i]) != cudaSuccess) { delete c; return DGPU_ERR_CUDA; }
    if (dgpu_tc_init(c) != DGPU_OK) {
        dgpu_ctx_destroy(c);
        return DGPU_ERR_CUDA;
    }
    *out = c;
    return DGPU_OK;
}

extern "C" int dgpu_ctx_destroy(dgpu_ctx *c)
{
    if (!c) return DGPU_OK;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    dgpu_batch_free(c);
    DevBuf *bufs[] = {&c->pos, &c->iscat, &c->aocc, &c->sel, &c->counts, &c->ph0, &c->du,
                      &c->dv, &c->dw, &c->w, &c->aph0, &c->adu, &c->adv, &c->adw, &c->aw, &c->istl,
                      &c->cfact, &c->part, &c->apart, &c->lat, &c->csf, &c->acsf, &c->dsi, &c->stats,
                      &c->flag, &c->tc_part, &c->tc_work, &c->tc_mult, &c->tc_vimg, &c->adj_qimg,
                      &c->adj_items, &c->gq, &c->gpart, &c->grad, &c->batch_desc, &c->batch_aux,
                      &c->ianis, &c->geff, &c->ghist, &c->lpos, &c->ltype, &c->locc, &c->lplan, &c->lfac,
                      &c->wbuf, &c->acc_csf, &c->acc_dsi, &c->slab_ph0, &c->rlist, &c->rsum, &c->tc_tab, &c->ph_tab, &c->filt, &c->filt_slice,
                      &c->aidx, &c->aaidx, &c->isymb, &c->dtab, &c->lorig};
    for (DevBuf *b : bufs) b->release();
    c->stage.release();
    for (cudaEvent_t e : c->run_ev) cudaEventDestroy(e);
    delete c->fs_main;
    delete c->fs_type;
    delete c->lot_keep;
    for (int i = 0; i < DGPU_NEV; i++)
        if (c->ev[i]) cudaEventDestroy(c->ev[i]);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return DGPU_OK;
}

extern "C" int dgpu_fourier_lmn(const double eck[12], const double vi[9], const int32_t inc[3],
                                int32_t lmn[6], double off_shift[9])
{
    if (!eck || !vi || !inc || !lmn || !off_shift) return DGPU_ERR_ARG;
    return dgpu_lmn_host(eck, vi, inc, lmn, off_shift);
}

// ---------------------------------------------------------------------------
static int check_inputs(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op)
{
    if (!ctx || !cr || !g || !op) return DGPU_ERR_ARG;
    if (cr->natoms < 1) return dgpu_set_error(ctx, DGPU_ERR_NO_ATOMS, "no atoms: no fourier will be calculated");
    if (!cr->pos || !cr->iscat || !cr->scat || !cr->occ || !cr->dw)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "crystal arrays missing");
    if (cr->nscat < 1 || cr->nscat > 63)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "nscat=%d outside 1..63", cr->nscat);
    for (int k = 0; k < 3; k++)
        if (g->inc[k] < 1) return dgpu_set_error(ctx, DGPU_ERR_ARG, "inc(%d)=%d", k + 1, g->inc[k]);
    if (op->power < 0 || op->power > 5) return dgpu_set_error(ctx, DGPU_ERR_ARG, "power=%d", op->power);
    if (op->phase != DGPU_PHASE_REF22 && op->phase != DGPU_PHASE_EXACT64)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "phase=%d", op->phase);
    if (op->form != DGPU_FORM_TABLE && op->form != DGPU_FORM_ANALYTIC)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "form=%d", op->form);
    if (op->fave > 0.0 && op->fave < 1.0 && !op->aver_cells)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "0<fave<1 needs the caller's cell selection");
    if (op->diff_scale < 0.0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "diff_scale<0");
    if (cr->is_anis && (cr->nanis < 1 || !cr->ianis || !cr->anis_full))
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "anisotropic crystal without nanis/ianis/anis_full");
    if (const dgpu_discamb *dc = op->discamb) {
        if (!dc->nsymm || !dc->isymm || !dc->form_tsc || !cr->isym)
            return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB needs nsymm, isymm, form_tsc and the atoms' isym");
        for (int k = 0; k < 3; k++)
            if (dc->maxhkl[k] < 0 || dc->maxhkl[k] > 4096)
                return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB maxhkl(%d)=%d", k + 1, dc->maxhkl[k]);
        for (int t = 0; t < cr->nscat; t++)
            if (dc->nsymm[t] < 0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB nsymm(%d)<0", t + 1);
        if (op->fave != 0.0)
            return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "DISCAMB form factors with <F> subtraction");
        if (op->ldbw && (cr->nanis < 1 || !cr->ianis || !cr->anis_full))
            return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB with temp use needs nanis/ianis/anis_full");
    }
    // lots: the checks of the lots command (fourier.f90:490-497) and the origins' range
    const bool lots = dgpu_lots_on(op);
    if (op->ilots != 0 && op->ilots != DGPU_LOT_OFF && !lots)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "ilots=%d", op->ilots);
    if (lots || !op->lperiod)
        for (int k = 0; k < 3; k++)
            if (op->ls_xyz[k] < 1 || op->ls_xyz[k] > cr->icc[k])
                return dgpu_set_error(ctx, DGPU_ERR_ARG, "ls_xyz(%d)=%d outside 1..icc", k + 1, op->ls_xyz[k]);
    if (lots && !op->lot_all) {
        if (op->nlots < 1 || !op->lot_origins)
            return dgpu_set_error(ctx, DGPU_ERR_ARG, "lots need nlots>0 origins (or lot_all)");
        int32_t cs[3];
        dgpu_csize(cr, op, cs);
        for (int64_t l = 0; l < op->nlots; l++)
            for (int k = 0; k < 3; k++)
                if (op->lot_origins[3 * l + k] < 1 || op->lot_origins[3 * l + k] > cs[k])
                    return dgpu_set_error(ctx, DGPU_ERR_ARG, "lot %lld origin(%d)=%d outside 1..%d", (long long)l + 1,
                                          k + 1, op->lot_origins[3 * l + k], cs[k]);
    }
    return DGPU_OK;
}

int dgpu_fill_formspec(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, const dgpu_grid *g,
                       FormSpec &fs)
{
    memset(&fs, 0, sizeof(fs));
    fs.mode = op->form;
    fs.nscat = cr->nscat;
    fs.lxray = op->lxray;
    fs.power = op->power;
    fs.ano = op->ano;
    fs.ldbw = op->ldbw && !cr->is_anis;
    fs.ngroup = cr->nscat;
    for (int t = 1; t <= cr->nscat; t++) fs.gtype[t] = t;
    for (int t = 0; t <= cr->nscat; t++) {
        for (int i = 0; i < 11; i++) fs.scat[11 * t + i] = cr->scat[11 * t + i];
        fs.occ[t] = cr->occ[t];
        fs.dw[t] = cr->dw[t];
        fs.delfr[t] = cr->delfr ? cr->delfr[t] : 0.0;
        fs.delfi[t] = cr->delfi ? cr->delfi[t] : 0.0;
    }
    memcpy(fs.rten, cr->rten, sizeof(fs.rten));
    for (int k = 0; k < 3; k++) fs.eck[k] = g->eck[k];
    memcpy(fs.vi, g->vi, sizeof(fs.vi));
    (void)ctx;
    return DGPU_OK;
}

// four_test_friedel (fourier_sup.f90:3645-3722)
int dgpu_friedel_test(const dgpu_grid *g, const dgpu_opts *op, int32_t fnum[3])
{
    const double eps = (double)1.0e-6f;
    for (int k = 0; k < 3; k++) fnum[k] = g->inc[k];
    if (!op->friedel || op->ano) return 0;
    if (!(fnum[0] % 2 && fnum[1] % 2 && fnum[2] % 2)) return 0;
    for (int k = 0; k < 3; k++) {
        double rut = g->eck[k] + g->vi[k] * (fnum[0] - 1) + g->vi[3 + k] * (fnum[1] - 1) + g->vi[6 + k] * (fnum[2] - 1);
        if (!(fabs(g->eck[k] + rut) < eps)) return 0;
    }
    for (int a = 0; a < 3; a++)
        if (fnum[a] > 1) {
            fnum[a] = (fnum[a] + 1) / 2;
            return a + 1;
        }
    return 0;
}

static bool cancelled(const dgpu_opts *op) { return op->cancel && *op->cancel; }

static int pick_engine(dgpu_ctx *ctx, const dgpu_opts *op)
{
    if (op->engine == DGPU_ENGINE_DIRECT) return DGPU_ENGINE_DIRECT;
    bool tc_ok = op->phase == DGPU_PHASE_EXACT64 && dgpu_tc_available(ctx);
    if (op->engine == DGPU_ENGINE_TC) return tc_ok ? DGPU_ENGINE_TC : -1;
    return tc_ok ? DGPU_ENGINE_TC : DGPU_ENGINE_DIRECT;
}

static int engine_sums(dgpu_ctx *ctx, int engine, DevBuf &ph0, DevBuf &du, DevBuf &dv, DevBuf &dw, DevBuf &w,
                       const int64_t *ts, int32_t ntype, const dgpu_opts *op, const BoxSpec &box, DevBuf &part,
                       PartRef *ref)
{
    memset(ref, 0, sizeof(*ref));
    if (engine == DGPU_ENGINE_TC)
        return dgpu_tc_sums(ctx, ph0.as<uint64_t>(), du.as<uint64_t>(), dv.as<uint64_t>(), dw.as<uint64_t>(),
                            w.as<float>(), ts, ntype, box, op, part, ref);
    int32_t nslice = 1;
    int rc = dgpu_direct_sums(ctx, ph0.as<uint64_t>(), du.as<uint64_t>(), dv.as<uint64_t>(), dw.as<uint64_t>(),
                              w.as<float>(), ts, ntype, op->phase == DGPU_PHASE_REF22, box, part, &nslice);
    ref->p = part.p;
    ref->nslice = nslice;
    return rc;
}

// The lots' engine launches (fourier_sup.f90:136-257), a chunk of lots per
// launch, in batches of chunks: every chunk of a batch is gathered and its
// (lot, group) types counted first, so that one host wait yields all their
// type ranges; scatter, engine launch and lot combine of the chunks then
// follow one another on the stream with no host wait between them (the
// tensor-core engine in its deferred mode, its error flag read once per
// batch).
#define LOT_BATCH_SLOTS ((int64_t)1 << 24)     // lot atom slots gathered per batch

namespace {
struct LotChunk {
    int64_t lot0, slot0, m;
    int32_t nl, ntype;
    size_t reg;                        // offset of the chunk's count region
    int64_t ts[2 * 64 + 4];
};
struct DeferGuard {
    dgpu_ctx *c;
    explicit DeferGuard(dgpu_ctx *x) : c(x) { c->tc_defer = 1; }
    ~DeferGuard() { c->tc_defer = 0; }
};
}  // namespace

static int lots_sums(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, const LotPlan &lp, int32_t ngroup,
                     const int32_t *eiscat, const PhaseGeom &geo, const BoxSpec &box, int engine, int64_t np,
                     const double2 *acsf_in, double2 *d_csf, double *d_dsi, int64_t *pairs, float *kernel_ms)
{
    const int64_t per_lot = lp.geo.per_lot;
    const int64_t nchunk = dgpu_cdiv(lp.nlots, lp.per_chunk);
    const int64_t chunk_slots = (int64_t)lp.per_chunk * per_lot;
    int64_t batch_slots = LOT_BATCH_SLOTS;
    if (const char *e = getenv("DGPU_LOT_BATCH_SLOTS")) {      // smaller batches (results are the same)
        const long long v = atoll(e);
        if (v > 0) batch_slots = v;
    }
    const int64_t cpb = chunk_slots > 0 && batch_slots / chunk_slots > 1 ? batch_slots / chunk_slots : 1;
    const FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
    int rc;
    for (int64_t c0 = 0; c0 < nchunk; c0 += cpb) {
        const int64_t nc = nchunk - c0 < cpb ? nchunk - c0 : cpb;
        std::vector<LotChunk> ch((size_t)nc);
        int64_t slots = 0;
        size_t rbytes = 0;
        for (int64_t i = 0; i < nc; i++) {
            LotChunk &k = ch[(size_t)i];
            k.lot0 = (c0 + i) * lp.per_chunk;
            k.nl = (int32_t)(lp.nlots - k.lot0 < lp.per_chunk ? lp.nlots - k.lot0 : lp.per_chunk);
            k.ntype = k.nl * ngroup;
            k.m = (int64_t)k.nl * per_lot;
            k.slot0 = slots;
            slots += k.m;
            k.reg = rbytes;
            rbytes += dgpu_prepare_region_bytes(k.m, k.ntype);
        }
        const size_t ns = (size_t)(slots > 0 ? slots : 1);
        DGPU_CUDA(ctx, ctx->lpos.ensure(ns * 3 * sizeof(double)));
        DGPU_CUDA(ctx, ctx->ltype.ensure(ns * sizeof(int32_t)));
        DGPU_CUDA(ctx, ctx->locc.ensure(ns * sizeof(float)));
        DGPU_CUDA(ctx, ctx->counts.ensure(rbytes));
        // type ranges land in pinned memory, so that their copies do not wait for the stream one by one
        const size_t tsn = sizeof(LotChunk::ts) / sizeof(int64_t);
        int64_t *hts = static_cast<int64_t *>(ctx->stage.take((size_t)nc * tsn * sizeof(int64_t)));
        if (!hts) return dgpu_set_error(ctx, DGPU_ERR_NOMEM, "pinned staging memory");
        for (int64_t i = 0; i < nc; i++) {
            const LotChunk &k = ch[(size_t)i];
            int64_t m = 0;
            rc = dgpu_lot_gather(ctx, lp, k.lot0, k.nl, cr->pos, eiscat, cr->atom_occ, k.slot0, &m);
            if (rc) return rc;
            const PrepRegion r = dgpu_prepare_region((char *)ctx->counts.p + k.reg, k.m, k.ntype);
            rc = dgpu_prepare_count(ctx, ctx->ltype.as<int32_t>() + k.slot0, k.m, k.ntype, nofold, r);
            if (rc) return rc;
            DGPU_CUDA(ctx, cudaMemcpyAsync(hts + i * tsn, r.d_ts, (2 * k.ntype + 1) * sizeof(int64_t),
                                           cudaMemcpyDeviceToHost, ctx->stream));
        }
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));        // the type ranges of every chunk
        for (int64_t i = 0; i < nc; i++)
            memcpy(ch[(size_t)i].ts, hts + i * tsn, (2 * ch[(size_t)i].ntype + 1) * sizeof(int64_t));
        ctx->stage.reset();
        // the largest chunk sizes the atom buffers before the run
        int64_t most = 1;
        for (const LotChunk &k : ch) most = k.ts[k.ntype] > most ? k.ts[k.ntype] : most;
        DGPU_CUDA(ctx, ctx->ph0.ensure((size_t)most * 8));
        DGPU_CUDA(ctx, ctx->du.ensure((size_t)most * 8));
        DGPU_CUDA(ctx, ctx->dv.ensure((size_t)most * 8));
        DGPU_CUDA(ctx, ctx->dw.ensure((size_t)most * 8));
        DGPU_CUDA(ctx, ctx->w.ensure((size_t)most * 4));
        DGPU_CUDA(ctx, ctx->aidx.ensure((size_t)most * 4));
        DGPU_CUDA(ctx, ctx->flag.ensure(64));
        DGPU_CUDA(ctx, cudaMemsetAsync(ctx->flag.as<int32_t>() + 8, 0, sizeof(int32_t), ctx->stream));
        while (ctx->run_ev.size() < 2 * (size_t)nc) {
            cudaEvent_t e;
            DGPU_CUDA(ctx, cudaEventCreate(&e));
            ctx->run_ev.push_back(e);
        }
        {
            DeferGuard defer(ctx);
            for (int64_t i = 0; i < nc; i++) {
                const LotChunk &k = ch[(size_t)i];
                const PrepRegion r = dgpu_prepare_region((char *)ctx->counts.p + k.reg, k.m, k.ntype);
                rc = dgpu_prepare_scatter(ctx, ctx->lpos.as<double>() + 3 * k.slot0, ctx->ltype.as<int32_t>() + k.slot0,
                                          cr->atom_occ ? ctx->locc.as<float>() + k.slot0 : nullptr, k.m, k.ntype, geo,
                                          nofold, r, k.ts[k.ntype], ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w);
                if (rc) return rc;
                int64_t nat = 0;
                for (int t = 0; t < k.ntype; t++) nat += k.ts[k.ntype + 1 + t];
                *pairs += nat * np;
                PartRef pref;
                memset(&pref, 0, sizeof(pref));
                DGPU_CUDA(ctx, cudaEventRecord(ctx->run_ev[2 * i], ctx->stream));
                if (nat > 0) {
                    rc = engine_sums(ctx, engine, ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w, k.ts, k.ntype, op, box,
                                     ctx->part, &pref);
                    if (rc) return rc;
                }
                DGPU_CUDA(ctx, cudaEventRecord(ctx->run_ev[2 * i + 1], ctx->stream));
                const int32_t last = k.lot0 + k.nl == lp.nlots ? k.nl - 1 : -1;
                rc = dgpu_lot_combine(ctx, ngroup, k.nl, box, nat > 0 ? &pref : nullptr, ctx->lfac.as<double2>(),
                                      acsf_in, d_csf, d_dsi, last);
                if (rc) return rc;
                if (cancelled(op)) return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
            }
        }
        rc = dgpu_tc_check(ctx);                                    // waits for the batch
        if (rc) return rc;
        for (int64_t i = 0; i < nc; i++) {
            float ms = 0.f;
            DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->run_ev[2 * i], ctx->run_ev[2 * i + 1]));
            *kernel_ms += ms;
        }
    }
    return DGPU_OK;
}

// Adjoint of the lots (fourier_sup.f90:136-277): dsi = ds dnorm sum_L |F_L|^2
// with F_L the lot's sum (atoms shifted by the lot origin) less <F>, so each
// lot contributes per-point weights Q_L,g = 2 ds dnorm G conj(F_L) fac_g to
// the atoms it holds.  The lots are taken chunk by chunk as in the forward
// pass (gather, type ranges, scatter, type sums of the forward's engine --
// F_L is recomputed, not stored), then Q of the chunk's (lot, group) types
// and the per-atom sums, which add into the gradient of each slot's source
// atom (atomically: an atom sits in several lots).  fsum (box points) gets
// sum_L F_L for the <F> term.  d_g: dchi2/dI on the full grid.
int dgpu_lots_adjoint(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op,
                      const BoxSpec &box, int32_t idim, const double *d_g, double *gpos, double *gocc, double2 *fsum)
{
    const LotKeep &K = *ctx->lot_keep;
    const LotPlan &lp = K.lp;
    const int64_t per_lot = lp.geo.per_lot;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    const FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
    const double scale = 2.0 * op->diff_scale * K.dnorm;
    const double2 *acsf = op->fave > 0.0 ? ctx->acsf.as<double2>() : nullptr;
    int rc;
    for (int64_t lot0 = 0; lot0 < lp.nlots; lot0 += lp.per_chunk) {
        const int32_t nl = (int32_t)(lp.nlots - lot0 < lp.per_chunk ? lp.nlots - lot0 : lp.per_chunk);
        const int32_t ntype = nl * K.ngroup;
        const int64_t m = (int64_t)nl * per_lot;
        if (m == 0) continue;
        DGPU_CUDA(ctx, ctx->lpos.ensure((size_t)m * 3 * sizeof(double)));
        DGPU_CUDA(ctx, ctx->ltype.ensure((size_t)m * sizeof(int32_t)));
        DGPU_CUDA(ctx, ctx->locc.ensure((size_t)m * sizeof(float)));
        DGPU_CUDA(ctx, ctx->lorig.ensure((size_t)m * sizeof(int32_t)));
        int64_t got = 0;
        rc = dgpu_lot_gather(ctx, lp, lot0, nl, cr->pos, K.eiscat, cr->atom_occ, 0, &got, ctx->lorig.as<int32_t>());
        if (rc) return rc;
        int64_t ts[2 * 64 + 4];
        rc = dgpu_prepare_atoms(ctx, ctx->lpos.as<double>(), ctx->ltype.as<int32_t>(),
                                cr->atom_occ ? ctx->locc.as<float>() : nullptr, m, ntype, K.geo, nofold, ctx->ph0,
                                ctx->du, ctx->dv, ctx->dw, ctx->w, ts);
        if (rc) return rc;
        if (ts[ntype] == 0) continue;
        PartRef pref;
        rc = engine_sums(ctx, K.engine, ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w, ts, ntype, op, box, ctx->part,
                         &pref);
        if (rc) return rc;
        DGPU_CUDA(ctx, ctx->gpart.ensure((size_t)ntype * nb * sizeof(float2)));
        rc = dgpu_lot_adj_q(ctx, K.ngroup, nl, box, idim, pref, ctx->lfac.as<double2>(), acsf, d_g, scale,
                            ctx->gpart.as<float2>(), fsum);
        if (rc) return rc;
        // slot -> source atom
        rc = dgpu_compose_index(ctx, ctx->aidx.as<int32_t>(), ctx->lorig.as<int32_t>(), ts[ntype]);
        if (rc) return rc;
        if (K.engine == DGPU_ENGINE_TC) {
            rc = dgpu_adjtc_sums(ctx, box, grid, ntype, ts, ctx->ph0.as<uint64_t>(), ctx->du.as<uint64_t>(),
                                 ctx->dv.as<uint64_t>(), ctx->dw.as<uint64_t>(), ctx->w.as<float>(),
                                 ctx->aidx.as<int32_t>(), ctx->gpart.as<float2>(), gpos, gocc);
        } else {
            rc = dgpu_adj_atom_sums(ctx, box, grid, ntype, ts, ctx->ph0.as<uint64_t>(), ctx->du.as<uint64_t>(),
                                    ctx->dv.as<uint64_t>(), ctx->dw.as<uint64_t>(), ctx->w.as<float>(),
                                    ctx->aidx.as<int32_t>(), ctx->gpart.as<float2>(), gpos, gocc, true);
        }
        if (rc) return rc;
        if (cancelled(op)) return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
    }
    return DGPU_OK;
}

// DISCAMB: the caller's tables into device memory, and a check that every
// point of the box maps into them (nint is monotonic and h linear over the
// box, so its corners bound the indices)
static int discamb_tables(dgpu_ctx *ctx, const dgpu_discamb *dc, int32_t nscat, const FormSpec &fs,
                          const BoxSpec &box, FormSpec &fsm)
{
    int64_t ntab = 0, tsize = 1;
    for (int t = 0; t < nscat; t++) ntab += dc->nsymm[t];
    for (int k = 0; k < 3; k++) tsize *= 2 * (int64_t)dc->maxhkl[k] + 1;
    if (ntab < 1 || ntab > 63 * (DGPU_DISC_MAXSYM + 1))
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB: %lld tables", (long long)ntab);
    for (int c = 0; c < 8; c++) {
        const int64_t ijl[3] = {(c & 1) ? box.f[0] - 1 : 0, (c & 2) ? box.f[1] - 1 : 0, (c & 4) ? box.f[2] - 1 : 0};
        for (int k = 0; k < 3; k++) {
            const double h = fs.eck[k] + fs.vi[k] * (double)ijl[0] + fs.vi[3 + k] * (double)ijl[1] +
                             fs.vi[6 + k] * (double)ijl[2];
            if (fabs(round(h)) > dc->maxhkl[k])
                return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB: h(%d)=%g outside the table's +-%d", k + 1, h,
                                      dc->maxhkl[k]);
        }
    }
    const size_t bytes = (size_t)(ntab * tsize) * sizeof(double2);
    DGPU_CUDA(ctx, ctx->dtab.ensure(bytes));
    DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->dtab.p, dc->form_tsc, bytes, cudaMemcpyHostToDevice, ctx->stream));
    fsm.disc = 1;
    fsm.dntab = (int32_t)ntab;
    for (int k = 0; k < 3; k++) fsm.dmax[k] = dc->maxhkl[k];
    fsm.dtab = ctx->dtab.as<double2>();
    return DGPU_OK;
}

// The whole path with device-resident crystal arrays and outputs.
int dgpu_four_run_dev(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op,
                        double2 *d_csf, double2 *d_acsf, double *d_dsi, dgpu_info *info)
{
    int rc = check_inputs(ctx, cr, g, op);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[0], ctx->stream));
    const int32_t *num = g->inc;
    const int64_t np = (int64_t)num[0] * num[1] * num[2];

    PhaseGeom geo;
    memset(&geo, 0, sizeof(geo));
    geo.mode = op->phase;
    rc = dgpu_lmn_host(g->eck, g->vi, g->inc, geo.lmn, geo.off);
    if (rc) return dgpu_set_error(ctx, rc, rc == DGPU_ERR_ZERO_INC ? "zero increment vector with inc>1"
                                                                   : "fourier_lmn failed");
    for (int k = 0; k < 3; k++) geo.eck[k] = g->eck[k];
    memcpy(geo.vi, g->vi, sizeof(geo.vi));

    int engine = pick_engine(ctx, op);
    if (engine < 0)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "tensor-core engine needs EXACT64 phases on sm_100+");

    // tables
    DGPU_CUDA(ctx, ctx->istl.ensure(np * sizeof(int32_t)));
    rc = dgpu_stltab_dev(ctx, g->eck, g->vi, num, cr->rten, ctx->istl.as<int32_t>());
    if (rc) return rc;
    DGPU_CUDA(ctx, ctx->cfact.ensure((size_t)cr->nscat * DGPU_NTAB * sizeof(double2)));
    rc = dgpu_formtab_dev(ctx, cr, op, ctx->cfact.as<double2>());
    if (rc) return rc;

    int32_t fnum[3];
    int idim = dgpu_friedel_test(g, op, fnum);
    BoxSpec box;
    for (int k = 0; k < 3; k++) { box.f[k] = fnum[k]; box.num[k] = num[k]; }
    FormSpec fs;
    dgpu_fill_formspec(ctx, cr, op, g, fs);

    DGPU_CUDA(ctx, cudaMemsetAsync(d_csf, 0, np * sizeof(double2), ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(d_dsi, 0, np * sizeof(double), ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(d_acsf, 0, np * sizeof(double2), ctx->stream));

    // partial-sum groups: the types, or the (type, ADP type) pairs (four_nanis)
    FormSpec fsm = fs;
    const int32_t *eiscat = cr->iscat;
    int32_t ngroup = cr->nscat;
    if (op->discamb) {
        rc = discamb_tables(ctx, op->discamb, cr->nscat, fs, box, fsm);
        if (rc) return rc;
    }
    if (cr->is_anis || op->discamb) {
        rc = dgpu_anis_groups(ctx, cr, op, fsm, &ngroup);
        if (rc) return rc;
        eiscat = ctx->geff.as<int32_t>();
    }
    const bool lots = dgpu_lots_on(op);
    int32_t cs[3];
    dgpu_csize(cr, op, cs);
    LotPlan lp;
    if (lots) {
        rc = dgpu_lot_plan(ctx, cr, op, ngroup, lp);
        if (rc) return rc;
    }

    int warn = 0;
    int32_t ncell = 0;
    ctx->aver.on = 0;
    delete ctx->lot_keep;
    ctx->lot_keep = nullptr;
    int64_t pairs_aver = 0, pairs = 0, refined = 0;
    float kernel_ms = 0.f;
    int64_t ts[2 * 64 + 4];
    // <F> of a box lattice in closed form: kept for the refinement of the
    // points where it cancels most of F
    int64_t ts_fold[2 * 64 + 4];
    bool aver_closed = false;
    int32_t alat_n[3] = {0, 0, 0};
    double alat_d[3] = {0, 0, 0}, anorm = 0.0;

    // ---- <F> (four_aver): cells drawn over csize, lattice of the crystal or of a lot ----
    if (op->fave < 0.0) {
        // ran1 <= fave never holds: no cell, <F> = 0 and the +1 warning (fourier_sup.f90:1235-1241,1323-1331)
        warn = DGPU_WARN_NO_CELL;
        dgpu_set_error(ctx, DGPU_WARN_NO_CELL, "no unit cell selected for <F>");
    } else if (op->fave != 0.0) {
        const int64_t ncells = (int64_t)cr->icc[0] * cr->icc[1] * cr->icc[2];
        FoldSpec fold = {1, cr->ncatoms, {cr->icc[0], cr->icc[1], cr->icc[2]},
                         {cr->dim0[0], cr->dim0[1], cr->dim0[2]}, nullptr};
        const bool whole = cs[0] == cr->icc[0] && cs[1] == cr->icc[1] && cs[2] == cr->icc[2];
        if (op->fave < 1.0 || !whole) {
            std::vector<uint8_t> sel((size_t)ncells, 0);
            for (int32_t kk = 0; kk < cs[2]; kk++)
                for (int32_t jj = 0; jj < cs[1]; jj++)
                    for (int32_t ii = 0; ii < cs[0]; ii++) {
                        const int64_t s = ii + (int64_t)cs[0] * (jj + (int64_t)cs[1] * kk);
                        const bool on = op->fave >= 1.0 || op->aver_cells[s] != 0;
                        sel[ii + (int64_t)cr->icc[0] * (jj + (int64_t)cr->icc[1] * kk)] = on ? 1 : 0;
                        ncell += on ? 1 : 0;
                    }
            DGPU_CUDA(ctx, ctx->sel.ensure(ncells));
            DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->sel.p, sel.data(), ncells, cudaMemcpyHostToDevice, ctx->stream));
            DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));      // sel is a host temporary
            fold.sel = ctx->sel.as<uint8_t>();
        } else {
            ncell = (int32_t)ncells;
        }
        rc = dgpu_prepare_atoms(ctx, cr->pos, cr->iscat, cr->atom_occ, cr->natoms, cr->nscat, geo, fold,
                                ctx->aph0, ctx->adu, ctx->adv, ctx->adw, ctx->aw, ts, &ctx->aaidx);
        if (rc) return rc;
        PartRef aref;
        DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
        rc = engine_sums(ctx, engine, ctx->aph0, ctx->adu, ctx->adv, ctx->adw, ctx->aw, ts, cr->nscat, op, box,
                         ctx->apart, &aref);
        if (rc) return rc;
        memcpy(ts_fold, ts, sizeof(int64_t) * (2 * cr->nscat + 1));
        for (int t = 0; t < cr->nscat; t++) pairs_aver += ts[cr->nscat + 1 + t] * np;
        // four_getav (fourier_sup.f90:2440-2510) + four_strucf(0, ...) on the full num:
        // a box (all cells at dim0, or a box lot at 0) has a closed form in EXACT64
        int32_t lat_n[3];
        double lat_d[3];
        for (int k = 0; k < 3; k++) {
            lat_n[k] = lots ? op->ls_xyz[k] : cr->icc[k];
            lat_d[k] = lots ? 0.0 : cr->dim0[k];
        }
        int32_t lat_nslice = 1;
        const int32_t closed = op->phase == DGPU_PHASE_EXACT64 && op->ilots != DGPU_LOT_ELI;
        if (!closed) {
            int64_t lts[2 * 1 + 4];
            int64_t nlat;
            if (op->ilots == DGPU_LOT_ELI) {
                nlat = (int64_t)lp.shape.size() / 3;
                std::vector<double> pts((size_t)nlat * 3);
                std::vector<int32_t> ones((size_t)nlat, 1);
                for (int64_t m = 0; m < 3 * nlat; m++) pts[m] = (double)lp.shape[m];
                DGPU_CUDA(ctx, ctx->lpos.ensure((size_t)nlat * 3 * sizeof(double)));
                DGPU_CUDA(ctx, ctx->ltype.ensure((size_t)nlat * sizeof(int32_t)));
                DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->lpos.p, pts.data(), pts.size() * sizeof(double),
                                               cudaMemcpyHostToDevice, ctx->stream));
                DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->ltype.p, ones.data(), ones.size() * sizeof(int32_t),
                                               cudaMemcpyHostToDevice, ctx->stream));
                DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));  // host temporaries
                FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
                rc = dgpu_prepare_atoms(ctx, ctx->lpos.as<double>(), ctx->ltype.as<int32_t>(), nullptr, nlat, 1, geo,
                                        nofold, ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w, lts);
                if (rc) return rc;
            } else {
                nlat = (int64_t)lat_n[0] * lat_n[1] * lat_n[2];
                rc = dgpu_prepare_lattice(ctx, lat_n, lat_d, geo, ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w);
                if (rc) return rc;
                lts[0] = 0;
                lts[1] = nlat;
            }
            BoxSpec full;
            for (int k = 0; k < 3; k++) { full.f[k] = num[k]; full.num[k] = num[k]; }
            rc = dgpu_direct_sums(ctx, ctx->ph0.as<uint64_t>(), ctx->du.as<uint64_t>(), ctx->dv.as<uint64_t>(),
                                  ctx->dw.as<uint64_t>(), ctx->w.as<float>(), lts, 1, op->phase == DGPU_PHASE_REF22,
                                  full, ctx->lat, &lat_nslice);
            if (rc) return rc;
            pairs_aver += nlat * np;
        }
        DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
        double norm = 0.0;
        if (ncell > 0) norm = 1.0 / ncell;
        else {
            warn = DGPU_WARN_NO_CELL;
            dgpu_set_error(ctx, DGPU_WARN_NO_CELL, "no unit cell selected for <F>");
        }
        rc = dgpu_aver_combine(ctx, fs, box, aref, ctx->istl.as<int32_t>(),
                               ctx->cfact.as<double2>(), closed ? nullptr : ctx->lat.as<double2>(), lat_nslice,
                               closed, lat_n, lat_d, norm, d_acsf);
        if (rc) return rc;
        aver_closed = closed && ncell > 0;
        for (int k = 0; k < 3; k++) {
            alat_n[k] = lat_n[k];
            alat_d[k] = lat_d[k];
        }
        anorm = norm;
        if (aver_closed) {
            ctx->aver.on = 1;
            ctx->aver.nscat = cr->nscat;
            memcpy(ctx->aver.lat_n, lat_n, sizeof(lat_n));
            memcpy(ctx->aver.lat_d, lat_d, sizeof(lat_d));
            ctx->aver.norm = norm;
            memcpy(ctx->aver.ts, ts, sizeof(int64_t) * (2 * cr->nscat + 1));
        }
        float ms = 0.f;
        DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
        kernel_ms += ms;
        if (cancelled(op)) return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
    }

    const double2 *acsf_in = op->fave > 0.0 ? d_acsf : nullptr;
    if (!lots) {
        // ---- type or group sums (fourier_sup.f90:195-244) ----
        FoldSpec nofold = {0, cr->ncatoms, {cr->icc[0], cr->icc[1], cr->icc[2]}, {0, 0, 0}, nullptr};
        rc = dgpu_prepare_atoms(ctx, cr->pos, eiscat, cr->atom_occ, cr->natoms, ngroup, geo, nofold, ctx->ph0,
                                ctx->du, ctx->dv, ctx->dw, ctx->w, ts);
        if (rc) return rc;
        memcpy(ctx->ts_main, ts, sizeof(int64_t) * (2 * ngroup + 1));
        PartRef pref;
        DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
        rc = engine_sums(ctx, engine, ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w, ts, ngroup, op, box, ctx->part,
                         &pref);
        if (rc) return rc;
        DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
        rc = dgpu_combine(ctx, fsm, box, pref, ctx->istl.as<int32_t>(), ctx->cfact.as<double2>(), acsf_in, d_csf,
                          d_dsi, op->diff_scale);
        if (rc) return rc;
        float ms = 0.f;
        DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
        kernel_ms += ms;
        if (engine == DGPU_ENGINE_TC && aver_closed) {
            // points where <F> cancels most of F: exact sums on CUDA cores
            RefineSpec r;
            memset(&r, 0, sizeof(r));
            r.box = box;
            r.fsm = &fsm;
            r.fst = &fs;
            r.istl = ctx->istl.as<int32_t>();
            r.cfact = ctx->cfact.as<double2>();
            r.ph0 = ctx->ph0.as<uint64_t>();
            r.du = ctx->du.as<uint64_t>();
            r.dv = ctx->dv.as<uint64_t>();
            r.dw = ctx->dw.as<uint64_t>();
            r.w = ctx->w.as<float>();
            r.ts_main = ts;
            r.ngroup = ngroup;
            r.aph0 = ctx->aph0.as<uint64_t>();
            r.adu = ctx->adu.as<uint64_t>();
            r.adv = ctx->adv.as<uint64_t>();
            r.adw = ctx->adw.as<uint64_t>();
            r.aw = ctx->aw.as<float>();
            r.ts_fold = ts_fold;
            r.nscat = cr->nscat;
            for (int k = 0; k < 3; k++) {
                r.lat_n[k] = alat_n[k];
                r.lat_d[k] = alat_d[k];
            }
            r.norm = anorm;
            r.diff_scale = op->diff_scale;
            DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));
            rc = dgpu_refine_aver(ctx, r, d_csf, d_acsf, d_dsi, &refined);
            if (rc) return rc;
            DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
            DGPU_CUDA(ctx, cudaEventSynchronize(ctx->ev[3]));
            DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
            kernel_ms += ms;
        }
        for (int t = 0; t < ngroup; t++) pairs += ts[ngroup + 1 + t] * np;
    } else {
        // ---- lots (fourier_sup.f90:136-257): chunks of lots, one engine launch each ----
        const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
        DGPU_CUDA(ctx, ctx->lfac.ensure((size_t)ngroup * nb * sizeof(double2)));
        rc = dgpu_group_factors(ctx, fsm, box, ctx->istl.as<int32_t>(), ctx->cfact.as<double2>(),
                                ctx->lfac.as<double2>());
        if (rc) return rc;
        rc = lots_sums(ctx, cr, op, lp, ngroup, eiscat, geo, box, engine, np, acsf_in, d_csf, d_dsi, &pairs,
                       &kernel_ms);
        if (rc) return rc;
        // dsi * icc1*icc2*icc3 / (ncell*nlots) when nlots != 1 (fourier_sup.f90:273-277)
        double dnorm = 1.0;
        if (lp.nlots != 1)
            dnorm = (double)((int64_t)cr->icc[0] * cr->icc[1] * cr->icc[2]) / (double)((int64_t)lp.ncell * lp.nlots);
        rc = dgpu_lot_scale(ctx, box, d_csf, d_dsi, dnorm * op->diff_scale, sqrt(op->diff_scale));
        if (rc) return rc;
        if (!ctx->lot_keep) ctx->lot_keep = new LotKeep();
        LotKeep &K = *ctx->lot_keep;
        K.lp = lp;
        K.ngroup = ngroup;
        K.engine = engine;
        K.eiscat = eiscat;
        K.geo = geo;
        K.dnorm = dnorm;
    }
    if (!ctx->fs_main) ctx->fs_main = new FormSpec();
    *ctx->fs_main = fsm;
    if (!ctx->fs_type) ctx->fs_type = new FormSpec();
    *ctx->fs_type = fs;
    if (cancelled(op)) return dgpu_set_error(ctx, DGPU_ERR_CANCELLED, "cancelled");
    rc = dgpu_friedel_mirror(ctx, box, idim, d_csf, d_acsf, d_dsi);
    if (rc) return rc;
    // the Lanczos filter of dsi (fourier_sup.f90:284-285), before the statistics
    rc = dgpu_four_filter_dev(ctx, num, op, d_dsi);
    if (rc) return rc;
    double res[7];
    rc = dgpu_qinfo(ctx, g->eck, g->vi, num, d_dsi, res);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[1], ctx->stream));
    DGPU_CUDA(ctx, cudaEventSynchronize(ctx->ev[1]));
    DGPU_CUDA(ctx, cudaGetLastError());
    if (info) {
        memset(info, 0, sizeof(*info));
        for (int k = 0; k < 3; k++) info->fnum[k] = fnum[k];
        info->friedel_dim = idim;
        for (int k = 0; k < 6; k++) info->lmn[k] = geo.lmn[k];
        for (int k = 0; k < 9; k++) info->off_shift[k] = geo.off[k];
        info->ncell = ncell;
        info->engine_used = engine;
        info->pairs = pairs;
        info->pairs_aver = pairs_aver;
        info->refined = refined;
        for (int k = 0; k < 7; k++) info->res[k] = res[k];
        info->kernel_ms = kernel_ms;
        for (int k = 0; k < 4; k++) info->tc_config[k] = engine == DGPU_ENGINE_TC ? ctx->tc_last[k] : -1;
        float tot = 0.f;
        DGPU_CUDA(ctx, cudaEventElapsedTime(&tot, ctx->ev[0], ctx->ev[1]));
        info->total_ms = tot;
    }
    return warn;
}

extern "C" int dgpu_four_run_device(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                                    const dgpu_opts *opts, double *d_csf, double *d_acsf, double *d_dsi,
                                    dgpu_info *info)
{
    if (!ctx || !cr || !grid || !opts || !d_csf || !d_dsi) return DGPU_ERR_ARG;
    int64_t np = (int64_t)grid->inc[0] * grid->inc[1] * grid->inc[2];
    double2 *acsf = (double2 *)d_acsf;
    if (!acsf) {
        DGPU_CUDA(ctx, ctx->acsf.ensure(np * sizeof(double2)));
        acsf = ctx->acsf.as<double2>();
    }
    return dgpu_four_run_dev(ctx, cr, grid, opts, (double2 *)d_csf, acsf, d_dsi, info);
}

// The per-atom arrays of a host crystal to the context's device buffers
// (enqueued on its stream); dc is the crystal with those device pointers.
int dgpu_stage_crystal(dgpu_ctx *ctx, const dgpu_crystal *cr, dgpu_crystal &dc)
{
    const int64_t n = cr->natoms;
    if (n < 1 || !cr->pos || !cr->iscat) return dgpu_set_error(ctx, DGPU_ERR_NO_ATOMS, "no atoms");
    DGPU_CUDA(ctx, ctx->pos.ensure(n * 3 * sizeof(double)));
    DGPU_CUDA(ctx, ctx->iscat.ensure(n * sizeof(int32_t)));
    DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->pos.p, cr->pos, n * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->iscat.p, cr->iscat, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    dc = *cr;
    dc.pos = ctx->pos.as<double>();
    dc.iscat = ctx->iscat.as<int32_t>();
    if (cr->atom_occ) {
        DGPU_CUDA(ctx, ctx->aocc.ensure(n * sizeof(float)));
        DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->aocc.p, cr->atom_occ, n * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
        dc.atom_occ = ctx->aocc.as<float>();
    }
    if (cr->ianis && cr->nanis >= 1) {
        DGPU_CUDA(ctx, ctx->ianis.ensure(n * sizeof(int32_t)));
        DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->ianis.p, cr->ianis, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        dc.ianis = ctx->ianis.as<int32_t>();
    }
    if (cr->isym) {
        DGPU_CUDA(ctx, ctx->isymb.ensure(n * sizeof(int32_t)));
        DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->isymb.p, cr->isym, n * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        dc.isym = ctx->isymb.as<int32_t>();
    }
    return DGPU_OK;
}

extern "C" int dgpu_four_run(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *opts,
                             double *csf, double *acsf, double *dsi, dgpu_info *info)
{
    if (!ctx || !cr || !grid || !opts || !csf || !dsi) return DGPU_ERR_ARG;
    int rc = check_inputs(ctx, cr, grid, opts);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t np = (int64_t)grid->inc[0] * grid->inc[1] * grid->inc[2];
    dgpu_crystal dc;
    rc = dgpu_stage_crystal(ctx, cr, dc);
    if (rc) return rc;
    DGPU_CUDA(ctx, ctx->csf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->acsf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->dsi.ensure(np * sizeof(double)));
    rc = dgpu_four_run_dev(ctx, &dc, grid, opts, ctx->csf.as<double2>(), ctx->acsf.as<double2>(),
                           ctx->dsi.as<double>(), info);
    if (rc < 0) return rc;
    DGPU_CUDA(ctx, cudaMemcpyAsync(csf, ctx->csf.p, np * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(dsi, ctx->dsi.p, np * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    if (acsf)
        DGPU_CUDA(ctx, cudaMemcpyAsync(acsf, ctx->acsf.p, np * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return rc;
}

// ---------------------------------------------------------------------------
// per-type drop-in: four_strucf + tcsf_form_iso
__global__ void k_xat_phase_prepare(const double *xat, int64_t n, double *pos3, int32_t *types)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    pos3[3 * k] = xat[k];
    pos3[3 * k + 1] = xat[n + k];
    pos3[3 * k + 2] = xat[2 * n + k];
    types[k] = 1;
}

extern "C" int dgpu_four_strucf(dgpu_ctx *ctx, const double *xat, int64_t nxat, const double uin[3],
                                const double vin[3], const double win[3], const double off_shift[9],
                                const int32_t lmn[6], const int32_t num[3], const int32_t fnum[3],
                                const double *cfact, const int32_t *istl, double *tcsf)
{
    if (!ctx || !uin || !vin || !win || !off_shift || !lmn || !num || !fnum || !tcsf) return DGPU_ERR_ARG;
    if (nxat < 0 || (nxat > 0 && !xat)) return DGPU_ERR_ARG;
    if (cfact && !istl) return dgpu_set_error(ctx, DGPU_ERR_ARG, "cfact without istl");
    for (int k = 0; k < 3; k++)
        if (num[k] < 1 || fnum[k] < 1 || fnum[k] > num[k]) return dgpu_set_error(ctx, DGPU_ERR_ARG, "num/fnum");
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t np = (int64_t)num[0] * num[1] * num[2];
    DGPU_CUDA(ctx, ctx->csf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->dsi.ensure(np * sizeof(double)));
    DGPU_CUDA(ctx, cudaMemsetAsync(ctx->csf.p, 0, np * sizeof(double2), ctx->stream));
    if (nxat > 0) {
        DGPU_CUDA(ctx, ctx->tc_work.ensure(nxat * 3 * sizeof(double)));
        DGPU_CUDA(ctx, ctx->pos.ensure(nxat * 3 * sizeof(double)));
        DGPU_CUDA(ctx, ctx->iscat.ensure(nxat * sizeof(int32_t)));
        DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->tc_work.p, xat, nxat * 3 * sizeof(double), cudaMemcpyHostToDevice,
                                       ctx->stream));
        k_xat_phase_prepare<<<(unsigned)dgpu_cdiv(nxat, 256), 256, 0, ctx->stream>>>(
            ctx->tc_work.as<double>(), nxat, ctx->pos.as<double>(), ctx->iscat.as<int32_t>());
        DGPU_CUDA(ctx, cudaGetLastError());
        PhaseGeom geo;
        memset(&geo, 0, sizeof(geo));
        geo.mode = DGPU_PHASE_REF22;
        memcpy(geo.lmn, lmn, sizeof(geo.lmn));
        for (int k = 0; k < 3; k++) { geo.vi[k] = uin[k]; geo.vi[3 + k] = vin[k]; geo.vi[6 + k] = win[k]; }
        memcpy(geo.off, off_shift, sizeof(geo.off));
        FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
        int64_t ts[8];
        int rc = dgpu_prepare_atoms(ctx, ctx->pos.as<double>(), ctx->iscat.as<int32_t>(), nullptr, nxat, 1, geo,
                                    nofold, ctx->ph0, ctx->du, ctx->dv, ctx->dw, ctx->w, ts);
        if (rc) return rc;
        BoxSpec box;
        for (int k = 0; k < 3; k++) { box.f[k] = fnum[k]; box.num[k] = num[k]; }
        int32_t nslice = 1;
        rc = dgpu_direct_sums(ctx, ctx->ph0.as<uint64_t>(), ctx->du.as<uint64_t>(), ctx->dv.as<uint64_t>(),
                              ctx->dw.as<uint64_t>(), ctx->w.as<float>(), ts, 1, 1, box, ctx->part, &nslice);
        if (rc) return rc;
        // form factor: table lookup through istl, or unity (the caller's
        // tables replace the cached ones)
        DGPU_CUDA(ctx, ctx->cfact.ensure(DGPU_NTAB * sizeof(double2)));
        DGPU_CUDA(ctx, ctx->istl.ensure(np * sizeof(int32_t)));
        ctx->stl_key.p = nullptr;
        ctx->cf_key.p = nullptr;
        if (cfact) {
            DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->cfact.p, cfact, DGPU_NTAB * sizeof(double2), cudaMemcpyHostToDevice,
                                           ctx->stream));
            DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->istl.p, istl, np * sizeof(int32_t), cudaMemcpyHostToDevice,
                                           ctx->stream));
        } else {
            double2 one[1] = {make_double2(1.0, 0.0)};
            DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->cfact.p, one, sizeof(double2), cudaMemcpyHostToDevice, ctx->stream));
            DGPU_CUDA(ctx, cudaMemsetAsync(ctx->istl.p, 0, np * sizeof(int32_t), ctx->stream));
        }
        FormSpec fs;
        memset(&fs, 0, sizeof(fs));
        fs.mode = DGPU_FORM_TABLE;
        fs.nscat = 1;
        fs.ngroup = 1;
        fs.gtype[1] = 1;
        PartRef pref = {ctx->part.p, nslice, 0};
        rc = dgpu_combine(ctx, fs, box, pref, ctx->istl.as<int32_t>(),
                          ctx->cfact.as<double2>(), nullptr, ctx->csf.as<double2>(), ctx->dsi.as<double>(), 1.0);
        if (rc) return rc;
    }
    DGPU_CUDA(ctx, cudaMemcpyAsync(tcsf, ctx->csf.p, np * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}

extern "C" int dgpu_four_stltab(dgpu_ctx *ctx, const dgpu_grid *grid, const double rten[9], int32_t *istl)
{
    if (!ctx || !grid || !rten || !istl) return DGPU_ERR_ARG;
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t np = (int64_t)grid->inc[0] * grid->inc[1] * grid->inc[2];
    DGPU_CUDA(ctx, ctx->istl.ensure(np * sizeof(int32_t)));
    int rc = dgpu_stltab_dev(ctx, grid->eck, grid->vi, grid->inc, rten, ctx->istl.as<int32_t>());
    DGPU_CUDA(ctx, cudaMemcpyAsync(istl, ctx->istl.p, np * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return rc;
}

extern "C" int dgpu_four_formtab(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *opts, double *cfact)
{
    if (!ctx || !cr || !opts || !cfact || !cr->scat || !cr->occ || !cr->dw) return DGPU_ERR_ARG;
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    DGPU_CUDA(ctx, ctx->cfact.ensure((size_t)cr->nscat * DGPU_NTAB * sizeof(double2)));
    int rc = dgpu_formtab_dev(ctx, cr, opts, ctx->cfact.as<double2>());
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaMemcpyAsync(cfact, ctx->cfact.p, (size_t)cr->nscat * DGPU_NTAB * sizeof(double2),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}

extern "C" int dgpu_four_increments(dgpu_ctx *ctx, const double *xat, int64_t nxat, const double uin[3],
                                    const double vin[3], const double win[3], const double off_shift[9],
                                    int64_t *inc_out)
{
    if (!ctx || !uin || !vin || !win || !off_shift || !inc_out || nxat < 0 || (nxat > 0 && !xat))
        return DGPU_ERR_ARG;
    if (nxat == 0) return DGPU_OK;
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    DGPU_CUDA(ctx, ctx->tc_work.ensure(nxat * 3 * sizeof(double) + 256 + nxat * 6 * sizeof(int64_t)));
    double *d_x = ctx->tc_work.as<double>();
    int64_t *d_o = (int64_t *)((char *)ctx->tc_work.p + ((nxat * 3 * sizeof(double) + 255) & ~(size_t)255));
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_x, xat, nxat * 3 * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    int rc = dgpu_increments_dev(ctx, d_x, nxat, uin, vin, win, off_shift, d_o);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaMemcpyAsync(inc_out, d_o, nxat * 6 * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}

extern "C" int dgpu_chi2_grad(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *opts,
                              const double *i_target, const double *weight, double *chi2, double *grad_pos,
                              double *grad_occ, dgpu_info *info)
{
    int rc = check_inputs(ctx, cr, grid, opts);
    if (rc) return rc;
    if (!i_target || !chi2) return dgpu_set_error(ctx, DGPU_ERR_ARG, "i_target/chi2 missing");
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    return dgpu_chi2_grad_impl(ctx, cr, grid, opts, i_target, weight, chi2, grad_pos, grad_occ, info);
}

extern "C" int dgpu_chi2_grad_device(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                                     const dgpu_opts *opts, const double *d_i_target, const double *d_weight,
                                     double *chi2, double *d_grad_pos, double *d_grad_occ, dgpu_info *info)
{
    int rc = check_inputs(ctx, cr, grid, opts);
    if (rc) return rc;
    if (!d_i_target || !chi2) return dgpu_set_error(ctx, DGPU_ERR_ARG, "i_target/chi2 missing");
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    return dgpu_chi2_grad_impl(ctx, cr, grid, opts, d_i_target, d_weight, chi2, d_grad_pos, d_grad_occ, info, true);
}
