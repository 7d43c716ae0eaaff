// Batched population: many independent crystals (a DIFFEV population --
// diffev/prog/with_mpi.f90:281-510 farms one four_run per member to MPI
// workers) evaluated together on one GPU.
//
// Every stage runs as ONE launch over all members: the atom preparation,
// tables, combine, Friedel mirror and, when targets are given, chi^2, Q and
// the tensor-core adjoint are member-indexed kernels (member blockIdx.y,
// descriptors in device memory), and all members' type sums share one
// persistent tcgen05 launch (a multi-problem work list, k_tc.cu).  The whole
// sequence -- host-to-device copies from pinned staging, kernels,
// device-to-host copies -- is captured once per batch shape into a CUDA
// graph and replayed on later calls (new coordinates, same shapes), so a
// population step costs one graph launch of a few nodes whatever the
// population size.
#include <math.h>
#include <stdlib.h>

#include <algorithm>
#include <chrono>

#include <vector>

#include "dgpu_internal.h"

namespace {

struct Member {
    int64_t natoms, abase, pbase;
    int32_t nscat, idim;   // nscat: partial-sum groups (types, or (type, ADP type) pairs)
    int32_t ntype;         // scattering types (cfact)
    int32_t nanis = 0;     // > 0: anisotropic member, gmap numbers its (type, ADP type) pairs
    std::vector<int32_t> gmap;
    int64_t ts[2 * 64 + 4];
    int64_t np, nb, nblk;
    BoxSpec box;
    PhaseGeom geo;
    dgpu_grid grid;
    double ds;
    double rten[9];
    int64_t istl_off, cfact_off, pt_off, g_off, q_off, grad_off, cnt_off, offs_off, tsd_off, chi_off;
    int64_t adj_item_off, adj_img_off;     // tensor-core adjoint: item and image offsets
    AdjTcPlan adj;
};

struct HostPinned {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes)
    {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaHostAlloc(&p, bytes < 256 ? 256 : bytes, cudaHostAllocDefault);
        if (e == cudaSuccess) cap = bytes < 256 ? 256 : bytes;
        return e;
    }
    ~HostPinned()
    {
        if (p) cudaFreeHost(p);
    }
};

}  // namespace

struct BatchState {
    std::vector<int64_t> sig;
    std::vector<Member> mem;
    bool targets = false, has_occ = false;
    int64_t adj_qmax_off = 0;              // byte offset of the members' Q scales in d_adj_items
    int64_t tot_atoms = 0, tot_pad = 0, tot_np = 0;
    TcPlan plan;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    DevBuf d_pos, d_isc, d_aocc, d_ph0, d_du, d_dv, d_dw, d_w, d_idx, d_cnt, d_offs, d_tsd;
    DevBuf d_istl, d_cfact, d_csf, d_dsi, d_g, d_q, d_chi, d_grad, d_coef, d_fs, d_it, d_wt, part, desc;
    DevBuf d_mult;                         // tensor-core step factors, 3 x tot_pad
    DevBuf d_vimg;                         // tensor-core V images
    DevBuf d_adj_items, d_adj_img;         // tensor-core adjoint: items (+ Q scales), Q images
    DevBuf d_prep_m, d_epi_m, d_adj_m, d_adjtc_p;   // member descriptors of the folded launches
    DevBuf d_chi_out;                      // chi^2 of every member, contiguous
    int64_t max_nblk = 1, max_np = 1, max_nb = 1, max_thr = 1, max_nimg = 1, adj_nitems = 0;
    int32_t max_nscat = 1;
    HostPinned h_pos, h_isc, h_aocc, h_it, h_wt, h_dsi, h_chi, h_grad;
    ~BatchState()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        DevBuf *b[] = {&d_pos, &d_isc, &d_aocc, &d_ph0, &d_du, &d_dv, &d_dw, &d_w, &d_idx, &d_cnt, &d_offs,
                       &d_tsd, &d_istl, &d_cfact, &d_csf, &d_dsi, &d_g, &d_q, &d_chi, &d_grad, &d_coef, &d_fs,
                       &d_it, &d_wt, &part, &desc, &d_prep_m, &d_epi_m, &d_adj_m, &d_adjtc_p, &d_chi_out};
        for (DevBuf *x : b) x->release();
        d_mult.release();
        d_vimg.release();
        d_adj_items.release();
        d_adj_img.release();
    }
};

void dgpu_batch_free(dgpu_ctx *ctx)
{
    for (int k = 0; k < 2; k++) {
        delete ctx->batch[k];
        ctx->batch[k] = nullptr;
    }
}

// Everything one population step runs, in stream order (capturable).
static int batch_enqueue(dgpu_ctx *ctx, BatchState &B, const dgpu_opts *op)
{
    cudaStream_t st = ctx->stream;
    const int32_t nc = (int32_t)B.mem.size();
    DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_pos.p, B.h_pos.p, B.tot_atoms * 3 * sizeof(double), cudaMemcpyHostToDevice, st));
    DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_isc.p, B.h_isc.p, B.tot_atoms * sizeof(int32_t), cudaMemcpyHostToDevice, st));
    if (B.has_occ)
        DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_aocc.p, B.h_aocc.p, B.tot_atoms * sizeof(float), cudaMemcpyHostToDevice, st));
    if (B.targets) {
        DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_it.p, B.h_it.p, B.tot_np * sizeof(double), cudaMemcpyHostToDevice, st));
        DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_wt.p, B.h_wt.p, B.tot_np * sizeof(double), cudaMemcpyHostToDevice, st));
        DGPU_CUDA(ctx, cudaMemsetAsync(B.d_grad.p, 0, B.tot_atoms * 4 * sizeof(double), st));
        DGPU_CUDA(ctx, cudaMemsetAsync(B.d_adj_items.as<uint8_t>() + B.adj_qmax_off, 0, (size_t)nc * sizeof(uint32_t),
                                       st));
    }
    const size_t pad = (size_t)B.tot_pad;
    DGPU_CUDA(ctx, cudaMemsetAsync(B.d_ph0.p, 0, pad * 8, st));
    DGPU_CUDA(ctx, cudaMemsetAsync(B.d_du.p, 0, pad * 8, st));
    DGPU_CUDA(ctx, cudaMemsetAsync(B.d_dv.p, 0, pad * 8, st));
    DGPU_CUDA(ctx, cudaMemsetAsync(B.d_dw.p, 0, pad * 8, st));
    DGPU_CUDA(ctx, cudaMemsetAsync(B.d_w.p, 0, pad * 4, st));
    DGPU_CUDA(ctx, cudaMemsetAsync(B.d_idx.p, 0xFF, pad * 4, st));
    DGPU_CUDA(ctx, cudaMemsetAsync(ctx->flag.as<int32_t>() + 10, 0, sizeof(int32_t), st));   // adjoint
    int rc = dgpu_prepare_members(ctx, B.d_prep_m.as<PrepMember>(), nc, B.max_nblk);
    if (rc) return rc;
    rc = dgpu_tc_mult_async(ctx, B.d_du.as<uint64_t>(), B.d_dv.as<uint64_t>(), B.d_dw.as<uint64_t>(),
                                B.tot_pad, B.tot_pad, B.d_mult.as<float2>());
    if (rc) return rc;
    rc = dgpu_tc_launch(ctx, B.plan);
    if (rc) return rc;
    rc = dgpu_epilogue_members(ctx, B.d_epi_m.as<EpiMember>(), nc, B.max_thr, B.max_np);
    if (rc) return rc;
    if (B.targets) {
        rc = dgpu_adjoint_members(ctx, B.d_adj_m.as<AdjMember>(), nc, B.max_nb);
        if (rc) return rc;
        rc = dgpu_adjtc_members(ctx, B.d_adjtc_p.as<AdjTcProb>(), nc, B.max_nimg,
                                reinterpret_cast<const AdjItem *>(B.d_adj_items.as<uint8_t>()), B.adj_nitems,
                                ctx->flag.as<int32_t>() + 10);
        if (rc) return rc;
        DGPU_CUDA(ctx, cudaMemcpyAsync(B.h_chi.p, B.d_chi_out.p, (size_t)nc * sizeof(double), cudaMemcpyDeviceToHost,
                                       st));
    }
    DGPU_CUDA(ctx, cudaMemcpyAsync(B.h_dsi.p, B.d_dsi.p, B.tot_np * sizeof(double), cudaMemcpyDeviceToHost, st));
    if (B.targets)
        DGPU_CUDA(ctx, cudaMemcpyAsync(B.h_grad.p, B.d_grad.p, B.tot_atoms * 4 * sizeof(double),
                                       cudaMemcpyDeviceToHost, st));
    return DGPU_OK;
}

// (type, ADP type) groups of an anisotropic member (four_nanis,
// fourier_sup.f90:4294-4326): the pairs present, numbered by type, then ADP
// type, as the single-crystal path numbers them; gmap[t*(nanis+1)+a] = group.
// Returns the group count, or -1 for an ADP type outside 1..nanis.
static int32_t member_groups(const dgpu_crystal &cr, std::vector<int32_t> &gmap)
{
    const int32_t na = cr.nanis;
    gmap.assign((size_t)(cr.nscat + 1) * (na + 1), 0);
    for (int64_t i = 0; i < cr.natoms; i++) {
        const int32_t t = cr.iscat[i];
        if (t < 1 || t > cr.nscat) continue;
        const int32_t a = cr.ianis[i];
        if (a < 1 || a > na) return -1;
        gmap[(size_t)t * (na + 1) + a] = 1;
    }
    int32_t g = 0;
    for (int32_t t = 1; t <= cr.nscat; t++)
        for (int32_t a = 1; a <= na; a++) {
            int32_t &e = gmap[(size_t)t * (na + 1) + a];
            if (e) e = ++g;
        }
    return g;
}

// the group of every atom of an anisotropic member (0: VOID)
static void member_group_ids(const dgpu_crystal &cr, const std::vector<int32_t> &gmap, int32_t *out)
{
    const int32_t na = cr.nanis;
    for (int64_t i = 0; i < cr.natoms; i++) {
        const int32_t t = cr.iscat[i];
        const int32_t a = (t >= 1 && t <= cr.nscat) ? cr.ianis[i] : 0;
        out[i] = (t >= 1 && t <= cr.nscat && a >= 1 && a <= na) ? gmap[(size_t)t * (na + 1) + a] : 0;
    }
}

// Member descriptors of the folded launches (fixed per batch shape: the
// buffers they point into belong to the batch state).
static int batch_members(dgpu_ctx *ctx, BatchState &B, int32_t nc, const dgpu_opts *op)
{
    std::vector<PrepMember> pm(nc);
    std::vector<EpiMember> em(nc);
    std::vector<AdjMember> am(nc);
    std::vector<AdjTcProb> tp(nc);
    const size_t cb = dgpu_formcoef_bytes();
    B.max_nblk = B.max_np = B.max_nb = B.max_thr = B.max_nimg = 1;
    B.max_nscat = 1;
    for (int c = 0; c < nc; c++) {
        const Member &m = B.mem[c];
        PrepMember &p = pm[c];
        memset(&p, 0, sizeof(p));
        p.pos = B.d_pos.as<double>() + 3 * m.abase;
        p.iscat = B.d_isc.as<int32_t>() + m.abase;
        p.aocc = B.has_occ ? B.d_aocc.as<float>() + m.abase : nullptr;
        p.n = m.natoms;
        p.nblk = m.nblk;
        p.nscat = m.nscat;
        p.ncf = m.ntype;
        p.ldbw_cf = (op->ldbw && m.nanis == 0) ? 1 : 0;
        for (int k = 0; k < 3; k++) p.num[k] = m.grid.inc[k];
        p.g = m.geo;
        p.counts = B.d_cnt.as<int32_t>() + m.cnt_off;
        p.offs = B.d_offs.as<int64_t>() + m.offs_off;
        p.ts = B.d_tsd.as<int64_t>() + m.tsd_off;
        p.ph0 = B.d_ph0.as<uint64_t>() + m.pbase;
        p.du = B.d_du.as<uint64_t>() + m.pbase;
        p.dv = B.d_dv.as<uint64_t>() + m.pbase;
        p.dw = B.d_dw.as<uint64_t>() + m.pbase;
        p.w = B.d_w.as<float>() + m.pbase;
        p.idx = B.d_idx.as<int32_t>() + m.pbase;
        memcpy(p.rten, m.rten, sizeof(p.rten));
        p.istl = B.d_istl.as<int32_t>() + m.istl_off;
        p.coef = (const char *)B.d_coef.p + c * cb;
        p.cfact = B.d_cfact.as<double2>() + m.cfact_off;
        B.max_nblk = std::max(B.max_nblk, m.nblk);
        B.max_np = std::max(B.max_np, m.np);
        B.max_nb = std::max(B.max_nb, m.nb);
        B.max_nscat = std::max(B.max_nscat, m.ntype);

        EpiMember &e = em[c];
        memset(&e, 0, sizeof(e));
        PartRef pr;
        dgpu_tc_partref(B.plan.probs[c], B.part.as<float2>() + B.plan.part_off[c], pr);
        if (!pr.f32) return dgpu_set_error(ctx, DGPU_ERR_CUDA, "batch: tensor-core partials are not FP32");
        e.fs = B.d_fs.as<FormSpec>() + c;
        e.box = m.box;
        e.part = (const float2 *)pr.p;
        e.nslice = pr.nslice;
        e.idim = m.idim;
        e.lay = dgpu_part_layout(pr, m.box);
        e.istl = p.istl;
        e.cfact = p.cfact;
        e.csf = B.d_csf.as<double2>() + m.pt_off;
        e.dsi = B.d_dsi.as<double>() + m.pt_off;
        e.ds = m.ds;
        e.sqds = sqrt(m.ds);
        e.np = m.np;
        B.max_thr = std::max(B.max_thr, e.lay.nthr);

        AdjMember &a = am[c];
        memset(&a, 0, sizeof(a));
        a.fs = e.fs;
        a.box = m.box;
        a.idim = m.idim;
        a.nscat = m.nscat;
        a.csf = e.csf;
        a.dsi = e.dsi;
        a.istl = p.istl;
        a.cfact = p.cfact;
        a.it = B.d_it.as<double>() + m.pt_off;
        a.wt = B.d_wt.as<double>() + m.pt_off;
        a.g = B.d_g.as<double>() + m.pt_off;
        a.chi = B.d_chi.as<double>() + m.chi_off;
        a.chi_out = B.d_chi_out.as<double>() + c;
        a.sqds = e.sqds;
        a.np = m.np;
        a.nb = m.nb;
        a.Q = B.d_q.as<float2>() + m.q_off;

        if (B.targets) {
            double *gpos = B.d_grad.as<double>() + m.grad_off;
            uint32_t *qmax = reinterpret_cast<uint32_t *>(B.d_adj_items.as<uint8_t>() + B.adj_qmax_off) + c;
            dgpu_adjtc_prob(m.adj, p.ph0, p.du, p.dv, p.dw, p.w, p.idx, a.Q, B.d_adj_img.as<uint8_t>() + m.adj_img_off,
                            qmax, gpos, gpos + 3 * m.natoms, tp[c]);
            B.max_nimg = std::max(B.max_nimg, m.adj.nimg);
        }
    }
    (void)op;
    DGPU_CUDA(ctx, B.d_prep_m.ensure(pm.size() * sizeof(PrepMember)));
    DGPU_CUDA(ctx, B.d_epi_m.ensure(em.size() * sizeof(EpiMember)));
    DGPU_CUDA(ctx, B.d_adj_m.ensure(am.size() * sizeof(AdjMember)));
    DGPU_CUDA(ctx, B.d_adjtc_p.ensure(tp.size() * sizeof(AdjTcProb)));
    DGPU_CUDA(ctx, cudaMemcpy(B.d_prep_m.p, pm.data(), pm.size() * sizeof(PrepMember), cudaMemcpyHostToDevice));
    DGPU_CUDA(ctx, cudaMemcpy(B.d_epi_m.p, em.data(), em.size() * sizeof(EpiMember), cudaMemcpyHostToDevice));
    DGPU_CUDA(ctx, cudaMemcpy(B.d_adj_m.p, am.data(), am.size() * sizeof(AdjMember), cudaMemcpyHostToDevice));
    DGPU_CUDA(ctx, cudaMemcpy(B.d_adjtc_p.p, tp.data(), tp.size() * sizeof(AdjTcProb), cudaMemcpyHostToDevice));
    return DGPU_OK;
}

static int batch_build(dgpu_ctx *ctx, BatchState &B, int32_t nc, const dgpu_crystal *crs, const dgpu_grid *grids,
                       const dgpu_opts *op)
{
    B.mem.assign(nc, Member());
    int64_t abase = 0, pbase = 0, np_tot = 0, istl = 0, cf = 0, q = 0, cnt = 0, tsd = 0;
    for (int c = 0; c < nc; c++) {
        Member &m = B.mem[c];
        const dgpu_crystal &cr = crs[c];
        m.natoms = cr.natoms;
        m.ntype = cr.nscat;
        m.nscat = cr.nscat;
        if (cr.is_anis) {
            m.nanis = cr.nanis;
            m.nscat = member_groups(cr, m.gmap);
            if (m.nscat < 0)
                return dgpu_set_error(ctx, DGPU_ERR_ARG, "member %d: ADP type outside 1..%d", c, cr.nanis);
            if (m.nscat > 63)
                return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "member %d: more than 63 (type, ADP type) groups", c);
            if (m.nscat == 0) m.nscat = 1;
            std::vector<int32_t> gid((size_t)cr.natoms);
            member_group_ids(cr, m.gmap, gid.data());
            dgpu_type_ranges(gid.data(), cr.natoms, m.nscat, m.ts);
        } else {
            dgpu_type_ranges(cr.iscat, cr.natoms, cr.nscat, m.ts);
        }
        m.abase = abase;
        m.pbase = pbase;
        m.grid = grids[c];
        m.ds = op->diff_scale;
        memcpy(m.rten, cr.rten, sizeof(m.rten));
        int32_t fnum[3];
        m.idim = dgpu_friedel_test(&grids[c], op, fnum);
        for (int k = 0; k < 3; k++) {
            m.box.f[k] = fnum[k];
            m.box.num[k] = grids[c].inc[k];
        }
        m.np = (int64_t)grids[c].inc[0] * grids[c].inc[1] * grids[c].inc[2];
        m.nb = (int64_t)fnum[0] * fnum[1] * fnum[2];
        m.nblk = dgpu_prepare_blocks(cr.natoms);
        memset(&m.geo, 0, sizeof(m.geo));
        m.geo.mode = DGPU_PHASE_EXACT64;
        for (int k = 0; k < 3; k++) m.geo.eck[k] = grids[c].eck[k];
        memcpy(m.geo.vi, grids[c].vi, sizeof(m.geo.vi));
        m.istl_off = istl;
        m.cfact_off = cf;
        m.pt_off = np_tot;
        m.g_off = np_tot;
        m.q_off = q;
        m.grad_off = 4 * abase;
        m.cnt_off = cnt;
        m.offs_off = cnt;
        m.tsd_off = tsd;
        m.chi_off = (int64_t)c * 520;
        abase += cr.natoms;
        pbase += m.ts[m.nscat] > 0 ? m.ts[m.nscat] : 0;
        pbase = (pbase + 31) / 32 * 32;
        np_tot += m.np;
        istl += m.np;
        cf += (int64_t)m.ntype * DGPU_NTAB;
        q += (int64_t)m.nscat * m.nb;
        cnt += m.nblk * m.nscat;
        tsd += 2 * m.nscat + 1;
    }
    B.tot_atoms = abase;
    B.tot_pad = pbase > 0 ? pbase : 32;
    B.tot_np = np_tot;
    B.has_occ = false;
    for (int c = 0; c < nc; c++) B.has_occ = B.has_occ || crs[c].atom_occ;
    const size_t na = (size_t)(abase > 0 ? abase : 1), npd = (size_t)B.tot_pad;
    DGPU_CUDA(ctx, B.d_pos.ensure(na * 3 * 8));
    DGPU_CUDA(ctx, B.d_isc.ensure(na * 4));
    DGPU_CUDA(ctx, B.d_aocc.ensure(na * 4));
    DGPU_CUDA(ctx, B.d_ph0.ensure(npd * 8));
    DGPU_CUDA(ctx, B.d_du.ensure(npd * 8));
    DGPU_CUDA(ctx, B.d_dv.ensure(npd * 8));
    DGPU_CUDA(ctx, B.d_dw.ensure(npd * 8));
    DGPU_CUDA(ctx, B.d_w.ensure(npd * 4));
    DGPU_CUDA(ctx, B.d_mult.ensure(npd * TC_MULT_ARRAYS * sizeof(float2)));
    DGPU_CUDA(ctx, B.d_idx.ensure(npd * 4));
    DGPU_CUDA(ctx, B.d_cnt.ensure((size_t)(cnt > 0 ? cnt : 1) * 4));
    DGPU_CUDA(ctx, B.d_offs.ensure((size_t)(cnt > 0 ? cnt : 1) * 8));
    DGPU_CUDA(ctx, B.d_tsd.ensure((size_t)(tsd > 0 ? tsd : 1) * 8));
    DGPU_CUDA(ctx, B.d_istl.ensure((size_t)istl * 4));
    DGPU_CUDA(ctx, B.d_cfact.ensure((size_t)cf * 16));
    DGPU_CUDA(ctx, B.d_csf.ensure((size_t)np_tot * 16));
    DGPU_CUDA(ctx, B.d_dsi.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.d_g.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.d_q.ensure((size_t)(q > 0 ? q : 1) * 8));
    DGPU_CUDA(ctx, B.d_chi.ensure((size_t)nc * 520 * 8));
    DGPU_CUDA(ctx, B.d_chi_out.ensure((size_t)nc * 8));
    DGPU_CUDA(ctx, B.d_grad.ensure(na * 4 * 8));
    DGPU_CUDA(ctx, B.d_it.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.d_wt.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.h_pos.ensure(na * 3 * 8));
    DGPU_CUDA(ctx, B.h_isc.ensure(na * 4));
    DGPU_CUDA(ctx, B.h_aocc.ensure(na * 4));
    DGPU_CUDA(ctx, B.h_it.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.h_wt.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.h_dsi.ensure((size_t)np_tot * 8));
    DGPU_CUDA(ctx, B.h_chi.ensure((size_t)nc * 8));
    DGPU_CUDA(ctx, B.h_grad.ensure(na * 4 * 8));
    DGPU_CUDA(ctx, ctx->flag.ensure(64));
    // per-member form-factor coefficients and FormSpecs
    const size_t cb = dgpu_formcoef_bytes();
    DGPU_CUDA(ctx, B.d_coef.ensure((size_t)nc * cb));
    DGPU_CUDA(ctx, B.d_fs.ensure((size_t)nc * sizeof(FormSpec)));
    std::vector<char> coef((size_t)nc * cb);
    std::vector<FormSpec> fs(nc);
    for (int c = 0; c < nc; c++) {
        dgpu_formcoef_fill(&crs[c], coef.data() + c * cb);
        dgpu_fill_formspec(ctx, &crs[c], op, &grids[c], fs[c]);
        const Member &m = B.mem[c];
        if (m.nanis > 0) {             // (type, ADP type) groups: four_dbw on top of a DW-free cfact
            FormSpec &f = fs[c];
            f.ngroup = m.nscat;
            for (int32_t t = 1; t <= crs[c].nscat; t++)
                for (int32_t a = 1; a <= m.nanis; a++) {
                    const int32_t g = m.gmap[(size_t)t * (m.nanis + 1) + a];
                    if (!g) continue;
                    f.gtype[g] = t;
                    for (int k = 0; k < 6; k++) f.gU[6 * g + k] = crs[c].anis_full[6 * (int64_t)(a - 1) + k];
                }
            if (f.ngroup == 1 && !m.gmap.empty() && f.gtype[1] == 0) f.gtype[1] = 1;
            f.adbw = op->ldbw ? 1 : 0;
            f.ldbw = 0;
            for (int k = 0; k < 3; k++) f.ar[k] = crs[c].ar[k];
        }
    }
    DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_coef.p, coef.data(), coef.size(), cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(B.d_fs.p, fs.data(), fs.size() * sizeof(FormSpec), cudaMemcpyHostToDevice,
                                   ctx->stream));
    // one multi-problem tensor-core plan over all members
    std::vector<TcInput> in(nc);
    for (int c = 0; c < nc; c++) {
        Member &m = B.mem[c];
        in[c].ph0 = B.d_ph0.as<uint64_t>() + m.pbase;
        in[c].du = B.d_du.as<uint64_t>() + m.pbase;
        in[c].dv = B.d_dv.as<uint64_t>() + m.pbase;
        in[c].dw = B.d_dw.as<uint64_t>() + m.pbase;
        in[c].w = B.d_w.as<float>() + m.pbase;
        in[c].mult = B.d_mult.as<float2>() + m.pbase;
        in[c].mult_stride = B.tot_pad;
        in[c].ts = m.ts;
        in[c].ntype = m.nscat;
        in[c].box = m.box;
        in[c].axis = -1;
    }
    const int N = op->tc_tile_n > 0 ? op->tc_tile_n : 64;
    int rc = dgpu_tc_plan(ctx, nc, in.data(), op, N, 4, B.plan, B.part, B.desc, &B.d_vimg);
    if (rc) return rc;
    // tensor-core adjoint plans: items and Q images of every member
    if (B.targets) {
        std::vector<AdjItem> items;
        int64_t img = 0;
        for (int c = 0; c < nc; c++) {
            Member &m = B.mem[c];
            dgpu_adjtc_plan(ctx, m.box, &m.grid, m.nscat, m.ts, m.adj);
            m.adj_item_off = (int64_t)items.size();
            for (AdjItem it : m.adj.items) {
                it.prob = c;
                items.push_back(it);
            }
            m.adj_img_off = img;
            img += (int64_t)dgpu_adjtc_img_bytes(m.adj);
        }
        B.adj_nitems = (int64_t)items.size();
        B.adj_qmax_off = (int64_t)((items.size() * sizeof(AdjItem) + 255) & ~(size_t)255);
        DGPU_CUDA(ctx, B.d_adj_items.ensure((size_t)B.adj_qmax_off + (size_t)nc * sizeof(uint32_t) + 256));
        DGPU_CUDA(ctx, B.d_adj_img.ensure((size_t)(img > 0 ? img : 256)));
        if (!items.empty())
            DGPU_CUDA(ctx, cudaMemcpy(B.d_adj_items.p, items.data(), items.size() * sizeof(AdjItem),
                                      cudaMemcpyHostToDevice));
    }
    rc = batch_members(ctx, B, nc, op);
    if (rc) return rc;
    // istl and cfact depend only on the batch shape: once here, not per step
    int32_t *flag = ctx->flag.as<int32_t>() + 12;
    DGPU_CUDA(ctx, cudaMemsetAsync(flag, 0, sizeof(int32_t), ctx->stream));
    rc = dgpu_tables_members(ctx, B.d_prep_m.as<PrepMember>(), nc, B.max_np, B.max_nscat, op, flag);
    if (rc) return rc;
    int32_t hflag = 0;
    DGPU_CUDA(ctx, cudaMemcpyAsync(&hflag, flag, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hflag) return dgpu_set_error(ctx, DGPU_ERR_STL_RANGE, "sin(theta)/lambda beyond the table in a member");
    return DGPU_OK;
}

// Options outside the population graph (<F>, lots, DISCAMB, REF22 phases,
// anomalous scattering, the CUDA-core engine, the Lanczos filter): every member through the
// single-crystal entries, with the same outputs.  batch_ms is then the wall
// time of the loop.
static int batch_by_member(dgpu_ctx *ctx, int32_t nc, const dgpu_crystal *crs, const dgpu_grid *grids,
                           const dgpu_opts *op, double *const *dsi, const double *const *i_target,
                           const double *const *weight, double *chi2, double *const *grad_pos,
                           double *const *grad_occ)
{
    // the caller's cell selection of four_aver applies to every member: one cell count
    if (op->aver_cells && op->fave > 0.0 && op->fave < 1.0)
        for (int c = 1; c < nc; c++)
            for (int k = 0; k < 3; k++)
                if (crs[c].icc[k] != crs[0].icc[k])
                    return dgpu_set_error(ctx, DGPU_ERR_ARG, "batch: aver_cells needs members of one cell count");
    const auto t0 = std::chrono::steady_clock::now();
    std::vector<double> csf;
    for (int c = 0; c < nc; c++) {
        const int64_t np = (int64_t)grids[c].inc[0] * grids[c].inc[1] * grids[c].inc[2];
        csf.resize((size_t)(2 * np));
        int rc = dgpu_four_run(ctx, &crs[c], &grids[c], op, csf.data(), nullptr, dsi[c], nullptr);
        if (rc < 0) return rc;                                 // warnings (> 0) pass, as in four_run
        if (i_target) {
            rc = dgpu_chi2_grad(ctx, &crs[c], &grids[c], op, i_target[c], weight ? weight[c] : nullptr, &chi2[c],
                                grad_pos ? grad_pos[c] : nullptr, grad_occ ? grad_occ[c] : nullptr, nullptr);
            if (rc < 0) return rc;
        }
    }
    ctx->batch_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    ctx->batch_by_member = true;
    return DGPU_OK;
}

extern "C" int dgpu_batch_run(dgpu_ctx *ctx, int32_t nc, const dgpu_crystal *crs, const dgpu_grid *grids,
                              const dgpu_opts *op, double *const *dsi, const double *const *i_target,
                              const double *const *weight, double *chi2, double *const *grad_pos,
                              double *const *grad_occ)
{
    if (!ctx || nc < 1 || !crs || !grids || !op || !dsi) return DGPU_ERR_ARG;
    const bool targets = i_target != nullptr;
    if (targets && !chi2) return dgpu_set_error(ctx, DGPU_ERR_ARG, "chi2 output missing");
    for (int c = 0; c < nc; c++)
        if (!dsi[c] || (targets && !i_target[c])) return dgpu_set_error(ctx, DGPU_ERR_ARG, "member %d: buffers", c);
    if (op->phase != DGPU_PHASE_EXACT64 || op->fave != 0.0 || op->ano || op->ilots == DGPU_LOT_BOX ||
        op->ilots == DGPU_LOT_ELI || op->discamb || op->engine == DGPU_ENGINE_DIRECT || op->filter ||
        !dgpu_tc_available(ctx))
        return batch_by_member(ctx, nc, crs, grids, op, dsi, i_target, weight, chi2, grad_pos, grad_occ);
    ctx->batch_by_member = false;
    if (targets && !chi2) return dgpu_set_error(ctx, DGPU_ERR_ARG, "chi2 output missing");
    for (int c = 0; c < nc; c++) {
        if (crs[c].natoms < 1 || !crs[c].pos || !crs[c].iscat || crs[c].nscat < 1 || crs[c].nscat > 63)
            return dgpu_set_error(ctx, DGPU_ERR_ARG, "batch member %d: bad crystal", c);
        if (crs[c].is_anis && (crs[c].nanis < 1 || !crs[c].ianis || !crs[c].anis_full))
            return dgpu_set_error(ctx, DGPU_ERR_ARG, "member %d: anisotropic without nanis/ianis/anis_full", c);
        if (!dsi[c] || (targets && !i_target[c])) return dgpu_set_error(ctx, DGPU_ERR_ARG, "member %d: buffers", c);
        for (int k = 0; k < 3; k++)
            if (grids[c].inc[k] < 1) return dgpu_set_error(ctx, DGPU_ERR_ARG, "member %d: inc", c);
    }
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    // batch shape signature: sizes, types and the options that shape the graph
    std::vector<int64_t> sig;
    sig.push_back(nc);
    sig.push_back(targets);
    sig.push_back(op->tc_tile_n);
    sig.push_back(op->form * 16 + op->ldbw * 4 + op->lxray * 2 + op->friedel);
    sig.push_back(op->power);
    sig.push_back((int64_t)(op->diff_scale * 1e12));
    for (int c = 0; c < nc; c++) {
        sig.push_back(crs[c].natoms);
        sig.push_back(crs[c].nscat);
        sig.push_back(crs[c].atom_occ != nullptr);
        int64_t ts[2 * 64 + 4];
        sig.push_back(crs[c].is_anis ? crs[c].nanis : 0);
        if (crs[c].is_anis) {
            // the groups present and their sizes, and the ADP tensors
            std::vector<int32_t> gmap, gid((size_t)crs[c].natoms);
            const int32_t ng = member_groups(crs[c], gmap);
            if (ng < 0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "member %d: ADP type outside 1..%d", c, crs[c].nanis);
            for (int32_t v : gmap) sig.push_back(v);
            member_group_ids(crs[c], gmap, gid.data());
            dgpu_type_ranges(gid.data(), crs[c].natoms, ng > 0 ? ng : 1, ts);
            for (int t = 0; t <= (ng > 0 ? ng : 1); t++) sig.push_back(ts[t]);
            for (int k = 0; k < 6 * crs[c].nanis; k++) sig.push_back((int64_t)(crs[c].anis_full[k] * 1e15));
            for (int k = 0; k < 3; k++) sig.push_back((int64_t)(crs[c].ar[k] * 1e15));
        } else {
            dgpu_type_ranges(crs[c].iscat, crs[c].natoms, crs[c].nscat, ts);
            for (int t = 0; t <= crs[c].nscat; t++) sig.push_back(ts[t]);
        }
        for (int k = 0; k < 12; k++) sig.push_back((int64_t)(grids[c].eck[k] * 1e9));
        for (int k = 0; k < 9; k++) sig.push_back((int64_t)(grids[c].vi[k] * 1e12));
        for (int k = 0; k < 3; k++) sig.push_back(grids[c].inc[k]);
        for (int t = 0; t <= crs[c].nscat; t++) {
            for (int i = 0; i < 11; i++) sig.push_back((int64_t)(crs[c].scat[11 * t + i] * 1e9));
            sig.push_back((int64_t)(crs[c].occ[t] * 1e9));
            sig.push_back((int64_t)(crs[c].dw[t] * 1e9));
        }
        for (int k = 0; k < 9; k++) sig.push_back((int64_t)(crs[c].rten[k] * 1e15));
    }
    // the two most recent batch shapes keep their graphs (a forward-only and a
    // forward-and-gradient step of one population alternate without rebuilds)
    if (ctx->batch[1] && ctx->batch[1]->sig == sig) std::swap(ctx->batch[0], ctx->batch[1]);
    if (!ctx->batch[0] || ctx->batch[0]->sig != sig) {
        delete ctx->batch[1];
        ctx->batch[1] = ctx->batch[0];
        ctx->batch[0] = new BatchState();
        ctx->batch[0]->sig = sig;
        ctx->batch[0]->targets = targets;
        int rc = batch_build(ctx, *ctx->batch[0], nc, crs, grids, op);
        if (rc) {
            dgpu_batch_free(ctx);
            return rc;
        }
    }
    BatchState &B = *ctx->batch[0];
    // stage this step's inputs in pinned memory
    for (int c = 0; c < nc; c++) {
        const Member &m = B.mem[c];
        memcpy((double *)B.h_pos.p + 3 * m.abase, crs[c].pos, m.natoms * 3 * sizeof(double));
        if (m.nanis > 0) member_group_ids(crs[c], m.gmap, (int32_t *)B.h_isc.p + m.abase);
        else memcpy((int32_t *)B.h_isc.p + m.abase, crs[c].iscat, m.natoms * sizeof(int32_t));
        if (B.has_occ) {
            float *o = (float *)B.h_aocc.p + m.abase;
            if (crs[c].atom_occ) memcpy(o, crs[c].atom_occ, m.natoms * sizeof(float));
            else for (int64_t i = 0; i < m.natoms; i++) o[i] = 1.0f;
        }
        if (targets) {
            memcpy((double *)B.h_it.p + m.pt_off, i_target[c], m.np * sizeof(double));
            double *w = (double *)B.h_wt.p + m.pt_off;
            if (weight && weight[c]) memcpy(w, weight[c], m.np * sizeof(double));
            else for (int64_t p = 0; p < m.np; p++) w[p] = 1.0;
        }
    }
    if (!B.exec) {
        DGPU_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
        int rc = batch_enqueue(ctx, B, op);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(ctx->stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return dgpu_set_error(ctx, DGPU_ERR_CUDA, "graph capture: %s", cudaGetErrorString(e));
        B.graph = g;
        DGPU_CUDA(ctx, cudaGraphInstantiate(&B.exec, B.graph, 0));
        DGPU_CUDA(ctx, cudaGraphUpload(B.exec, ctx->stream));    // outside the timed launch
    }
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
    DGPU_CUDA(ctx, cudaGraphLaunch(B.exec, ctx->stream));
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    float ms = 0.f;
    DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]));
    ctx->batch_ms = ms;
    int32_t flags[8];
    DGPU_CUDA(ctx, cudaMemcpy(flags, ctx->flag.as<int32_t>() + 8, sizeof(flags), cudaMemcpyDeviceToHost));
    if (flags[0]) return dgpu_set_error(ctx, DGPU_ERR_TIMEOUT, "tensor-core kernel wait gave up (site %d)", flags[0]);
    if (flags[2]) return dgpu_set_error(ctx, DGPU_ERR_TIMEOUT, "tensor-core adjoint wait gave up (site %d)", flags[2]);
    for (int c = 0; c < nc; c++) {
        const Member &m = B.mem[c];
        memcpy(dsi[c], (double *)B.h_dsi.p + m.pt_off, m.np * sizeof(double));
        if (targets) {
            chi2[c] = ((double *)B.h_chi.p)[c];
            const double *gpos = (double *)B.h_grad.p + m.grad_off;
            if (grad_pos && grad_pos[c]) memcpy(grad_pos[c], gpos, m.natoms * 3 * sizeof(double));
            if (grad_occ && grad_occ[c]) memcpy(grad_occ[c], gpos + 3 * m.natoms, m.natoms * sizeof(double));
        }
    }
    return DGPU_OK;
}

extern "C" double dgpu_batch_last_ms(const dgpu_ctx *ctx) { return ctx ? ctx->batch_ms : 0.0; }

extern "C" int64_t dgpu_batch_graph_nodes(const dgpu_ctx *ctx, int64_t *kernels)
{
    if (kernels) *kernels = 0;
    if (!ctx || ctx->batch_by_member || !ctx->batch[0] || !ctx->batch[0]->graph) return 0;
    size_t n = 0;
    if (cudaGraphGetNodes(ctx->batch[0]->graph, nullptr, &n) != cudaSuccess) return 0;
    if (kernels && n) {
        std::vector<cudaGraphNode_t> nodes(n);
        if (cudaGraphGetNodes(ctx->batch[0]->graph, nodes.data(), &n) == cudaSuccess)
            for (size_t i = 0; i < n; i++) {
                cudaGraphNodeType t;
                if (cudaGraphNodeGetType(nodes[i], &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) (*kernels)++;
            }
    }
    return (int64_t)n;
}
