// Anisotropic-ADP groups and lot crystals of four_run.
//
//  * groups: an anisotropic crystal is summed per (scattering type, ADP type)
//    pair present (four_nanis, discus/prog/fourier_sup.f90:4294-4326; the
//    loop over them, :195-219), each group then multiplied by its type's
//    cfact and its four_dbw (tcsf_form_aniso, fourier_form.f90:106-143);
//    with DISCAMB form factors per (type, symmetry operation, ADP type)
//    (:166-193), multiplied by its table and four_dbw (tcsf_form_discamb,
//    fourier_form.f90:63-102).
//    The pairs are counted on the device, numbered on the host (by type, then
//    ADP type) and every atom gets its group number, which the rest of the
//    pipeline treats as its type.
//  * lots: the atoms of a box or ellipsoid of ls_xyz unit cells starting at
//    an origin cell, wrapped once at the crystal's edge and shifted by the
//    lot origin (four_getatm / four_getatm_anis, fourier_sup.f90:1852-1968,
//    2015-2138; celltoindex, celltoindex.f90:21-23).  A chunk of lots is
//    gathered into one atom set whose types are (lot, group) pairs, so that
//    one launch of the type-sum engine covers many lots.
#include <vector>

#include "dgpu_internal.h"
#include "dgpu_lots.h"

#define GH_SHARED 4096
#define DISC_MAXSYM DGPU_DISC_MAXSYM

// Slot of an atom: its type, or with DISCAMB (slut != null) the table slot of
// its (type, symmetry operation); 0 when the symmetry has no table.
__device__ __forceinline__ int32_t group_slot(int32_t t, const int32_t *isym, const int32_t *slut, int64_t i)
{
    if (!slut) return t;
    const int32_t y = isym[i];
    return (y >= 0 && y <= DISC_MAXSYM) ? slut[t * (DISC_MAXSYM + 1) + y] : 0;
}

// (slot, ADP type) histogram: hist[s*(nanis+1)+a]; bad counts atoms of a real
// type whose ADP type lies outside 1..nanis or whose symmetry has no table.
// ianis null: every atom has ADP type 1.
__global__ void k_group_hist(const int32_t *__restrict__ iscat, const int32_t *__restrict__ ianis,
                             const int32_t *__restrict__ isym, const int32_t *__restrict__ slut, int64_t n,
                             int32_t nscat, int32_t nslot, int32_t nanis, int32_t *hist, int32_t *bad)
{
    __shared__ int32_t sh[GH_SHARED];
    const int32_t nb = (nslot + 1) * (nanis + 1);
    const bool use_sh = nb <= GH_SHARED;
    if (use_sh)
        for (int k = threadIdx.x; k < nb; k += blockDim.x) sh[k] = 0;
    __syncthreads();
    int32_t nbad = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t t = iscat[i];
        if (t < 1 || t > nscat) continue;
        const int32_t a = ianis ? ianis[i] : 1;
        const int32_t sl = group_slot(t, isym, slut, i);
        if (a < 1 || a > nanis || sl < 1) {
            nbad++;
            continue;
        }
        const int32_t b = sl * (nanis + 1) + a;
        if (use_sh) atomicAdd(&sh[b], 1);
        else atomicAdd(&hist[b], 1);
    }
    if (nbad) atomicAdd(bad, nbad);
    __syncthreads();
    if (use_sh)
        for (int k = threadIdx.x; k < nb; k += blockDim.x)
            if (sh[k]) atomicAdd(&hist[k], sh[k]);
}

// group of every atom (0 for VOID or out-of-range types)
__global__ void k_group_map(const int32_t *__restrict__ iscat, const int32_t *__restrict__ ianis,
                            const int32_t *__restrict__ isym, const int32_t *__restrict__ slut, int64_t n,
                            int32_t nscat, int32_t nanis, const int32_t *__restrict__ gmap, int32_t *__restrict__ geff)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t t = iscat[i];
    int32_t g = 0;
    if (t >= 1 && t <= nscat) {
        const int32_t a = ianis ? ianis[i] : 1;
        const int32_t sl = group_slot(t, isym, slut, i);
        if (a >= 1 && a <= nanis && sl >= 1) g = gmap[sl * (nanis + 1) + a];
    }
    geff[i] = g;
}

// Groups of the partial sums: (type, ADP type) pairs of an anisotropic
// crystal, or with DISCAMB form factors (type, symmetry operation, ADP type)
// triples (fourier_sup.f90:166-193).  Numbered by type, then symmetry in the
// order of the type's table list, then ADP type (the reference's ADP order
// is first appearance, four_nanis: only the FP64 order of the final sum over
// groups differs).  With DISCAMB, fs gets each group's table and the device
// tables must already be in fs.dtab.
int dgpu_anis_groups(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, FormSpec &fs, int32_t *ngroup)
{
    const int64_t n = cr->natoms;
    const dgpu_discamb *dc = op->discamb;
    // ADP types: always for an anisotropic crystal; with DISCAMB when given
    const int32_t *ianis = cr->nanis >= 1 ? cr->ianis : nullptr;
    const int32_t nanis = ianis ? cr->nanis : 1;
    // DISCAMB: slot of every (type, symmetry operation) with a table
    int32_t nslot = cr->nscat;
    std::vector<int32_t> slut, slot_type;
    if (dc) {
        slut.assign((size_t)(cr->nscat + 1) * (DISC_MAXSYM + 1), 0);
        slot_type.assign(1, 0);
        nslot = 0;
        for (int t = 1; t <= cr->nscat; t++)
            for (int k = 0; k < dc->nsymm[t - 1]; k++) {
                const int32_t y = dc->isymm[nslot];
                if (y < 0 || y > DISC_MAXSYM)
                    return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB symmetry number %d outside 0..%d", y,
                                          DISC_MAXSYM);
                int32_t &e = slut[(size_t)t * (DISC_MAXSYM + 1) + y];
                if (e) return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB symmetry %d listed twice for type %d", y, t);
                e = ++nslot;
                slot_type.push_back(t);
            }
        if (nslot != fs.dntab)           // the caller's nsymm changed since the tables were copied
            return dgpu_set_error(ctx, DGPU_ERR_ARG, "DISCAMB: %d tables listed, %d copied", nslot, fs.dntab);
    }
    const int64_t nbins = (int64_t)(nslot + 1) * (nanis + 1);
    if (nbins > ((int64_t)1 << 30))
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "nanis=%d too large", cr->nanis);
    const size_t lut_n = slut.size();
    DGPU_CUDA(ctx, ctx->ghist.ensure((size_t)(nbins + 16 + lut_n) * sizeof(int32_t)));
    int32_t *d_hist = ctx->ghist.as<int32_t>();
    int32_t *d_bad = d_hist + nbins;
    int32_t *d_slut = dc ? d_bad + 16 : nullptr;
    DGPU_CUDA(ctx, cudaMemsetAsync(d_hist, 0, (size_t)(nbins + 16) * sizeof(int32_t), ctx->stream));
    if (dc)
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_slut, slut.data(), lut_n * sizeof(int32_t), cudaMemcpyHostToDevice,
                                       ctx->stream));
    const int32_t *isym = dc ? cr->isym : nullptr;
    const int64_t want = dgpu_cdiv(n, 1024);
    const unsigned nblk = (unsigned)(want < 8 * ctx->nsm ? (want > 0 ? want : 1) : 8 * ctx->nsm);
    k_group_hist<<<nblk, 1024, 0, ctx->stream>>>(cr->iscat, ianis, isym, d_slut, n, cr->nscat, nslot, nanis, d_hist,
                                                 d_bad);
    DGPU_CUDA(ctx, cudaGetLastError());
    std::vector<int32_t> hist((size_t)nbins + 1);
    DGPU_CUDA(ctx, cudaMemcpyAsync(hist.data(), d_hist, (size_t)(nbins + 1) * sizeof(int32_t),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));        // also: the host tables were read
    if (hist[nbins] > 0)
        return dgpu_set_error(ctx, DGPU_ERR_ARG,
                              dc ? "%d atoms with an ADP type outside 1..%d or a symmetry without a DISCAMB table"
                                 : "%d atoms with an ADP type outside 1..%d",
                              hist[nbins], nanis);
    std::vector<int32_t> gmap((size_t)nbins, 0);
    int32_t g = 0;
    for (int sl = 1; sl <= nslot; sl++)
        for (int a = 1; a <= nanis; a++) {
            const int64_t b = (int64_t)sl * (nanis + 1) + a;
            if (hist[b] == 0) continue;
            if (++g > 63)
                return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, dc ? "more than 63 (type, symmetry, ADP type) groups"
                                                                    : "more than 63 (type, ADP type) groups");
            gmap[b] = g;
            fs.gtype[g] = dc ? slot_type[sl] : sl;
            fs.gtab[g] = sl - 1;
            for (int k = 0; k < 6; k++)
                fs.gU[6 * g + k] = cr->anis_full ? cr->anis_full[6 * (int64_t)(a - 1) + k] : 0.0;
        }
    if (g == 0) {                 // no scattering atom at all: one empty group
        g = 1;
        fs.gtype[1] = 1;
        fs.gtab[1] = 0;
        for (int k = 0; k < 6; k++) fs.gU[6 + k] = 0.0;
    }
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_hist, gmap.data(), (size_t)nbins * sizeof(int32_t), cudaMemcpyHostToDevice,
                                   ctx->stream));
    DGPU_CUDA(ctx, ctx->geff.ensure((size_t)(n > 0 ? n : 1) * sizeof(int32_t)));
    k_group_map<<<(unsigned)dgpu_cdiv(n, 256), 256, 0, ctx->stream>>>(cr->iscat, ianis, isym, d_slut, n, cr->nscat,
                                                                      nanis, d_hist, ctx->geff.as<int32_t>());
    DGPU_CUDA(ctx, cudaGetLastError());
    // the map lives in ghist until the kernel has read it
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    fs.ngroup = g;
    fs.adbw = op->ldbw ? 1 : 0;
    fs.ldbw = 0;
    for (int k = 0; k < 3; k++) fs.ar[k] = cr->ar[k];
    *ngroup = g;
    return DGPU_OK;
}

// ---------------------------------------------------------------------------
// lots

bool dgpu_lot_member(const dgpu_opts *op, int32_t ii, int32_t jj, int32_t kk)
{
    if (op->ilots != DGPU_LOT_ELI) return true;
    const int32_t d[3] = {ii, jj, kk};
    double xt[3];
    for (int k = 0; k < 3; k++) {
        const double x0 = (double)op->ls_xyz[k] / 2.0;
        const double u = (double)d[k] - x0 + 0.5;
        xt[k] = u * u / (x0 * x0);
    }
    return (xt[0] + xt[1] + xt[2]) <= 1.0;
}

void dgpu_csize(const dgpu_crystal *cr, const dgpu_opts *op, int32_t cs[3])
{
    for (int k = 0; k < 3; k++) {
        const int32_t c = cr->icc[k] - op->ls_xyz[k] + 1;
        cs[k] = op->lperiod ? cr->icc[k] : (c > 1 ? c : 1);
    }
}

bool dgpu_lots_on(const dgpu_opts *op) { return op->ilots == DGPU_LOT_BOX || op->ilots == DGPU_LOT_ELI; }

int dgpu_lot_plan(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, int32_t ngroup, LotPlan &lp)
{
    int32_t cs[3];
    dgpu_csize(cr, op, cs);
    lp.nlots = op->lot_all ? (int64_t)cs[0] * cs[1] * cs[2] : op->nlots;
    lp.ngroup = ngroup;
    lp.per_chunk = 63 / ngroup;
    if (lp.per_chunk < 1) lp.per_chunk = 1;
    LotGeom &g = lp.geo;
    memset(&g, 0, sizeof(g));
    for (int k = 0; k < 3; k++) {
        g.icc[k] = cr->icc[k];
        g.ls[k] = op->ls_xyz[k];
        g.dim0[k] = cr->dim0[k];
        g.dlo[k] = (int64_t)llround(cr->dim_lo[k]);
    }
    g.ncatoms = cr->ncatoms;
    g.ngroup = ngroup;
    g.natoms = cr->natoms;
    g.cr_end = (int64_t)cr->ncatoms * cr->icc[0] * cr->icc[1] * cr->icc[2];
    g.nextra = cr->natoms > g.cr_end ? cr->natoms - g.cr_end : 0;
    // origins: DISCUS order for lot_all (fourier_sup.f90:141-147), else the caller's
    std::vector<int32_t> host;
    host.reserve((size_t)(3 * lp.nlots));
    for (int64_t l = 0; l < lp.nlots; l++) {
        int32_t lb[3];
        if (op->lot_all) {
            int64_t ii = l;
            lb[2] = (int32_t)(ii / ((int64_t)cs[0] * cs[1])) + 1;
            ii -= (int64_t)(lb[2] - 1) * cs[0] * cs[1];
            lb[1] = (int32_t)(ii / cs[0]) + 1;
            ii -= (int64_t)(lb[1] - 1) * cs[0];
            lb[0] = (int32_t)(ii % cs[0]) + 1;
        } else {
            for (int k = 0; k < 3; k++) lb[k] = op->lot_origins[3 * l + k];
        }
        for (int k = 0; k < 3; k++) host.push_back(lb[k]);
    }
    // cells of the lot shape, in the reference's loop order (z slowest)
    g.ncs = 0;
    const size_t shape_at = host.size();
    for (int32_t kk = 0; kk < g.ls[2]; kk++)
        for (int32_t jj = 0; jj < g.ls[1]; jj++)
            for (int32_t ii = 0; ii < g.ls[0]; ii++)
                if (dgpu_lot_member(op, ii, jj, kk)) {
                    host.push_back(ii);
                    host.push_back(jj);
                    host.push_back(kk);
                    g.ncs++;
                }
    const size_t member_at = host.size();
    for (int32_t kk = 0; kk < g.ls[2]; kk++)
        for (int32_t jj = 0; jj < g.ls[1]; jj++)
            for (int32_t ii = 0; ii < g.ls[0]; ii++) host.push_back(dgpu_lot_member(op, ii, jj, kk) ? 1 : 0);
    g.per_lot = (int64_t)g.ncs * g.ncatoms + g.nextra;
    lp.ncell = g.ncs;
    DGPU_CUDA(ctx, ctx->lplan.ensure(host.size() * sizeof(int32_t)));
    DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->lplan.p, host.data(), host.size() * sizeof(int32_t), cudaMemcpyHostToDevice,
                                   ctx->stream));
    lp.d_orig = ctx->lplan.as<int32_t>();
    lp.d_shape = lp.d_orig + shape_at;
    lp.d_member = lp.d_orig + member_at;
    // every lattice point of the lot shape, for <F> (four_getav, fourier_sup.f90:2467-2506)
    lp.shape.assign(host.begin() + shape_at, host.begin() + member_at);
    return DGPU_OK;
}

// One thread per slot of a chunk: slot s = L*per_lot + r; r < ncs*ncatoms is
// site r%ncatoms of lot cell r/ncatoms, the rest are the atoms stored after
// the periodic block, kept when INT(pos) is a cell of the lot.
__global__ void k_lot_gather(LotGeom g, int64_t lot0, int32_t nlot, const int32_t *__restrict__ orig,
                             const int32_t *__restrict__ shape, const int32_t *__restrict__ member,
                             const double *__restrict__ pos, const int32_t *__restrict__ geff,
                             const float *__restrict__ aocc, double *__restrict__ lpos, int32_t *__restrict__ ltype,
                             float *__restrict__ locc, int32_t *__restrict__ lorig)
{
    const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= (int64_t)nlot * g.per_lot) return;
    const int32_t L = (int32_t)(s / g.per_lot);
    const int64_t r = s - (int64_t)L * g.per_lot;
    const int32_t *lb = orig + 3 * (lot0 + L);
    int64_t src = -1;
    int32_t d[3];
    const int64_t nreg = (int64_t)g.ncs * g.ncatoms;
    if (r < nreg) {
        const int64_t c = r / g.ncatoms, is = r - c * g.ncatoms;
        int64_t ic[3];
        for (int k = 0; k < 3; k++) {
            d[k] = shape[3 * c + k];
            ic[k] = d[k] + lb[k];
            if (ic[k] > g.icc[k]) ic[k] -= g.icc[k];
        }
        const int64_t ia = ((ic[2] - 1) * g.icc[0] * g.icc[1] + (ic[1] - 1) * g.icc[0] + (ic[0] - 1)) * g.ncatoms + is;
        if (ia < g.natoms) src = ia;
    } else {
        const int64_t ir = g.cr_end + (r - nreg);
        bool ok = true;
        for (int k = 0; k < 3; k++) {
            const int64_t ic = (int64_t)pos[3 * ir + k] - g.dlo[k] + 1;    // INT truncates toward zero
            if (ic < 1 || ic > g.icc[k]) {
                ok = false;
                d[k] = 0;
                continue;
            }
            int64_t dk = ic - lb[k];
            if (dk < 0) dk += g.icc[k];
            if (dk >= g.ls[k]) ok = false;
            d[k] = (int32_t)dk;
        }
        if (ok && member[d[0] + (int64_t)g.ls[0] * (d[1] + (int64_t)g.ls[1] * d[2])]) src = ir;
    }
    const int32_t t = src >= 0 ? geff[src] : 0;
    if (t > 0) {
        for (int k = 0; k < 3; k++) {
            double off = g.dim0[k] + (double)lb[k] - 1.0;
            if (d[k] + lb[k] > g.icc[k]) off -= (double)g.icc[k];
            lpos[3 * s + k] = pos[3 * src + k] - off;
        }
        ltype[s] = L * g.ngroup + t;
        locc[s] = aocc ? aocc[src] : 1.0f;
        if (lorig) lorig[s] = (int32_t)src;
    } else {
        for (int k = 0; k < 3; k++) lpos[3 * s + k] = 0.0;
        ltype[s] = 0;
        locc[s] = 0.0f;
        if (lorig) lorig[s] = -1;
    }
}

int dgpu_lot_gather(dgpu_ctx *ctx, const LotPlan &lp, int64_t lot0, int32_t nlot, const double *pos,
                    const int32_t *geff, const float *aocc, int64_t slot0, int64_t *nslots, int32_t *lorig)
{
    const int64_t m = (int64_t)nlot * lp.geo.per_lot;
    *nslots = m;
    if (m == 0) return DGPU_OK;
    if ((size_t)(slot0 + m) * 3 * sizeof(double) > ctx->lpos.cap ||
        (size_t)(slot0 + m) * sizeof(int32_t) > ctx->ltype.cap || (size_t)(slot0 + m) * sizeof(float) > ctx->locc.cap)
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "lot buffers hold fewer than %lld slots", (long long)(slot0 + m));
    k_lot_gather<<<(unsigned)dgpu_cdiv(m, 256), 256, 0, ctx->stream>>>(
        lp.geo, lot0, nlot, lp.d_orig, lp.d_shape, lp.d_member, pos, geff, aocc, ctx->lpos.as<double>() + 3 * slot0,
        ctx->ltype.as<int32_t>() + slot0, ctx->locc.as<float>() + slot0, lorig ? lorig + slot0 : nullptr);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}
