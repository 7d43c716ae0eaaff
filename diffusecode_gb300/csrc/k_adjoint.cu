// Adjoint of four_run: chi^2 = sum_h wt(h) (I(h) - It(h))^2 over the full
// grid and its gradient with respect to every atom position (lattice units)
// and per-atom occupancy weight.  Replaces the finite-difference derivatives
// REFINE and RMC obtain by re-running whole macros
// (refine/prog/refine_run.f90:491-759).
//
// With I = ds |F|^2, F = sum_t c_t(h) sum_j w_j exp(2 pi i h.r_j) (t runs over
// the forward pass's groups: types, or (type, ADP type) pairs whose c_t
// carries the anisotropic Debye-Waller term):
//   dchi2/dw_j   = Re T0_j
//   dchi2/dr_j,k = -2 pi w_j ( eck_k Im T0_j + sum_a vi_a,k Im T_a,j )
//   T0_j  = sum_h Q_t(h) exp(2 pi i h.r_j),  T_a,j = sum_h n_a(h) Q_t(h) exp(...)
//   Q_t(h) = 2 ds G(h) conj(F(h)) c_t(h),    G = dchi2/dI = 2 wt (I - It)
// h = eck + n_0 vi_0 + n_1 vi_1 + n_2 vi_2.  The sums run over the Friedel-
// reduced box; a box point whose mirror lies outside the box carries the
// mirror's G as well (I(-h) = I(h) without anomalous scattering).  The phase
// of every (atom, point) pair is the exact 64-bit fixed point of the forward
// pass; phasors in FP32, sums in FP32 over 256-point tiles and FP64 across.
// With <F> subtracted (four_aver) the folded atoms form a second atom set
// with their own Q (k_adj_qa); both sets add into the same gradient.
#include <math.h>

#include "dgpu_form.cuh"
#include "dgpu_lots.h"

#define ADJ_NT 128
#define ADJ_TP 256

__device__ __forceinline__ double2 ld_adj(const double2 *p) { return *p; }
__device__ __forceinline__ double2 ld_adj(const float2 *p)
{
    const float2 v = *p;
    return make_double2((double)v.x, (double)v.y);
}

// block bx of nbx (256 threads): g over a grid-stride range, this block's chi^2 part
__device__ __forceinline__ void adj_g_block(const double *__restrict__ dsi, const double *__restrict__ it,
                                            const double *__restrict__ wt, int64_t np, double *__restrict__ g,
                                            double *__restrict__ chi_part, int64_t bx, int64_t nbx)
{
    __shared__ double sh[256];
    double acc = 0.0;
    for (int64_t p = bx * blockDim.x + threadIdx.x; p < np; p += nbx * blockDim.x) {
        const double d = dsi[p] - it[p];
        const double w = wt ? wt[p] : 1.0;
        g[p] = 2.0 * w * d;
        acc += w * d * d;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) chi_part[bx] = sh[0];
}

__global__ void k_adj_g(const double *__restrict__ dsi, const double *__restrict__ it,
                        const double *__restrict__ wt, int64_t np, double *__restrict__ g,
                        double *__restrict__ chi_part)
{
    adj_g_block(dsi, it, wt, np, g, chi_part, blockIdx.x, gridDim.x);
}

__global__ void k_adj_chi(const double *part, int n, double *out)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < n; k++) s += part[k];
        *out = s;
    }
}

// Box point pb: its grid coordinates c, grid index and the weight G it
// carries.  The forward pass computes the box and copies the rest
// (four_apply_friedel, k_mirror): a point past the halved axis' middle is
// its mirror's conjugate, and on the middle slab the second half (by the
// linear index L over the later axes) copies the first, while the centre
// is conjugated in place.  So a computed point carries its own G plus that
// of every copy of it; a copied point carries nothing (skip), and at the
// centre csf holds conj(F) (cj).  Without anomalous scattering and with
// Friedel-symmetric form factors the copies equal what a direct
// computation would give, so the rule only matters for complex (DISCAMB)
// factors, but it is what the forward pass does in every case.
__device__ __forceinline__ double adj_point(const BoxSpec &box, int32_t halved, const double *__restrict__ g,
                                            int64_t pb, int32_t c[3], int64_t &idx, bool &skip, bool &cj)
{
    c[0] = (int32_t)(pb % box.f[0]);
    c[1] = (int32_t)((pb / box.f[0]) % box.f[1]);
    c[2] = (int32_t)(pb / ((int64_t)box.f[0] * box.f[1]));
    const int32_t *n = box.num;
    idx = c[0] + (int64_t)n[0] * (c[1] + (int64_t)n[1] * c[2]);
    double G = g[idx];
    skip = false;
    cj = false;
    if (halved >= 1) {
        const int a = halved - 1;
        const int64_t m = (n[0] - 1 - c[0]) + (int64_t)n[0] * ((n[1] - 1 - c[1]) + (int64_t)n[1] * (n[2] - 1 - c[2]));
        if (c[a] < box.f[a] - 1) {
            G += g[m];
        } else {
            int64_t L = 0, N = 1;
            for (int k = a + 1; k < 3; k++) {
                L = L * n[k] + c[k];
                N *= n[k];
            }
            if (2 * L < N - 1) G += g[m];
            else if (2 * L > N - 1) skip = true;
            else cj = true;
        }
    }
    return G;
}

// Q_t(p) on the box, FP32 complex, layout [t][box point]
__device__ __forceinline__ void adj_q_point(const FormSpec *fs, const BoxSpec &box, int32_t halved,
                                            const double *__restrict__ g, const double2 *__restrict__ csf,
                                            const int32_t *__restrict__ istl, const double2 *__restrict__ cfact,
                                            double sqds, float2 *__restrict__ Q, int64_t pb)
{
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    if (pb >= nb) return;
    int32_t c[3];
    int64_t idx;
    bool skip, cj;
    const double G = adj_point(box, halved, g, pb, c, idx, skip, cj);
    // conj(F) with F = csf / sqrt(ds):  2 ds G conj(F) c_t = 2 sqrt(ds) G conj(csf) c_t
    double2 f = csf[idx];
    if (cj) f.y = -f.y;
    const double sc = skip ? 0.0 : 2.0 * sqds * G;
    double h[3];
    if (form_needs_h(fs)) form_hvec(fs, c[0], c[1], c[2], h);
    for (int t = 1; t <= fs->ngroup; t++) {
        const double2 cc = form_group(fs, cfact, istl[idx], t, h);
        const double cr = cc.x, ci = cc.y;
        // conj(f) * c = (fr - i fi)(cr + i ci)
        const double qr = sc * (f.x * cr + f.y * ci);
        const double qi = sc * (f.x * ci - f.y * cr);
        Q[(int64_t)(t - 1) * nb + pb] = make_float2((float)qr, (float)qi);
    }
}

__global__ void k_adj_q(const FormSpec *fs, BoxSpec box, int32_t halved, const double *__restrict__ g,
                        const double2 *__restrict__ csf, const int32_t *__restrict__ istl,
                        const double2 *__restrict__ cfact, double sqds, float2 *__restrict__ Q)
{
    adj_q_point(fs, box, halved, g, csf, istl, cfact, sqds, Q, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// member-indexed g, chi^2 and Q of a batch (member blockIdx.y, or blockIdx.x
// for the one-block chi^2 sum)
#define ADJ_G_BLOCKS 512
__global__ void k_adj_g_m(const AdjMember *__restrict__ M)
{
    const AdjMember &m = M[blockIdx.y];
    adj_g_block(m.dsi, m.it, m.wt, m.np, m.g, m.chi, blockIdx.x, ADJ_G_BLOCKS);
}

__global__ void k_adj_chi_m(const AdjMember *__restrict__ M)
{
    const AdjMember &m = M[blockIdx.x];
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int k = 0; k < ADJ_G_BLOCKS; k++) s += m.chi[k];
        m.chi[ADJ_G_BLOCKS] = s;
        *m.chi_out = s;
    }
}

__global__ void k_adj_q_m(const AdjMember *__restrict__ M)
{
    const AdjMember &m = M[blockIdx.y];
    adj_q_point(m.fs, m.box, m.idim, m.g, m.csf, m.istl, m.cfact, m.sqds, m.Q,
                (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

int dgpu_adjoint_members(dgpu_ctx *ctx, const AdjMember *d_m, int32_t nc, int64_t max_nb)
{
    if (nc < 1) return DGPU_OK;
    k_adj_g_m<<<dim3(ADJ_G_BLOCKS, (unsigned)nc), 256, 0, ctx->stream>>>(d_m);
    k_adj_chi_m<<<(unsigned)nc, 32, 0, ctx->stream>>>(d_m);
    k_adj_q_m<<<dim3((unsigned)dgpu_cdiv(max_nb, 256), (unsigned)nc), 256, 0, ctx->stream>>>(d_m);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

// Q of the folded atoms.  With <F> subtracted, F = sum_t c_t S_t - A and
// A(h) = norm L(h) sum_t c_t(h) S^fold_t(h) (four_aver: the atoms of the
// selected cells moved into one cell, L the closed-form lattice sum of the
// crystal, norm = 1/ncell), so the folded atoms take
//   Q^A_t(h) = -norm L(h) 2 ds G(h) conj(F(h)) c_t(h)
// with the per-type factor c_t of the <F> combine.  Layout [t][box point].
// fbox (lots): F per box point, freshly summed (sum over the lots of F_L,
// unscaled: sqds then carries ds dnorm), instead of csf.
__global__ void k_adj_qa(const FormSpec *fs, BoxSpec box, int32_t halved, const double *__restrict__ g,
                         const double2 *__restrict__ csf, const int32_t *__restrict__ istl,
                         const double2 *__restrict__ cfact, double sqds, int32_t l0, int32_t l1, int32_t l2,
                         double d0, double d1, double d2, double norm, float2 *__restrict__ Q,
                         const double2 *__restrict__ fbox)
{
    const int64_t pb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    if (pb >= nb) return;
    int32_t c[3];
    int64_t idx;
    bool skip, cj;
    const double G = adj_point(box, halved, g, pb, c, idx, skip, cj);
    double h[3];
    form_hvec(fs, c[0], c[1], c[2], h);
    const double2 L = lattice_closed(h, l0, l1, l2, d0, d1, d2);
    double2 f = fbox ? fbox[pb] : csf[idx];
    if (cj && !fbox) f.y = -f.y;
    // -norm L 2 sqrt(ds) G conj(F)
    const double sc = skip ? 0.0 : -2.0 * sqds * G * norm;
    const double2 b = make_double2(sc * (L.x * f.x + L.y * f.y), sc * (L.y * f.x - L.x * f.y));
    const int32_t q = istl ? istl[idx] : 0;
    for (int t = 1; t <= fs->nscat; t++) {
        const double2 m = cmul(b, form_cfact(fs, cfact, q, t, h));
        Q[(int64_t)(t - 1) * nb + pb] = make_float2((float)m.x, (float)m.y);
    }
}

struct AdjGeom {
    int32_t f[3];
    int64_t pbox;
    double eck[3], vi[9];
};

// one thread per prepared atom of one type: sums over all box points; ATOMIC
// when several slots of a launch may share a source atom (lots)
template <bool ATOMIC>
__global__ void __launch_bounds__(ADJ_NT) k_adj_atoms(const uint64_t *__restrict__ ph0, const uint64_t *__restrict__ du,
                                                      const uint64_t *__restrict__ dv, const uint64_t *__restrict__ dw,
                                                      const float *__restrict__ w, const int32_t *__restrict__ aidx,
                                                      int64_t a_lo, int64_t a_hi, const float2 *__restrict__ Q,
                                                      AdjGeom g, double *__restrict__ grad_pos,
                                                      double *__restrict__ grad_occ)
{
    __shared__ float2 sq[ADJ_TP];
    const int64_t a = a_lo + (int64_t)blockIdx.x * ADJ_NT + threadIdx.x;
    const bool valid = a < a_hi;
    const uint64_t p0 = valid ? ph0[a] : 0, d0 = valid ? du[a] : 0, d1 = valid ? dv[a] : 0, d2 = valid ? dw[a] : 0;
    uint64_t ph_plane = p0, ph_row = p0, ph = p0;
    int32_t i = 0, j = 0, l = 0;
    double T0r = 0.0, T0i = 0.0, T1 = 0.0, T2 = 0.0, T3 = 0.0;
    for (int64_t base = 0; base < g.pbox; base += ADJ_TP) {
        const int cnt = (int)min((int64_t)ADJ_TP, g.pbox - base);
        __syncthreads();
        for (int k = threadIdx.x; k < cnt; k += ADJ_NT) sq[k] = Q[base + k];
        __syncthreads();
        float a0r = 0.f, a0i = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
        for (int k = 0; k < cnt; k++) {
            const float2 q = sq[k];
            float s, c;
            __sincosf((float)(int32_t)(ph >> 32) * 1.4629180792671596e-09f, &s, &c);
            const float zr = q.x * c - q.y * s;
            const float zi = q.x * s + q.y * c;
            a0r += zr;
            a0i += zi;
            a1 = fmaf((float)i, zi, a1);
            a2 = fmaf((float)j, zi, a2);
            a3 = fmaf((float)l, zi, a3);
            // next point of the box, first axis fastest (uniform across the block)
            ++i;
            ph += d0;
            if (i == g.f[0]) {
                i = 0;
                ++j;
                ph_row += d1;
                if (j == g.f[1]) {
                    j = 0;
                    ++l;
                    ph_plane += d2;
                    ph_row = ph_plane;
                }
                ph = ph_row;
            }
        }
        T0r += a0r;
        T0i += a0i;
        T1 += a1;
        T2 += a2;
        T3 += a3;
    }
    if (!valid) return;
    const int32_t o = aidx[a];
    if (o < 0) return;
    // added to: an atom also appears once among the folded atoms of <F>
    // (launched after its main sums, on the same stream)
    const double wj = (double)w[a];
    if (grad_occ) {
        if (ATOMIC) atomicAdd(&grad_occ[o], T0r);
        else grad_occ[o] += T0r;
    }
    if (grad_pos) {
        const double zpi = 6.283185307179586476925286766559;
        for (int k = 0; k < 3; k++) {
            const double v = -zpi * wj * (g.eck[k] * T0i + g.vi[k] * T1 + g.vi[3 + k] * T2 + g.vi[6 + k] * T3);
            if (ATOMIC) atomicAdd(&grad_pos[3 * (int64_t)o + k], v);
            else grad_pos[3 * (int64_t)o + k] += v;
        }
    }
}

// Lots: Q of the (lot, group) types of a chunk on the box.  F_L = sum_g
// fac_g S_L,g - <F> (FP64 from the engine's partials, slices first), G by
// the Friedel rule of adj_point; Q_L,g = scale G conj(F_L) fac_g, layout
// [L*ngroup + g][box point]; fsum += F_L over the lots (box order).
template <class P>
__global__ void k_lot_adj_q(int32_t ngroup, int32_t nlot, BoxSpec box, int32_t halved, const P *__restrict__ part,
                            int32_t nslice, PartLayout lay, const double2 *__restrict__ fac,
                            const double2 *__restrict__ acsf, const double *__restrict__ g, double scale,
                            float2 *__restrict__ Q, double2 *__restrict__ fsum)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i, j, l;
    if (r >= lay.nthr || !part_point(lay, box, r, i, j, l)) return;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    const int64_t pb = i + (int64_t)box.f[0] * (j + (int64_t)box.f[1] * l);
    int32_t c[3];
    int64_t idx;
    bool skip, cj;
    const double G = adj_point(box, halved, g, pb, c, idx, skip, cj);
    double2 a = acsf ? acsf[idx] : make_double2(0.0, 0.0);
    if (cj) a.y = -a.y;                          // the mirror conjugated the centre in place
    const int64_t off = i * lay.s0 + j * lay.s1 + l * lay.s2;
    double2 fs = make_double2(0.0, 0.0);
    for (int L = 0; L < nlot; L++) {
        double2 F = make_double2(-a.x, -a.y);
        for (int q = 0; q < ngroup; q++) {
            const P *pt = part + (int64_t)(L * ngroup + q) * nslice * lay.slab + off;
            double2 sl = make_double2(0.0, 0.0);
            for (int k = 0; k < nslice; k++) {
                const double2 v = ld_adj(pt + (int64_t)k * lay.slab);
                sl.x += v.x;
                sl.y += v.y;
            }
            const double2 m = cmul(sl, fac[(int64_t)q * nb + pb]);
            F.x += m.x;
            F.y += m.y;
        }
        fs.x += F.x;
        fs.y += F.y;
        const double sc = skip ? 0.0 : scale * G;
        for (int q = 0; q < ngroup; q++) {
            const double2 f = fac[(int64_t)q * nb + pb];
            // conj(F) f
            const double qr = sc * (F.x * f.x + F.y * f.y), qi = sc * (F.x * f.y - F.y * f.x);
            Q[(int64_t)(L * ngroup + q) * nb + pb] = make_float2((float)qr, (float)qi);
        }
    }
    if (fsum) {
        const double2 o = fsum[pb];
        fsum[pb] = make_double2(o.x + fs.x, o.y + fs.y);
    }
}

int dgpu_lot_adj_q(dgpu_ctx *ctx, int32_t ngroup, int32_t nlot, const BoxSpec &box, int32_t halved,
                   const PartRef &part, const double2 *fac, const double2 *acsf, const double *g, double scale,
                   float2 *Q, double2 *fsum)
{
    const PartLayout lay = dgpu_part_layout(part, box);
    const unsigned nblk = (unsigned)dgpu_cdiv(lay.nthr, 256);
    const int32_t nslice = part.nslice > 0 ? part.nslice : 1;
    if (part.f32)
        k_lot_adj_q<float2><<<nblk, 256, 0, ctx->stream>>>(ngroup, nlot, box, halved, (const float2 *)part.p, nslice,
                                                            lay, fac, acsf, g, scale, Q, fsum);
    else
        k_lot_adj_q<double2><<<nblk, 256, 0, ctx->stream>>>(ngroup, nlot, box, halved, (const double2 *)part.p,
                                                             nslice, lay, fac, acsf, g, scale, Q, fsum);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

__global__ void k_compose_index(int32_t *__restrict__ idx, const int32_t *__restrict__ src, int64_t n)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int32_t k = idx[i];
    idx[i] = k >= 0 ? src[k] : -1;
}

int dgpu_compose_index(dgpu_ctx *ctx, int32_t *idx, const int32_t *src, int64_t n)
{
    if (n < 1) return DGPU_OK;
    k_compose_index<<<(unsigned)dgpu_cdiv(n, 256), 256, 0, ctx->stream>>>(idx, src, n);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_adj_atom_sums(dgpu_ctx *ctx, const BoxSpec &box, const dgpu_grid *grid, int32_t ntype, const int64_t *ts,
                       const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw,
                       const float *w, const int32_t *aidx, const float2 *Q, double *gpos, double *gocc, bool atomic)
{
    AdjGeom ag;
    for (int k = 0; k < 3; k++) {
        ag.f[k] = box.f[k];
        ag.eck[k] = grid->eck[k];
    }
    ag.pbox = (int64_t)box.f[0] * box.f[1] * box.f[2];
    memcpy(ag.vi, grid->vi, sizeof(ag.vi));
    for (int t = 0; t < ntype; t++) {
        const int64_t lo = ts[t], hi = ts[t + 1];
        if (hi <= lo) continue;
        const unsigned nblk = (unsigned)dgpu_cdiv(hi - lo, ADJ_NT);
        if (atomic)
            k_adj_atoms<true><<<nblk, ADJ_NT, 0, ctx->stream>>>(ph0, du, dv, dw, w, aidx, lo, hi,
                                                                 Q + (int64_t)t * ag.pbox, ag, gpos, gocc);
        else
            k_adj_atoms<false><<<nblk, ADJ_NT, 0, ctx->stream>>>(ph0, du, dv, dw, w, aidx, lo, hi,
                                                                  Q + (int64_t)t * ag.pbox, ag, gpos, gocc);
        DGPU_CUDA(ctx, cudaGetLastError());
    }
    return DGPU_OK;
}

// device: the crystal's per-atom arrays, i_target, weight and the two
// gradient arrays are device pointers (chi2 stays a host pointer)
int dgpu_chi2_grad_impl(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op,
                        const double *i_target, const double *weight, double *chi2, double *grad_pos,
                        double *grad_occ, dgpu_info *info, bool device)
{
    if (op->ano) return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "gradient with anomalous scattering");
    if (op->filter) return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "gradient of a filtered intensity");
    if (op->phase != DGPU_PHASE_EXACT64)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "gradient needs EXACT64 phases");
    const int64_t n = cr->natoms;
    const int64_t np = (int64_t)grid->inc[0] * grid->inc[1] * grid->inc[2];
    // forward pass (host inputs are staged first)
    dgpu_crystal dc = *cr;
    int rc = device ? (int)DGPU_OK : dgpu_stage_crystal(ctx, cr, dc);
    if (rc) return rc;
    DGPU_CUDA(ctx, ctx->csf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->acsf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->dsi.ensure(np * sizeof(double)));
    dgpu_info fwd;
    rc = dgpu_four_run_dev(ctx, &dc, grid, op, ctx->csf.as<double2>(), ctx->acsf.as<double2>(),
                           ctx->dsi.as<double>(), &fwd);
    if (rc < 0) return rc;
    // <F> subtracted: its folded atoms carry gradient too (closed-form lattice
    // sum: EXACT64 without lots; no selected cell leaves <F> = 0)
    const bool fold = op->fave > 0.0 && fwd.ncell > 0;
    if (fold && !ctx->aver.on)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "gradient with <F> of a non-box lattice");
    // lots: the forward pass kept its plan; the per-lot sums are redone below
    const bool lots = ctx->lot_keep != nullptr;
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[2], ctx->stream));

    // adjoint weights g(h) and chi^2
    const int nblk = 512;
    DGPU_CUDA(ctx, ctx->gq.ensure(np * sizeof(double) * 3 + (size_t)nblk * sizeof(double) + 64));
    double *d_it = ctx->gq.as<double>();
    double *d_wt = d_it + np;
    double *d_g = d_wt + np;
    double *d_chi = d_g + np;
    const cudaMemcpyKind in_kind = device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_it, i_target, np * sizeof(double), in_kind, ctx->stream));
    if (weight) DGPU_CUDA(ctx, cudaMemcpyAsync(d_wt, weight, np * sizeof(double), in_kind, ctx->stream));
    k_adj_g<<<nblk, 256, 0, ctx->stream>>>(ctx->dsi.as<double>(), d_it, weight ? d_wt : nullptr, np, d_g, d_chi);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_adj_chi<<<1, 32, 0, ctx->stream>>>(d_chi, nblk, d_chi + nblk);
    DGPU_CUDA(ctx, cudaGetLastError());

    // Q on the Friedel box
    BoxSpec box;
    for (int k = 0; k < 3; k++) {
        box.f[k] = fwd.fnum[k];
        box.num[k] = grid->inc[k];
    }
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    // the forward pass's groups: types, or (type, ADP type) pairs
    const FormSpec fs = *ctx->fs_main;
    const int32_t ngroup = fs.ngroup;
    // device copies: the main FormSpec, then the per-type one of <F>
    const size_t fso = (sizeof(FormSpec) + 63) & ~(size_t)63;
    DGPU_CUDA(ctx, ctx->stats.ensure(fso + sizeof(FormSpec)));
    FormSpec *d_fs = ctx->stats.as<FormSpec>();
    FormSpec *d_fst = (FormSpec *)((char *)ctx->stats.p + fso);
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_fs, &fs, sizeof(FormSpec), cudaMemcpyHostToDevice, ctx->stream));
    const int32_t nfold = fold ? ctx->aver.nscat : 0;
    DGPU_CUDA(ctx, ctx->grad.ensure(n * 4 * sizeof(double)));
    double *d_gpos = ctx->grad.as<double>();
    double *d_gocc = d_gpos + 3 * n;
    DGPU_CUDA(ctx, cudaMemsetAsync(d_gpos, 0, n * 4 * sizeof(double), ctx->stream));
    // lots: every lot's atoms get their own weights (sum_L F_L kept for <F>)
    double2 *d_fsum = nullptr;
    if (lots) {
        if (fold) {
            DGPU_CUDA(ctx, ctx->lat.ensure((size_t)nb * sizeof(double2)));
            d_fsum = ctx->lat.as<double2>();
            DGPU_CUDA(ctx, cudaMemsetAsync(d_fsum, 0, (size_t)nb * sizeof(double2), ctx->stream));
        }
        rc = dgpu_lots_adjoint(ctx, &dc, grid, op, box, fwd.friedel_dim, d_g, d_gpos, d_gocc, d_fsum);
        if (rc) return rc;
    }
    DGPU_CUDA(ctx, ctx->gpart.ensure((size_t)(ngroup + nfold) * nb * sizeof(float2)));
    if (!lots) {
        k_adj_q<<<(unsigned)dgpu_cdiv(nb, 256), 256, 0, ctx->stream>>>(
            d_fs, box, fwd.friedel_dim, d_g, ctx->csf.as<double2>(), ctx->istl.as<int32_t>(),
            ctx->cfact.as<double2>(), sqrt(op->diff_scale), ctx->gpart.as<float2>());
        DGPU_CUDA(ctx, cudaGetLastError());
    }
    float2 *d_qa = ctx->gpart.as<float2>() + (int64_t)ngroup * nb;
    if (fold) {
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_fst, ctx->fs_type, sizeof(FormSpec), cudaMemcpyHostToDevice, ctx->stream));
        const auto &av = ctx->aver;
        // with lots: F = sum_L F_L unscaled, so the weight is 2 ds dnorm
        const double sq = lots ? op->diff_scale * ctx->lot_keep->dnorm : sqrt(op->diff_scale);
        k_adj_qa<<<(unsigned)dgpu_cdiv(nb, 256), 256, 0, ctx->stream>>>(
            d_fst, box, fwd.friedel_dim, d_g, ctx->csf.as<double2>(), ctx->istl.as<int32_t>(),
            ctx->cfact.as<double2>(), sq, av.lat_n[0], av.lat_n[1], av.lat_n[2], av.lat_d[0], av.lat_d[1],
            av.lat_d[2], av.norm, d_qa, d_fsum);
        DGPU_CUDA(ctx, cudaGetLastError());
    }

    // per-atom sums (atoms prepared by the forward pass, grouped by type)
    AdjGeom ag;
    for (int k = 0; k < 3; k++) {
        ag.f[k] = box.f[k];
        ag.eck[k] = grid->eck[k];
    }
    ag.pbox = nb;
    memcpy(ag.vi, grid->vi, sizeof(ag.vi));
    // the main atoms (by group), then the folded atoms of <F> (by type)
    struct AtomSet {
        DevBuf *ph0, *du, *dv, *dw, *w, *idx;
        const int64_t *ts;
        int32_t n;
        const float2 *Q;
    };
    const AtomSet sets[2] = {
        {&ctx->ph0, &ctx->du, &ctx->dv, &ctx->dw, &ctx->w, &ctx->aidx, ctx->ts_main, ngroup, ctx->gpart.as<float2>()},
        {&ctx->aph0, &ctx->adu, &ctx->adv, &ctx->adw, &ctx->aw, &ctx->aaidx, ctx->aver.ts, nfold, d_qa}};
    for (const AtomSet &A : sets) {
        if (A.n == 0 || (lots && &A == &sets[0])) continue;     // lots: summed per lot above
        if (fwd.engine_used == DGPU_ENGINE_TC) {
            // same sums on the tensor cores, with the forward pass's engine
            rc = dgpu_adjtc_sums(ctx, box, grid, A.n, A.ts, A.ph0->as<uint64_t>(), A.du->as<uint64_t>(),
                                 A.dv->as<uint64_t>(), A.dw->as<uint64_t>(), A.w->as<float>(), A.idx->as<int32_t>(),
                                 A.Q, d_gpos, d_gocc);
            if (rc) return rc;
        } else {
            for (int t = 0; t < A.n; t++) {
                const int64_t lo = A.ts[t], hi = A.ts[t + 1];
                if (hi <= lo) continue;
                k_adj_atoms<false><<<(unsigned)dgpu_cdiv(hi - lo, ADJ_NT), ADJ_NT, 0, ctx->stream>>>(
                    A.ph0->as<uint64_t>(), A.du->as<uint64_t>(), A.dv->as<uint64_t>(), A.dw->as<uint64_t>(),
                    A.w->as<float>(), A.idx->as<int32_t>(), lo, hi, A.Q + (int64_t)t * nb, ag, d_gpos, d_gocc);
                DGPU_CUDA(ctx, cudaGetLastError());
            }
        }
    }
    DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[3], ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(chi2, d_chi + nblk, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    const cudaMemcpyKind out_kind = device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (grad_pos)
        DGPU_CUDA(ctx, cudaMemcpyAsync(grad_pos, d_gpos, n * 3 * sizeof(double), out_kind, ctx->stream));
    if (grad_occ) DGPU_CUDA(ctx, cudaMemcpyAsync(grad_occ, d_gocc, n * sizeof(double), out_kind, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (info) {
        *info = fwd;
        float ms = 0.f;
        DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]));
        info->total_ms = ms;          // adjoint part; the forward's own time is in kernel_ms
    }
    return DGPU_OK;
}

// Enqueue-only adjoint of one crystal whose forward results (csf, dsi, istl,
// cfact, prepared atoms) are on the device.  g: np doubles, chi: 513 doubles
// (chi[512] receives chi^2), Q: nscat*pbox float2; gpos (3*natoms) and gocc
// (natoms) must be zeroed by the caller.  With cuda_core_sums false only g,
// chi^2 and Q are produced (the tensor-core sums follow from Q).
int dgpu_adjoint_async(dgpu_ctx *ctx, const FormSpec *d_fs, const BoxSpec &box, int32_t friedel_dim,
                       const dgpu_grid *grid, double diff_scale, int32_t nscat, const int64_t *ts,
                       const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw,
                       const float *w, const int32_t *aidx, const double2 *csf, const double *dsi,
                       const int32_t *istl, const double2 *cfact, const double *it, const double *wt, double *g,
                       double *chi, float2 *Q, double *gpos, double *gocc, bool cuda_core_sums)
{
    const int64_t np = (int64_t)box.num[0] * box.num[1] * box.num[2];
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    k_adj_g<<<512, 256, 0, ctx->stream>>>(dsi, it, wt, np, g, chi);
    k_adj_chi<<<1, 32, 0, ctx->stream>>>(chi, 512, chi + 512);
    k_adj_q<<<(unsigned)dgpu_cdiv(nb, 256), 256, 0, ctx->stream>>>(d_fs, box, friedel_dim, g, csf, istl, cfact,
                                                                     sqrt(diff_scale), Q);
    DGPU_CUDA(ctx, cudaGetLastError());
    if (!cuda_core_sums) return DGPU_OK;      // the caller runs the per-atom sums on the tensor cores
    AdjGeom ag;
    for (int k = 0; k < 3; k++) {
        ag.f[k] = box.f[k];
        ag.eck[k] = grid->eck[k];
    }
    ag.pbox = nb;
    memcpy(ag.vi, grid->vi, sizeof(ag.vi));
    for (int t = 0; t < nscat; t++) {
        const int64_t lo = ts[t], hi = ts[t + 1];
        if (hi <= lo) continue;
        k_adj_atoms<false><<<(unsigned)dgpu_cdiv(hi - lo, ADJ_NT), ADJ_NT, 0, ctx->stream>>>(
            ph0, du, dv, dw, w, aidx, lo, hi, Q + (int64_t)t * nb, ag, gpos, gocc);
    }
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}
