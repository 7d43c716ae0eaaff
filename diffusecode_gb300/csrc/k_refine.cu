// Exact recomputation of the points where <F> cancels most of F.
//
// With the average structure factor subtracted (four_aver, fourier_sup.f90:
// 1194-1357, then csf = F - acsf at :250-254), a point near a Bragg position
// of the average lattice has |F| and |<F>| many times larger than the
// incoherent level while F - <F> stays small.  The tensor-core engine's type
// sums carry a relative error of a few 1e-7 (FP32 accumulation in TMEM), so
// there the error of |F - <F>|^2 grows with |<F>| / sqrt(N <|f|^2>): about
// 3.4e-7 times that ratio, measured against FP64.  Those points are found
// after the combine (|acsf|^2 > REFINE_TAU * N <|f|^2>) and their type sums
// -- of the crystal and of the atoms folded into one cell -- are evaluated
// again on CUDA cores: FP32 phasors of the exact 64-bit phase by table-driven
// angle addition (1024-entry table of exp(2 pi i j / 1024) in shared memory
// times a two-term series for the remainder, the method of Tang's
// table-driven elementary functions), FP32 sums of short chunks, FP64 across
// chunks and threads.  csf, acsf and dsi of those
// points are then formed with the same form-factor and lattice code as the
// combine kernels.
//
//  * k_refine_select: one thread per point of the Friedel-reduced box,
//    appends the flagged points to a list;
//  * k_refine_sums: work item = (8 listed points, type, atom slice);
//    FP64 partial per (point, type, slice).  The list is sorted with the
//    box axis along which the flagged points are most often neighbours
//    innermost, so that a point is usually the previous one plus one step
//    along that axis and its phase the previous phase plus one 64-bit add;
//  * k_refine_combine: one thread per listed point.
#include <algorithm>
#include <vector>

#include "dgpu_form.cuh"
#include "dgpu_phasor.cuh"
#include "tc_ptx.cuh"

#define RF_PTS 8            // points per work item (each atom's data is read once for all of them)
#define RF_NT 256
#define RF_CHUNK 16         // atoms per FP32 partial before it is added in FP64 (at the most coherent
                            // points FP32 chunks of 32 atoms round alike chunk after chunk: 1.8e-5)
#define RF_SLICE 65536      // atoms per work item
struct RefineTypes {
    int64_t ts[65];         // type ranges of a prepared atom set (0-based types)
    double n[64];           // atoms per type
    int32_t ntype;
};

// flag points with |<F>|^2 > tau * sum_t n_t |cfact_t|^2
__global__ void k_refine_select(const FormSpec *fs, BoxSpec box, const int32_t *__restrict__ istl,
                                const double2 *__restrict__ cfact, const double2 *__restrict__ acsf,
                                const RefineTypes rt, double tau, int32_t *__restrict__ list,
                                int32_t *__restrict__ count)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    if (p >= nb) return;
    const int64_t i = p % box.f[0], j = (p / box.f[0]) % box.f[1], l = p / ((int64_t)box.f[0] * box.f[1]);
    const int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    const double2 a = acsf[idx];
    double h[3];
    form_hvec(fs, i, j, l, h);
    const int32_t q = istl ? istl[idx] : 0;
    double floor = 0.0;
    for (int t = 1; t <= fs->nscat; t++) {
        const double2 c = form_cfact(fs, cfact, q, t, h);
        floor += rt.n[t - 1] * (c.x * c.x + c.y * c.y);
    }
    if (a.x * a.x + a.y * a.y > tau * floor) {
        const int32_t k = atomicAdd(count, 1);
        list[k] = (int32_t)p;
    }
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// The atoms of one work item: FP32 sums of RF_CHUNK atoms per point, added
// to FP64.  RUN: the points are consecutive along the step axis sa and
// their phases one 64-bit add apart.
template <bool RUN>
__device__ __forceinline__ void refine_loop(int64_t lo, int64_t hi, const uint64_t *__restrict__ ph0,
                                            const uint64_t *__restrict__ du, const uint64_t *__restrict__ dv,
                                            const uint64_t *__restrict__ dw, const float *__restrict__ w,
                                            const float2 *__restrict__ tab, const uint32_t (*sn)[3],
                                            const int32_t *sstp, double (*acc)[RF_NT], float (&chk)[RF_PTS][2],
                                            int sa, bool f0, bool f1, bool f2)
{
    const uint32_t m0 = sn[0][0], m1 = sn[0][1], m2 = sn[0][2];
    int c = 0;
    for (int64_t a = lo + threadIdx.x; a < hi; a += RF_NT) {
        // an axis of extent 1 has n = 0 at every point: its step is not read
        const uint64_t b = ph0[a] + PH_ROUND, d0 = f0 ? du[a] : 0, d1 = f1 ? dv[a] : 0, d2 = f2 ? dw[a] : 0;
        const uint64_t ds = sa == 0 ? d0 : sa == 1 ? d1 : d2;
        const PhWeight wa = ph_weight(w[a]);
        uint64_t ph = b + (uint64_t)m0 * d0 + (uint64_t)m1 * d1 + (uint64_t)m2 * d2;
#pragma unroll
        for (int k = 0; k < RF_PTS; k++) {
            if (k > 0) {
                if (RUN || sstp[k]) ph += ds;
                else ph = b + (uint64_t)sn[k][0] * d0 + (uint64_t)sn[k][1] * d1 + (uint64_t)sn[k][2] * d2;
            }
            const float2 e = ph_phasor(ph, tab, wa);
            chk[k][0] += e.x;
            chk[k][1] += e.y;
        }
        if (++c == RF_CHUNK) {
            c = 0;
#pragma unroll
            for (int k = 0; k < RF_PTS; k++) {
                acc[2 * k][threadIdx.x] += (double)chk[k][0];
                acc[2 * k + 1][threadIdx.x] += (double)chk[k][1];
                chk[k][0] = chk[k][1] = 0.f;
            }
        }
    }
}

// out[((k * ntype + t) * nsl + s)]: the type-t sum over atom slice s at
// listed point k (box coordinates from the list entry).  The FP64 sums of
// the chunks live in shared memory (one column per thread): 3 blocks of 256
// threads per SM.
__global__ void __launch_bounds__(RF_NT, 3)
k_refine_sums(const int32_t *__restrict__ list, int32_t npts, BoxSpec box, const uint64_t *__restrict__ ph0,
              const uint64_t *__restrict__ du, const uint64_t *__restrict__ dv, const uint64_t *__restrict__ dw,
              const float *__restrict__ w, const float2 *__restrict__ gtab, const RefineTypes rt, int32_t nsl,
              int32_t sa, double2 *__restrict__ out)
{
    __shared__ double red[RF_NT / 32][RF_PTS][2];
    __shared__ float2 tab[PH_TAB];
    __shared__ double acc[2 * RF_PTS][RF_NT];
    for (int j = threadIdx.x; j < PH_TAB; j += RF_NT) tab[j] = gtab[j];
#pragma unroll
    for (int k = 0; k < 2 * RF_PTS; k++) acc[k][threadIdx.x] = 0.0;
    const int64_t item = blockIdx.x;
    const int s = (int)(item % nsl);
    const int t = (int)((item / nsl) % rt.ntype);
    const int pg = (int)(item / ((int64_t)nsl * rt.ntype));
    const int64_t lo = rt.ts[t] + (int64_t)s * RF_SLICE;
    const int64_t hi = min(rt.ts[t + 1], lo + RF_SLICE);
    // the points' box coordinates; s_stp[k]: point k is point k-1 plus one step along axis sa
    __shared__ uint32_t s_n[RF_PTS][3];
    __shared__ int32_t s_stp[RF_PTS];
    if (threadIdx.x < RF_PTS) {
        const int k = threadIdx.x, pk = pg * RF_PTS + k;
        const int64_t p = pk < npts ? list[pk] : 0, q = pk > 0 && pk - 1 < npts ? list[pk - 1] : 0;
        const uint32_t c[3] = {(uint32_t)(p % box.f[0]), (uint32_t)((p / box.f[0]) % box.f[1]),
                               (uint32_t)(p / ((int64_t)box.f[0] * box.f[1]))};
        const uint32_t e[3] = {(uint32_t)(q % box.f[0]), (uint32_t)((q / box.f[0]) % box.f[1]),
                               (uint32_t)(q / ((int64_t)box.f[0] * box.f[1]))};
        bool st = k > 0 && pk < npts;
        for (int a = 0; a < 3; a++) {
            s_n[k][a] = c[a];
            st = st && c[a] == e[a] + (a == sa ? 1u : 0u);
        }
        s_stp[k] = st;
    }
    __syncthreads();
    float chk[RF_PTS][2];
#pragma unroll
    for (int k = 0; k < RF_PTS; k++) chk[k][0] = chk[k][1] = 0.f;
    bool run = true;                 // every point the previous one plus one step along axis sa
#pragma unroll
    for (int k = 1; k < RF_PTS; k++) run = run && s_stp[k] != 0;
    const bool f0 = box.f[0] > 1, f1 = box.f[1] > 1, f2 = box.f[2] > 1;
    if (run)
        refine_loop<true>(lo, hi, ph0, du, dv, dw, w, tab, s_n, s_stp, acc, chk, sa, f0, f1, f2);
    else
        refine_loop<false>(lo, hi, ph0, du, dv, dw, w, tab, s_n, s_stp, acc, chk, sa, f0, f1, f2);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < RF_PTS; k++) {
        const double x = warp_sum(acc[2 * k][threadIdx.x] + (double)chk[k][0]);
        const double y = warp_sum(acc[2 * k + 1][threadIdx.x] + (double)chk[k][1]);
        if (lane == 0) {
            red[wid][k][0] = x;
            red[wid][k][1] = y;
        }
    }
    __syncthreads();
    if (threadIdx.x < RF_PTS) {
        const int k = threadIdx.x, pk = pg * RF_PTS + k;
        double x = 0.0, y = 0.0;
        for (int v = 0; v < RF_NT / 32; v++) {
            x += red[v][k][0];
            y += red[v][k][1];
        }
        if (pk < npts) out[((int64_t)pk * rt.ntype + t) * nsl + s] = make_double2(x, y);
    }
}

// csf, acsf and dsi of the listed points from the exact sums: the group sums
// sf (main atom set) and the type sums sa (folded atoms), as k_combine and
// k_aver_combine form them (closed-form lattice)
__global__ void k_refine_combine(const int32_t *__restrict__ list, int32_t npts, const FormSpec *fsm,
                                 const FormSpec *fst, BoxSpec box, const int32_t *__restrict__ istl,
                                 const double2 *__restrict__ cfact, const double2 *__restrict__ sf, int32_t nslf,
                                 const double2 *__restrict__ sa, int32_t nsla, int32_t c0, int32_t c1, int32_t c2,
                                 double d0, double d1, double d2, double norm, double ds, double sqds,
                                 double2 *__restrict__ csf, double2 *__restrict__ acsf, double *__restrict__ dsi)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npts) return;
    const int64_t p = list[k];
    const int64_t i = p % box.f[0], j = (p / box.f[0]) % box.f[1], l = p / ((int64_t)box.f[0] * box.f[1]);
    const int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    double h[3];
    form_hvec(fst, i, j, l, h);
    const int32_t q = istl ? istl[idx] : 0;
    double2 A = make_double2(0.0, 0.0);
    for (int t = 1; t <= fst->nscat; t++) {
        double2 s = make_double2(0.0, 0.0);
        for (int u = 0; u < nsla; u++) {
            const double2 v = sa[((int64_t)k * fst->nscat + (t - 1)) * nsla + u];
            s.x += v.x;
            s.y += v.y;
        }
        const double2 m = cmul(s, form_cfact(fst, cfact, q, t, h));
        A.x += m.x;
        A.y += m.y;
    }
    const double2 L = lattice_closed(h, c0, c1, c2, d0, d1, d2);
    const double2 av = cmul(A, L);
    const double2 a = make_double2(av.x * norm, av.y * norm);
    double2 F = make_double2(0.0, 0.0);
    for (int g = 1; g <= fsm->ngroup; g++) {
        double2 s = make_double2(0.0, 0.0);
        for (int u = 0; u < nslf; u++) {
            const double2 v = sf[((int64_t)k * fsm->ngroup + (g - 1)) * nslf + u];
            s.x += v.x;
            s.y += v.y;
        }
        const double2 m = cmul(s, form_group(fsm, cfact, q, g, h));
        F.x += m.x;
        F.y += m.y;
    }
    F.x -= a.x;
    F.y -= a.y;
    acsf[idx] = a;
    csf[idx] = make_double2(F.x * sqds, F.y * sqds);
    dsi[idx] = (F.x * F.x + F.y * F.y) * ds;
}

static void fill_types(RefineTypes &rt, const int64_t *ts, int32_t ntype)
{
    memset(&rt, 0, sizeof(rt));
    rt.ntype = ntype;
    for (int t = 0; t <= ntype; t++) rt.ts[t] = ts[t];
    for (int t = 0; t < ntype; t++) rt.n[t] = (double)ts[ntype + 1 + t];
}

static int32_t slices_of(const RefineTypes &rt)
{
    int64_t most = 1;
    for (int t = 0; t < rt.ntype; t++) most = std::max(most, rt.ts[t + 1] - rt.ts[t]);
    return (int32_t)dgpu_cdiv(most, RF_SLICE);
}

int dgpu_refine_aver(dgpu_ctx *ctx, const RefineSpec &r, double2 *csf, double2 *acsf, double *dsi, int64_t *nref)
{
    *nref = 0;
    const BoxSpec &box = r.box;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    if (nb < 1) return DGPU_OK;
    if (nb > 0x7fffffffLL) return dgpu_set_error(ctx, DGPU_ERR_ARG, "box too large for the refinement list");
    RefineTypes rm, ra;
    fill_types(rm, r.ts_main, r.ngroup);
    fill_types(ra, r.ts_fold, r.nscat);
    // two FormSpec blocks, the point list and its count
    const size_t fsb = (sizeof(FormSpec) + 255) & ~(size_t)255;
    DGPU_CUDA(ctx, ctx->rlist.ensure(2 * fsb + 256 + (size_t)nb * sizeof(int32_t)));
    FormSpec *d_fsm = ctx->rlist.as<FormSpec>();
    FormSpec *d_fst = (FormSpec *)((char *)ctx->rlist.p + fsb);
    int32_t *d_count = (int32_t *)((char *)ctx->rlist.p + 2 * fsb);
    int32_t *d_list = (int32_t *)((char *)ctx->rlist.p + 2 * fsb + 256);
    const float2 *d_tab = ctx->ph_tab.as<float2>();
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_fsm, r.fsm, sizeof(FormSpec), cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_fst, r.fst, sizeof(FormSpec), cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(d_count, 0, sizeof(int32_t), ctx->stream));
    k_refine_select<<<(unsigned)dgpu_cdiv(nb, 256), 256, 0, ctx->stream>>>(d_fst, box, r.istl, r.cfact, acsf, ra,
                                                                           REFINE_TAU, d_list, d_count);
    DGPU_CUDA(ctx, cudaGetLastError());
    int32_t npts = 0;
    DGPU_CUDA(ctx, cudaMemcpyAsync(&npts, d_count, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));      // the FormSpec blocks and npts
    if (npts == 0) return DGPU_OK;
    int32_t sa = 0;
    {
        // The appends above come in no fixed order.  Step axis: the box axis
        // along which flagged points most often have a flagged neighbour;
        // the list is sorted with that axis innermost.
        std::vector<int32_t> h((size_t)npts);
        DGPU_CUDA(ctx, cudaMemcpyAsync(h.data(), d_list, (size_t)npts * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        std::sort(h.begin(), h.end());
        const int64_t st[3] = {1, box.f[0], (int64_t)box.f[0] * box.f[1]};
        int64_t best = -1;
        for (int a = 0; a < 3; a++) {
            if (box.f[a] < 2) continue;
            int64_t adj = 0;
            for (int32_t p : h) {
                const int64_t c = (p / st[a]) % box.f[a];
                if (c + 1 < box.f[a] && std::binary_search(h.begin(), h.end(), (int32_t)(p + st[a]))) adj++;
            }
            if (adj > best) {
                best = adj;
                sa = a;
            }
        }
        const int o1 = sa == 0 ? 1 : 0, o2 = 3 - sa - o1;     // the other axes, outer
        auto key = [&](int32_t p) {
            const int64_t c[3] = {p % box.f[0], (p / box.f[0]) % box.f[1], p / ((int64_t)box.f[0] * box.f[1])};
            return (c[o2] * box.f[o1] + c[o1]) * box.f[sa] + c[sa];
        };
        std::sort(h.begin(), h.end(), [&](int32_t x, int32_t y) { return key(x) < key(y); });
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_list, h.data(), (size_t)npts * sizeof(int32_t), cudaMemcpyHostToDevice,
                                       ctx->stream));
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // h is a host temporary
    }
    const int32_t nslf = slices_of(rm), nsla = slices_of(ra);
    const int64_t ngrp = dgpu_cdiv(npts, RF_PTS);
    DGPU_CUDA(ctx, ctx->rsum.ensure((size_t)npts * ((size_t)r.ngroup * nslf + (size_t)r.nscat * nsla) *
                                    sizeof(double2)));
    double2 *sf = ctx->rsum.as<double2>();
    double2 *sa_sum = sf + (size_t)npts * r.ngroup * nslf;
    const int64_t itf = ngrp * r.ngroup * nslf, ita = ngrp * r.nscat * nsla;
    if (itf > 0x7fffffffLL || ita > 0x7fffffffLL) return dgpu_set_error(ctx, DGPU_ERR_ARG, "refinement too large");
    k_refine_sums<<<(unsigned)itf, RF_NT, 0, ctx->stream>>>(d_list, npts, box, r.ph0, r.du, r.dv, r.dw, r.w, d_tab,
                                                            rm, nslf, sa, sf);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_refine_sums<<<(unsigned)ita, RF_NT, 0, ctx->stream>>>(d_list, npts, box, r.aph0, r.adu, r.adv, r.adw, r.aw,
                                                            d_tab, ra, nsla, sa, sa_sum);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_refine_combine<<<(unsigned)dgpu_cdiv(npts, 128), 128, 0, ctx->stream>>>(
        d_list, npts, d_fsm, d_fst, box, r.istl, r.cfact, sf, nslf, sa_sum, nsla, r.lat_n[0], r.lat_n[1], r.lat_n[2],
        r.lat_d[0], r.lat_d[1], r.lat_d[2], r.norm, r.diff_scale, sqrt(r.diff_scale), csf, acsf, dsi);
    DGPU_CUDA(ctx, cudaGetLastError());
    *nref = npts;
    return DGPU_OK;
}
