// Epilogue kernels of four_run (discus/prog/fourier_sup.f90:136-294):
//   * combine: csf = sum_g factor_g(point) * S_g - acsf ; dsi = |csf|^2
//     (tcsf_form_iso / tcsf_form_aniso, fourier_form.f90:106-177;
//     fourier_sup.f90:205,232,250-254), with diff_scale applied
//     (fourier_sup.f90:281-282);
//   * lots: the same per lot of a chunk, dsi accumulated over the lots and
//     normalised by icc1*icc2*icc3 / (ncell*nlots) (fourier_sup.f90:136-277);
//   * <F>: acsf = (sum_t cfact_t * Savg_t) * lattice / ncell
//     (four_aver, fourier_sup.f90:1194-1357); the lattice sum is either the
//     direct sum over all cells or its closed form (a product of three
//     geometric series);
//   * Friedel mirror (four_apply_friedel, fourier_sup.f90:3726-3757), with the
//     net effect of its sequential in-place loop on the middle slab;
//   * four_qinfo statistics (fourier_sup.f90:2859-2942).
#include "dgpu_form.cuh"
#include "dgpu_lots.h"

__device__ __forceinline__ double2 ld_part(const double2 *p) { return *p; }
__device__ __forceinline__ double2 ld_part(const float2 *p)
{
    float2 v = *p;
    return make_double2((double)v.x, (double)v.y);
}

// element offsets of a partial-sum array (see PartRef)
// Strides of the partial sums along the box axes, and the order in which the
// combine kernels walk them: thread r takes slot r of the partials' own layout
// (axis a0 innermost), so that the reads of the partials -- the bulk of the
// traffic -- are coalesced; padding slots of the tensor-core layout idle.
// (PartLayout: dgpu_internal.h)
PartLayout dgpu_part_layout(const PartRef &r, const BoxSpec &box)
{
    PartLayout L;
    int64_t s[3];
    if (r.s[0] == 0) {
        s[0] = 1;
        s[1] = box.f[0];
        s[2] = (int64_t)box.f[0] * box.f[1];
        L.slab = s[2] * box.f[2];
    } else {
        for (int k = 0; k < 3; k++) s[k] = r.s[k];
        L.slab = r.slab;
    }
    L.s0 = s[0];
    L.s1 = s[1];
    L.s2 = s[2];
    // axes by stride; of two equal strides the axis of extent 1 goes first
    int a[3] = {0, 1, 2};
    auto before = [&](int x, int y) { return s[x] < s[y] || (s[x] == s[y] && box.f[x] == 1 && box.f[y] != 1); };
    for (int p = 0; p < 3; p++)
        for (int q = p + 1; q < 3; q++)
            if (before(a[q], a[p])) {
                const int t = a[p];
                a[p] = a[q];
                a[q] = t;
            }
    L.a0 = a[0];
    L.a1 = a[1];
    L.a2 = a[2];
    L.m1 = s[a[1]];
    L.m2 = s[a[2]];
    L.nthr = L.m2 * box.f[a[2]];
    return L;
}


// (hi, lo) += x in float-float: Knuth's TwoSum, the error carried in lo
__device__ __forceinline__ void ff_add(float &hi, float &lo, float x)
{
    const float s = hi + x, bp = s - hi;
    lo += (hi - (s - bp)) + (x - bp);
    hi = s;
}

// The sum of a group's K-slice partials at one point, in slice order, eight
// slices loaded before any is added (loads in flight).  FP32 partials are
// added in float-float (TwoSum, 48-bit significands) rather than FP64, whose
// rate on this part bounded the combine; FP64 partials in FP64.
__device__ __forceinline__ double2 slice_sum(const float2 *__restrict__ pt, int32_t nslice, int64_t slab)
{
    float hx = 0.f, lx = 0.f, hy = 0.f, ly = 0.f;
    for (int k0 = 0; k0 < nslice; k0 += 8) {
        float2 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = k0 + u < nslice ? pt[(int64_t)(k0 + u) * slab] : make_float2(0.f, 0.f);
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (k0 + u < nslice) {
                ff_add(hx, lx, v[u].x);
                ff_add(hy, ly, v[u].y);
            }
    }
    return make_double2((double)hx + (double)lx, (double)hy + (double)ly);
}

__device__ __forceinline__ double2 slice_sum(const double2 *__restrict__ pt, int32_t nslice, int64_t slab)
{
    double2 s = make_double2(0.0, 0.0);
    for (int k0 = 0; k0 < nslice; k0 += 8) {
        double2 v[8];
#pragma unroll
        for (int u = 0; u < 8; u++) v[u] = k0 + u < nslice ? pt[(int64_t)(k0 + u) * slab] : make_double2(0.0, 0.0);
#pragma unroll
        for (int u = 0; u < 8; u++)
            if (k0 + u < nslice) {
                s.x += v[u].x;
                s.y += v[u].y;
            }
    }
    return s;
}

template <class P>
__device__ __forceinline__ void combine_slot(const FormSpec *fs, const BoxSpec &box, const P *__restrict__ part,
                                             int32_t nslice, const PartLayout &lay, const int32_t *__restrict__ istl,
                                             const double2 *__restrict__ cfact, const double2 *__restrict__ acsf,
                                             double2 *__restrict__ csf, double *__restrict__ dsi, double ds,
                                             double sqds, int64_t r)
{
    int64_t i, j, l;
    if (r >= lay.nthr || !part_point(lay, box, r, i, j, l)) return;
    int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    double h[3];
    if (form_needs_h(fs)) form_hvec(fs, i, j, l, h);
    int32_t q = istl ? istl[idx] : 0;
    double2 F = make_double2(0.0, 0.0);
    for (int t = 1; t <= fs->ngroup; t++) {
        const P *pt = part + (int64_t)(t - 1) * nslice * lay.slab + i * lay.s0 + j * lay.s1 + l * lay.s2;
        const double2 s = slice_sum(pt, nslice, lay.slab);
        double2 c = form_group(fs, cfact, q, t, h);
        double2 m = cmul(s, c);
        F.x += m.x;
        F.y += m.y;
    }
    if (acsf) {
        double2 a = acsf[idx];
        F.x -= a.x;
        F.y -= a.y;
    }
    csf[idx] = make_double2(F.x * sqds, F.y * sqds);
    dsi[idx] = (F.x * F.x + F.y * F.y) * ds;
}

template <class P>
__global__ void k_combine(const FormSpec *fs, BoxSpec box, const P *__restrict__ part,
                          int32_t nslice, PartLayout lay, const int32_t *__restrict__ istl,
                          const double2 *__restrict__ cfact, const double2 *__restrict__ acsf,
                          double2 *__restrict__ csf, double *__restrict__ dsi, double ds, double sqds)
{
    combine_slot(fs, box, part, nslice, lay, istl, cfact, acsf, csf, dsi, ds, sqds,
                 (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

template <class P>
__global__ void k_aver_combine(const FormSpec *fs, BoxSpec box, const P *__restrict__ apart,
                               int32_t anslice, PartLayout lay, const int32_t *__restrict__ istl,
                               const double2 *__restrict__ cfact, const double2 *__restrict__ lat,
                               int32_t lat_nslice, int32_t lat_closed, int32_t c0, int32_t c1,
                               int32_t c2, double d0, double d1, double d2, double norm,
                               double2 *__restrict__ acsf)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i, j, l;
    if (r >= lay.nthr || !part_point(lay, box, r, i, j, l)) return;
    int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    int64_t nfull = (int64_t)box.num[0] * box.num[1] * box.num[2];
    double h[3];
    form_hvec(fs, i, j, l, h);
    int32_t q = istl ? istl[idx] : 0;
    double2 A = make_double2(0.0, 0.0);
    for (int t = 1; t <= fs->nscat; t++) {
        double2 s = make_double2(0.0, 0.0);
        const P *pt = apart + (int64_t)(t - 1) * anslice * lay.slab + i * lay.s0 + j * lay.s1 + l * lay.s2;
        for (int k = 0; k < anslice; k++) {
            double2 v = ld_part(pt + (int64_t)k * lay.slab);
            s.x += v.x;
            s.y += v.y;
        }
        double2 m = cmul(s, form_cfact(fs, cfact, q, t, h));
        A.x += m.x;
        A.y += m.y;
    }
    double2 L;
    if (lat_closed) {
        L = lattice_closed(h, c0, c1, c2, d0, d1, d2);
    } else {
        L = make_double2(0.0, 0.0);
        for (int k = 0; k < lat_nslice; k++) {
            double2 v = lat[(int64_t)k * nfull + idx];
            L.x += v.x;
            L.y += v.y;
        }
    }
    const double2 av = cmul(A, L);
    acsf[idx] = make_double2(av.x * norm, av.y * norm);
}

// four_apply_friedel: points past the halved axis' middle take the conjugate
// of their mirror; on the middle slab the sequential loop leaves the first
// half, conjugates the centre and mirrors the second half.
__device__ __forceinline__ void mirror_point(const BoxSpec &box, int32_t a, double2 *csf, double2 *acsf,
                                             double *dsi, int64_t p)
{
    const int32_t *n = box.num;
    int64_t np = (int64_t)n[0] * n[1] * n[2];
    if (p >= np) return;
    int32_t c[3] = {(int32_t)(p % n[0]), (int32_t)((p / n[0]) % n[1]), (int32_t)(p / ((int64_t)n[0] * n[1]))};
    int32_t mid = box.f[a] - 1;
    if (c[a] < mid) return;
    int64_t m = (n[0] - 1 - c[0]) + (int64_t)n[0] * ((n[1] - 1 - c[1]) + (int64_t)n[1] * (n[2] - 1 - c[2]));
    if (c[a] == mid) {
        // linear index over the later axes, last axis fastest
        int64_t L = 0, N = 1;
        for (int k = a + 1; k < 3; k++) {
            L = L * n[k] + c[k];
            N *= n[k];
        }
        if (2 * L < N - 1) return;
        if (2 * L == N - 1) {
            csf[p].y = -csf[p].y;
            if (acsf) acsf[p].y = -acsf[p].y;
            return;
        }
    }
    double2 v = csf[m];
    csf[p] = make_double2(v.x, -v.y);
    if (acsf) {
        double2 u = acsf[m];
        acsf[p] = make_double2(u.x, -u.y);
    }
    dsi[p] = dsi[m];
}

__global__ void k_mirror(BoxSpec box, int32_t a, double2 *csf, double2 *acsf, double *dsi)
{
    mirror_point(box, a, csf, acsf, dsi, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// member-indexed combine and mirror of a batch (member blockIdx.y)
__global__ void k_combine_m(const EpiMember *__restrict__ M)
{
    const EpiMember &m = M[blockIdx.y];
    combine_slot<float2>(m.fs, m.box, m.part, m.nslice, m.lay, m.istl, m.cfact, nullptr, m.csf, m.dsi, m.ds,
                         m.sqds, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void k_mirror_m(const EpiMember *__restrict__ M)
{
    const EpiMember &m = M[blockIdx.y];
    if (m.idim < 1 || m.idim > 3) return;
    mirror_point(m.box, m.idim - 1, m.csf, nullptr, m.dsi, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

int dgpu_epilogue_members(dgpu_ctx *ctx, const EpiMember *d_m, int32_t nc, int64_t max_thr, int64_t max_np)
{
    if (nc < 1) return DGPU_OK;
    k_combine_m<<<dim3((unsigned)dgpu_cdiv(max_thr, 256), (unsigned)nc), 256, 0, ctx->stream>>>(d_m);
    k_mirror_m<<<dim3((unsigned)dgpu_cdiv(max_np, 256), (unsigned)nc), 256, 0, ctx->stream>>>(d_m);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

struct QStat {
    double bmax, bmin, dmax, dmin, dsum, dsum2;
    long long nd;
};

__device__ __forceinline__ void qmerge(QStat &a, const QStat &b)
{
    a.bmax = fmax(a.bmax, b.bmax);
    a.bmin = fmin(a.bmin, b.bmin);
    a.dmax = fmax(a.dmax, b.dmax);
    a.dmin = fmin(a.dmin, b.dmin);
    a.dsum += b.dsum;
    a.dsum2 += b.dsum2;
    a.nd += b.nd;
}

// Whether h = e + v0 i + v1 j + v2 l can be an integer: the FP32 estimate
// errs by at most 7 roundings of 2^-24 times mag = |e| + |v0| i + |v1| j +
// |v2| l (four inputs, three FMAs), well inside 1e-6 mag + 1e-5, so an
// estimate farther than that from every integer rules the point out and the
// FP64 test in the reference's order is needed only near integers.
__device__ __forceinline__ bool maybe_integral(float e, float v0, float v1, float v2, float fi, float fj, float fl)
{
    const float h = fmaf(v2, fl, fmaf(v1, fj, fmaf(v0, fi, e)));
    const float mag = fabsf(e) + fabsf(v0) * fi + fabsf(v1) * fj + fabsf(v2) * fl;
    return fabsf(h - rintf(h)) <= fmaf(1e-6f, mag, 1e-5f);
}

#define QNT 256
__global__ void k_qinfo_part(double e0, double e1, double e2, FormSpec const *fs, int32_t n0,
                             int32_t n1, int32_t n2, const double *dsi, QStat *out)
{
    QStat s = {-9999.0, (double)1e19f, -9999.0, (double)1e19f, 0.0, 0.0, 0};
    int64_t np = (int64_t)n0 * n1 * n2;
    double e[3] = {e0, e1, e2};
    float ef[3], vf[9];
#pragma unroll
    for (int k = 0; k < 3; k++) ef[k] = (float)e[k];
#pragma unroll
    for (int k = 0; k < 9; k++) vf[k] = (float)fs->vi[k];
    const bool narrow = np <= (int64_t)0xFFFFFFFFll;     // 32-bit index arithmetic
    for (int64_t p = (int64_t)blockIdx.x * QNT + threadIdx.x; p < np; p += (int64_t)gridDim.x * QNT) {
        int64_t i, j, l;
        if (narrow) {
            const uint32_t q = (uint32_t)p, a = q / (uint32_t)n0;
            i = q - a * (uint32_t)n0;
            j = a % (uint32_t)n1;
            l = a / (uint32_t)n1;
        } else {
            i = p % n0;
            j = (p / n0) % n1;
            l = p / ((int64_t)n0 * n1);
        }
        const float fi = (float)i, fj = (float)j, fl = (float)l;
        bool bragg = true;
#pragma unroll
        for (int k = 0; k < 3; k++) bragg = bragg && maybe_integral(ef[k], vf[k], vf[3 + k], vf[6 + k], fi, fj, fl);
        if (bragg)
            for (int k = 0; k < 3; k++) {
                double h = __dadd_rn(__dadd_rn(__dadd_rn(e[k], __dmul_rn(fs->vi[k], (double)fi)),
                                               __dmul_rn(fs->vi[3 + k], (double)fj)),
                                     __dmul_rn(fs->vi[6 + k], (double)fl));
                bragg = bragg && (h == trunc(h));
            }
        double v = dsi[p];
        if (bragg) {
            s.bmax = fmax(s.bmax, v);
            s.bmin = fmin(s.bmin, v);
        } else {
            s.dmax = fmax(s.dmax, v);
            s.dmin = fmin(s.dmin, v);
            s.dsum += v;
            s.dsum2 += v * v;
            s.nd++;
        }
    }
    __shared__ QStat sh[QNT];
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = QNT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) qmerge(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x == 0) out[blockIdx.x] = sh[0];
}

__global__ void k_qinfo_final(const QStat *part, int n, double *res)
{
    __shared__ QStat sh[QNT];
    QStat s = {-9999.0, (double)1e19f, -9999.0, (double)1e19f, 0.0, 0.0, 0};
    for (int k = threadIdx.x; k < n; k += QNT) qmerge(s, part[k]);
    sh[threadIdx.x] = s;
    __syncthreads();
    for (int o = QNT / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) qmerge(sh[threadIdx.x], sh[threadIdx.x + o]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    s = sh[0];
    double ave = 0.0, sig = 0.0;
    if (s.nd) {
        ave = s.dsum / (double)s.nd;
        sig = sqrt(s.dsum2 / (double)s.nd - ave * ave);
    }
    res[0] = 6.0;
    res[1] = s.dmin;
    res[2] = s.dmax;
    res[3] = ave;
    res[4] = sig;
    res[5] = s.bmin;
    res[6] = s.bmax;
}

// ---------------------------------------------------------------------------
static int upload_formspec(dgpu_ctx *ctx, const FormSpec &fs, FormSpec **d)
{
    DGPU_CUDA(ctx, ctx->stats.ensure(sizeof(FormSpec) + 4096 * sizeof(QStat) + 64));
    *d = ctx->stats.as<FormSpec>();
    DGPU_CUDA(ctx, cudaMemcpyAsync(*d, &fs, sizeof(FormSpec), cudaMemcpyHostToDevice, ctx->stream));
    return DGPU_OK;
}

int dgpu_combine(dgpu_ctx *ctx, const FormSpec &fs, const BoxSpec &box, const PartRef &part,
                 const int32_t *istl, const double2 *cfact,
                 const double2 *acsf_in, double2 *csf, double *dsi, double diff_scale)
{
    FormSpec *d;
    int rc = upload_formspec(ctx, fs, &d);
    if (rc) return rc;
    const PartLayout lay = dgpu_part_layout(part, box);
    const unsigned nblk = (unsigned)dgpu_cdiv(lay.nthr, 256);
    if (part.f32)
        k_combine<float2><<<nblk, 256, 0, ctx->stream>>>(d, box, (const float2 *)part.p, part.nslice, lay, istl,
                                                          cfact, acsf_in, csf, dsi, diff_scale, sqrt(diff_scale));
    else
        k_combine<double2><<<nblk, 256, 0, ctx->stream>>>(d, box, (const double2 *)part.p, part.nslice, lay, istl,
                                                           cfact, acsf_in, csf, dsi, diff_scale, sqrt(diff_scale));
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // FormSpec block reused next
    return DGPU_OK;
}

int dgpu_aver_combine(dgpu_ctx *ctx, const FormSpec &fs, const BoxSpec &box, const PartRef &apart,
                      const int32_t *istl, const double2 *cfact, const double2 *lat,
                      int32_t lat_nslice, int32_t lat_closed, const int32_t icc[3],
                      const double dim0[3], double norm, double2 *acsf)
{
    FormSpec *d;
    int rc = upload_formspec(ctx, fs, &d);
    if (rc) return rc;
    const PartLayout lay = dgpu_part_layout(apart, box);
    const unsigned nblk = (unsigned)dgpu_cdiv(lay.nthr, 256);
    if (apart.f32)
        k_aver_combine<float2><<<nblk, 256, 0, ctx->stream>>>(
            d, box, (const float2 *)apart.p, apart.nslice, lay, istl, cfact, lat, lat_nslice, lat_closed, icc[0],
            icc[1], icc[2], dim0[0], dim0[1], dim0[2], norm, acsf);
    else
        k_aver_combine<double2><<<nblk, 256, 0, ctx->stream>>>(
            d, box, (const double2 *)apart.p, apart.nslice, lay, istl, cfact, lat, lat_nslice, lat_closed, icc[0],
            icc[1], icc[2], dim0[0], dim0[1], dim0[2], norm, acsf);
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}

int dgpu_friedel_mirror(dgpu_ctx *ctx, const BoxSpec &box, int32_t idim, double2 *csf, double2 *acsf,
                        double *dsi)
{
    if (idim < 1 || idim > 3) return DGPU_OK;
    int64_t np = (int64_t)box.num[0] * box.num[1] * box.num[2];
    k_mirror<<<(unsigned)dgpu_cdiv(np, 256), 256, 0, ctx->stream>>>(box, idim - 1, csf, acsf, dsi);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_qinfo(dgpu_ctx *ctx, const double eck[3], const double vi[9], const int32_t num[3],
               const double *dsi, double res[7])
{
    FormSpec fs;
    memset(&fs, 0, sizeof(fs));
    memcpy(fs.vi, vi, sizeof(fs.vi));
    FormSpec *d;
    int rc = upload_formspec(ctx, fs, &d);
    if (rc) return rc;
    QStat *parts = (QStat *)((char *)ctx->stats.p + ((sizeof(FormSpec) + 63) & ~(size_t)63));
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    int nblk = (int)(dgpu_cdiv(np, QNT) < 1024 ? dgpu_cdiv(np, QNT) : 1024);
    if (nblk < 1) nblk = 1;
    DGPU_CUDA(ctx, ctx->flag.ensure(64 + 7 * sizeof(double)));
    double *d_res = (double *)((char *)ctx->flag.p + 64);
    k_qinfo_part<<<nblk, QNT, 0, ctx->stream>>>(eck[0], eck[1], eck[2], d, num[0], num[1], num[2], dsi, parts);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_qinfo_final<<<1, QNT, 0, ctx->stream>>>(parts, nblk, d_res);
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaMemcpyAsync(res, d_res, 7 * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}

// enqueue-only combine: FormSpec already in device memory
int dgpu_combine_async(dgpu_ctx *ctx, const FormSpec *d_fs, const BoxSpec &box, const PartRef &part,
                       const int32_t *istl, const double2 *cfact, double2 *csf, double *dsi, double diff_scale)
{
    const PartLayout lay = dgpu_part_layout(part, box);
    const unsigned nblk = (unsigned)dgpu_cdiv(lay.nthr, 256);
    if (part.f32)
        k_combine<float2><<<nblk, 256, 0, ctx->stream>>>(d_fs, box, (const float2 *)part.p, part.nslice, lay, istl,
                                                          cfact, nullptr, csf, dsi, diff_scale, sqrt(diff_scale));
    else
        k_combine<double2><<<nblk, 256, 0, ctx->stream>>>(d_fs, box, (const double2 *)part.p, part.nslice, lay,
                                                           istl, cfact, nullptr, csf, dsi, diff_scale,
                                                           sqrt(diff_scale));
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

// ---------------------------------------------------------------------------
// Lots (fourier_sup.f90:136-277).  The group factors do not depend on the
// lot: they are tabulated once per run on the box, fac[(g-1)*nb + box point].
__global__ void k_group_factors(const FormSpec *fs, BoxSpec box, const int32_t *__restrict__ istl,
                                const double2 *__restrict__ cfact, double2 *__restrict__ fac)
{
    const int64_t pb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    if (pb >= nb) return;
    const int64_t i = pb % box.f[0], j = (pb / box.f[0]) % box.f[1], l = pb / ((int64_t)box.f[0] * box.f[1]);
    const int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    double h[3];
    if (form_needs_h(fs)) form_hvec(fs, i, j, l, h);
    const int32_t q = istl ? istl[idx] : 0;
    for (int g = 1; g <= fs->ngroup; g++) fac[(int64_t)(g - 1) * nb + pb] = form_group(fs, cfact, q, g, h);
}

// One chunk of nlot lots whose partial sums come as nlot*ngroup types (lot-
// major): dsi += sum_L |sum_g fac_g S_{L,g} - acsf|^2 (unscaled) and, for the
// chunk's lot `last` (-1: none), csf = its F - acsf (unscaled).  part == null:
// the chunk has no atoms.
template <class P>
__global__ void k_lot_combine(int32_t ngroup, int32_t nlot, BoxSpec box, const P *__restrict__ part,
                              int32_t nslice, PartLayout lay, const double2 *__restrict__ fac,
                              const double2 *__restrict__ acsf, double2 *__restrict__ csf,
                              double *__restrict__ dsi, int32_t last)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i, j, l;
    if (r >= lay.nthr || !part_point(lay, box, r, i, j, l)) return;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    const int64_t pb = i + (int64_t)box.f[0] * (j + (int64_t)box.f[1] * l);
    const int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    const double2 a = acsf ? acsf[idx] : make_double2(0.0, 0.0);
    const int64_t off = i * lay.s0 + j * lay.s1 + l * lay.s2;
    double acc = 0.0;
    if constexpr (sizeof(P) == sizeof(float2)) {
        // FP32 partials (tensor-core engine): the group products in FP32 --
        // the partials carry FP32 rounding already -- with the group factors
        // of the point loaded once; F - <F> and |.|^2 in FP64
        constexpr int GMAX = 8;
        float2 fg[GMAX];
#pragma unroll
        for (int g = 0; g < GMAX; g++) {
            const double2 f = g < ngroup ? fac[(int64_t)g * nb + pb] : make_double2(0.0, 0.0);
            fg[g] = make_float2((float)f.x, (float)f.y);
        }
        for (int L = 0; L < nlot; L++) {
            float fr = 0.f, fi = 0.f;
            if (part)
                for (int g = 0; g < ngroup; g++) {
                    const P *pt = part + (int64_t)(L * ngroup + g) * nslice * lay.slab + off;
                    float sr = 0.f, si = 0.f;
                    for (int k = 0; k < nslice; k++) {
                        const float2 v = *reinterpret_cast<const float2 *>(pt + (int64_t)k * lay.slab);
                        sr += v.x;
                        si += v.y;
                    }
                    float2 f;
                    if (g < GMAX) f = fg[g];
                    else {
                        const double2 fd = fac[(int64_t)g * nb + pb];
                        f = make_float2((float)fd.x, (float)fd.y);
                    }
                    fr = fmaf(sr, f.x, fmaf(-si, f.y, fr));
                    fi = fmaf(sr, f.y, fmaf(si, f.x, fi));
                }
            const double2 F = make_double2((double)fr - a.x, (double)fi - a.y);
            acc += F.x * F.x + F.y * F.y;
            if (L == last) csf[idx] = F;
        }
    } else {
        for (int L = 0; L < nlot; L++) {
            double2 F = make_double2(0.0, 0.0);
            if (part)
                for (int g = 0; g < ngroup; g++) {
                    const P *pt = part + (int64_t)(L * ngroup + g) * nslice * lay.slab + off;
                    double2 s = make_double2(0.0, 0.0);
                    for (int k = 0; k < nslice; k++) {
                        const double2 v = ld_part(pt + (int64_t)k * lay.slab);
                        s.x += v.x;
                        s.y += v.y;
                    }
                    const double2 m = cmul(s, fac[(int64_t)g * nb + pb]);
                    F.x += m.x;
                    F.y += m.y;
                }
            F.x -= a.x;
            F.y -= a.y;
            acc += F.x * F.x + F.y * F.y;
            if (L == last) csf[idx] = F;
        }
    }
    dsi[idx] += acc;
}

// k_lot_combine for FP32 partials with nq = ngroup * nslice partials per lot
// known at compile time: partial q = g * nslice + k of lot L sits at
// (L * NQ + q) * slab, and LB lots' partials are loaded before any is used,
// so that each thread keeps about eight loads in flight (the kernel reads
// nlot * nq partials per point and is bound by those reads).  The arithmetic
// is the generic kernel's, operation for operation: a group's slices are
// added first, then multiplied by its factor.  Without <F> (AV false) F of a
// lot is an FP32 pair and |F|^2 is summed over the lots in float-float (exact
// FMA products, TwoSum, 48-bit significands) rather than FP64, whose rate on
// this part made that sum the kernel's bound; F - <F> keeps FP64.
template <int NQ, bool AV>
__global__ void k_lot_combine_f32(int32_t nslice, int32_t nlot, BoxSpec box, const float2 *__restrict__ part,
                                  PartLayout lay, const double2 *__restrict__ fac, const double2 *__restrict__ acsf,
                                  double2 *__restrict__ csf, double *__restrict__ dsi, int32_t last)
{
    constexpr int LB = NQ >= 8 ? 1 : 8 / NQ;
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    int64_t i, j, l;
    if (r >= lay.nthr || !part_point(lay, box, r, i, j, l)) return;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    const int64_t pb = i + (int64_t)box.f[0] * (j + (int64_t)box.f[1] * l);
    const int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    const double2 a = AV ? acsf[idx] : make_double2(0.0, 0.0);
    const float2 *p0 = part + i * lay.s0 + j * lay.s1 + l * lay.s2;
    const int64_t slab = lay.slab;
    float2 fq[NQ];                         // the group factor of each partial of a lot
#pragma unroll
    for (int q = 0; q < NQ; q++) {
        const double2 f = fac[(int64_t)(q / nslice) * nb + pb];
        fq[q] = make_float2((float)f.x, (float)f.y);
    }
    double acc = 0.0;
    float ah = 0.f, al = 0.f;              // float-float sum of |F|^2 (AV false)
    for (int L0 = 0; L0 < nlot; L0 += LB) {
        float2 v[LB][NQ];
#pragma unroll
        for (int b = 0; b < LB; b++)
#pragma unroll
            for (int q = 0; q < NQ; q++)
                v[b][q] = L0 + b < nlot ? __ldg(p0 + ((int64_t)(L0 + b) * NQ + q) * slab) : make_float2(0.f, 0.f);
#pragma unroll
        for (int b = 0; b < LB; b++) {
            if (L0 + b < nlot) {
                // the slices of a group added first (in slice order), then the
                // group product: the generic kernel's arithmetic
                float fr = 0.f, fi = 0.f, sr = 0.f, si = 0.f;
#pragma unroll
                for (int q = 0; q < NQ; q++) {
                    sr += v[b][q].x;
                    si += v[b][q].y;
                    if ((q + 1) % nslice == 0) {
                        fr = fmaf(sr, fq[q].x, fmaf(-si, fq[q].y, fr));
                        fi = fmaf(sr, fq[q].y, fmaf(si, fq[q].x, fi));
                        sr = 0.f;
                        si = 0.f;
                    }
                }
                if (AV) {
                    const double2 F = make_double2((double)fr - a.x, (double)fi - a.y);
                    acc += F.x * F.x + F.y * F.y;
                    if (L0 + b == last) csf[idx] = F;
                } else {
                    const float pr = fr * fr, pi = fi * fi;
                    const float er = fmaf(fr, fr, -pr), ei = fmaf(fi, fi, -pi);   // exact product errors
                    ff_add(ah, al, pr);
                    ff_add(ah, al, pi);
                    al += er + ei;
                    if (L0 + b == last) csf[idx] = make_double2((double)fr, (double)fi);
                }
            }
        }
    }
    dsi[idx] += AV ? acc : (double)ah + (double)al;
}

// dsi *= dscale, csf *= cscale on the box (lot normalisation and diff_scale)
__global__ void k_lot_scale(BoxSpec box, double2 *__restrict__ csf, double *__restrict__ dsi, double dscale,
                            double cscale)
{
    const int64_t pb = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    if (pb >= nb) return;
    const int64_t i = pb % box.f[0], j = (pb / box.f[0]) % box.f[1], l = pb / ((int64_t)box.f[0] * box.f[1]);
    const int64_t idx = i + (int64_t)box.num[0] * (j + (int64_t)box.num[1] * l);
    dsi[idx] *= dscale;
    const double2 c = csf[idx];
    csf[idx] = make_double2(c.x * cscale, c.y * cscale);
}

int dgpu_group_factors(dgpu_ctx *ctx, const FormSpec &fs, const BoxSpec &box, const int32_t *istl,
                       const double2 *cfact, double2 *fac)
{
    FormSpec *d;
    int rc = upload_formspec(ctx, fs, &d);
    if (rc) return rc;
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    k_group_factors<<<(unsigned)dgpu_cdiv(nb, 256), 256, 0, ctx->stream>>>(d, box, istl, cfact, fac);
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));   // FormSpec block reused next
    return DGPU_OK;
}

int dgpu_lot_combine(dgpu_ctx *ctx, int32_t ngroup, int32_t nlot, const BoxSpec &box, const PartRef *part,
                     const double2 *fac, const double2 *acsf, double2 *csf, double *dsi, int32_t last)
{
    PartRef none;
    memset(&none, 0, sizeof(none));
    const PartRef &r = part ? *part : none;
    const PartLayout lay = dgpu_part_layout(r, box);
    const unsigned nblk = (unsigned)dgpu_cdiv(lay.nthr, 256);
    const int32_t nslice = r.nslice > 0 ? r.nslice : 1;
    const int32_t nq = ngroup * nslice;
    if (r.f32 && r.p && nq >= 1 && nq <= 8) {
        const float2 *p = (const float2 *)r.p;
        switch (nq) {
#define LOT_F32(Q)                                                                                              \
    case Q:                                                                                                     \
        if (acsf)                                                                                               \
            k_lot_combine_f32<Q, true><<<nblk, 256, 0, ctx->stream>>>(nslice, nlot, box, p, lay, fac, acsf, csf,  \
                                                                      dsi, last);                               \
        else                                                                                                    \
            k_lot_combine_f32<Q, false><<<nblk, 256, 0, ctx->stream>>>(nslice, nlot, box, p, lay, fac, acsf, csf, \
                                                                       dsi, last);                              \
        break;
            LOT_F32(1) LOT_F32(2) LOT_F32(3) LOT_F32(4) LOT_F32(5) LOT_F32(6) LOT_F32(7) LOT_F32(8)
#undef LOT_F32
        }
    } else if (r.f32)
        k_lot_combine<float2><<<nblk, 256, 0, ctx->stream>>>(ngroup, nlot, box, (const float2 *)r.p, nslice, lay,
                                                              fac, acsf, csf, dsi, last);
    else
        k_lot_combine<double2><<<nblk, 256, 0, ctx->stream>>>(ngroup, nlot, box, (const double2 *)r.p, nslice,
                                                               lay, fac, acsf, csf, dsi, last);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_lot_scale(dgpu_ctx *ctx, const BoxSpec &box, double2 *csf, double *dsi, double dscale, double cscale)
{
    const int64_t nb = (int64_t)box.f[0] * box.f[1] * box.f[2];
    k_lot_scale<<<(unsigned)dgpu_cdiv(nb, 256), 256, 0, ctx->stream>>>(box, csf, dsi, dscale, cscale);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}
