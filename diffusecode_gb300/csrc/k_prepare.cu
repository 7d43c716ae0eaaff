// Atom preparation and lookup tables.
//
//  * per-atom phase data: the reference's integer increments
//    (discus/prog/four_strucf_OMP_mod.f90:135-149, REF22) or an exact 64-bit
//    fixed-point h.r mod 1 (EXACT64), gathered by type in a stable order
//    (four_getatm LOT_OFF, discus/prog/fourier_sup.f90:1839-1848) or folded
//    into the unit cell for <F> (four_aver, fourier_sup.f90:1243-1281);
//  * istl (four_stltab, fourier_sup.f90:2637-2687) and cfact
//    (four_formtab, fourier_sup.f90:2691-2743) on the device.
#include <vector>

#include "dgpu_internal.h"

#define PREP_BLK 1024
#define MAXT 64

// ---------------------------------------------------------------------------
// phase arithmetic

// a*x products and sums kept unfused: the reference's xinc = u1*x1+u2*x2+u3*x3
__device__ __forceinline__ double dot3_nc(const double *a, double x0, double x1, double x2)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], x0), __dmul_rn(a[1], x1)), __dmul_rn(a[2], x2));
}

// NINT(64*I2PI*(x - INT(x) + 0)) : the 2^22 increment of one atom
__device__ __forceinline__ int64_t inc22(double x)
{
    double fr = __dadd_rn(__dsub_rn(x, trunc(x)), 0.0);
    return (int64_t)llround(__dmul_rn(4194304.0, fr));
}

// frac(a x) as a 64-bit fixed-point turn, exactly (truncated to 2^-64): the
// two 53-bit significands are multiplied as integers (106-bit product) and
// shifted by the exponents; a negative product is negated modulo 2^64.
// Integer arithmetic, because this part's FP64 rate is low.
__device__ __forceinline__ uint64_t fx64_mul(double a, double x)
{
    const uint64_t ba = (uint64_t)__double_as_longlong(a), bx = (uint64_t)__double_as_longlong(x);
    const int ea = (int)((ba >> 52) & 0x7FF), ex = (int)((bx >> 52) & 0x7FF);
    const uint64_t ma = (ba & 0xFFFFFFFFFFFFFull) | (ea ? (1ull << 52) : 0ull);
    const uint64_t mx = (bx & 0xFFFFFFFFFFFFFull) | (ex ? (1ull << 52) : 0ull);
    // a x = ma mx 2^(e_a + e_x); the fixed point wants that times 2^64, modulo 2^64
    const int s = (ea ? ea - 1075 : -1074) + (ex ? ex - 1075 : -1074) + 64;
    const uint64_t lo = ma * mx, hi = __umul64hi(ma, mx);
    uint64_t r;
    if (s >= 64) r = 0;
    else if (s >= 0) r = lo << s;
    else if (s > -64) r = (lo >> -s) | (hi << (64 + s));
    else if (s > -128) r = hi >> (-s - 64);
    else r = 0;
    return ((ba ^ bx) >> 63) ? 0ull - r : r;
}

// frac(a.x) as a 64-bit fixed-point turn (the sum of the three exact terms
// modulo one turn)
__device__ __forceinline__ uint64_t frac64_dot(const double *a, double x0, double x1, double x2)
{
    return fx64_mul(a[0], x0) + fx64_mul(a[1], x1) + fx64_mul(a[2], x2);
}

struct PhaseOut {
    uint64_t ph0, du, dv, dw;
};

__device__ __forceinline__ PhaseOut atom_phase(const PhaseGeom &g, double x0, double x1, double x2)
{
    PhaseOut o;
    if (g.mode == DGPU_PHASE_REF22) {
        int64_t iu = inc22(dot3_nc(g.vi + 0, x0, x1, x2));
        int64_t iv = inc22(dot3_nc(g.vi + 3, x0, x1, x2));
        int64_t iw = inc22(dot3_nc(g.vi + 6, x0, x1, x2));
        int64_t ju = inc22(dot3_nc(g.off + 0, x0, x1, x2));
        int64_t jv = inc22(dot3_nc(g.off + 3, x0, x1, x2));
        int64_t jw = inc22(dot3_nc(g.off + 6, x0, x1, x2));
        int64_t base = (int64_t)g.lmn[0] * iu + (int64_t)g.lmn[1] * iv + (int64_t)g.lmn[2] * iw
                     + (int64_t)g.lmn[3] * ju + (int64_t)g.lmn[4] * jv + (int64_t)g.lmn[5] * jw;
        // unit 2^-22 turn -> 2^-64 turn; bits 6..21 of iarg become bits 48..63
        o.ph0 = (uint64_t)base << 42;
        o.du = (uint64_t)iu << 42;
        o.dv = (uint64_t)iv << 42;
        o.dw = (uint64_t)iw << 42;
    } else {
        o.ph0 = frac64_dot(g.eck, x0, x1, x2);
        o.du = frac64_dot(g.vi + 0, x0, x1, x2);
        o.dv = frac64_dot(g.vi + 3, x0, x1, x2);
        o.dw = frac64_dot(g.vi + 6, x0, x1, x2);
    }
    return o;
}

// effective type of atom i: 0 = not summed
__device__ __forceinline__ int eff_type(const int32_t *iscat, int64_t i, int64_t n, int32_t nscat,
                                        const FoldSpec &fs)
{
    if (i >= n) return 0;
    int t = iscat[i];
    if (t < 1 || t > nscat) return 0;
    if (fs.fold) {
        int64_t ncell = (int64_t)fs.icc[0] * fs.icc[1] * fs.icc[2];
        if (i >= ncell * fs.ncatoms) return 0;     // only atoms in DISCUS cell order
        int64_t c = i / fs.ncatoms;
        if (fs.sel && !fs.sel[c]) return 0;
    }
    return t;
}

// block bx of the per-(type, block) counts
__device__ __forceinline__ void type_count_body(const int32_t *iscat, int64_t n, int32_t nscat, const FoldSpec &fs,
                                                int32_t *counts, int64_t nblk, int64_t bx)
{
    __shared__ int32_t hist[MAXT];
    for (int t = threadIdx.x; t < MAXT; t += blockDim.x) hist[t] = 0;
    __syncthreads();
    int64_t i = bx * PREP_BLK + threadIdx.x;
    int t = eff_type(iscat, i, n, nscat, fs);
    if (t) atomicAdd(&hist[t], 1);
    __syncthreads();
    for (int tt = threadIdx.x; tt < nscat; tt += blockDim.x)
        counts[(int64_t)tt * nblk + bx] = hist[tt + 1];
}

__global__ void k_type_count(const int32_t *iscat, int64_t n, int32_t nscat, FoldSpec fs,
                             int32_t *counts, int64_t nblk)
{
    type_count_body(iscat, n, nscat, fs, counts, nblk, blockIdx.x);
}

// Exclusive scan of the per-(type, block) counts into int64 offsets, one CTA.
// Each type's range starts on a multiple of TYPE_ALIGN atoms; the gap after a
// type is padding (zero phase, zero weight) so that every 64-atom group of a
// type (one tensor-core stage) is aligned and complete.
#define TYPE_ALIGN 64
__device__ __forceinline__ void scan_counts_body(const int32_t *counts, int64_t *offs, int64_t nblk,
                                                 int32_t nscat, int64_t *type_start)
{
    __shared__ int64_t warp_sums[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int t = 0; t < nscat; t++) {
        if (threadIdx.x == 0) {
            carry = (carry + TYPE_ALIGN - 1) / TYPE_ALIGN * TYPE_ALIGN;
            type_start[t] = carry;
        }
        __syncthreads();
        const int64_t seg = (int64_t)t * nblk;
        for (int64_t base = 0; base < nblk; base += blockDim.x) {
            int64_t i = base + threadIdx.x;
            int64_t v = i < nblk ? counts[seg + i] : 0;
            int64_t x = v;
            for (int o = 1; o < 32; o <<= 1) {
                int64_t y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane == 31) warp_sums[wid] = x;
            __syncthreads();
            if (wid == 0) {
                int64_t s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
                for (int o = 1; o < 32; o <<= 1) {
                    int64_t y = __shfl_up_sync(0xffffffffu, s, o);
                    if (lane >= o) s += y;
                }
                warp_sums[lane] = s;
            }
            __syncthreads();
            int64_t incl = x + (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
            if (i < nblk) offs[seg + i] = incl - v;
            __syncthreads();
            if (threadIdx.x == blockDim.x - 1) carry = incl;
            __syncthreads();
        }
        if (threadIdx.x == 0) type_start[nscat + 1 + t] = carry - type_start[t];   // real atoms of type t
        __syncthreads();
    }
    if (threadIdx.x == 0) type_start[nscat] = (carry + TYPE_ALIGN - 1) / TYPE_ALIGN * TYPE_ALIGN;
}

__global__ void k_scan_counts(const int32_t *counts, int64_t len, int64_t *offs,
                              int64_t nblk, int32_t nscat, int64_t *type_start)
{
    scan_counts_body(counts, offs, nblk, nscat, type_start);
    (void)len;
}

// A fixed pseudo-random bijection of [0, n): a four-round Feistel network on
// the smallest even number of bits that covers n, cycle-walked back into
// [0, n).  The atoms of a type are summed in this order rather than in the
// crystal's: every K slice and every accumulator chain of the engines is then
// a random sample of the crystal, so a partial sum is large only where the
// whole sum is (near a Bragg position, atoms stored cell after cell give
// partial sums that are coherent and cancel only in the total).
__device__ __forceinline__ uint32_t slot_perm(uint32_t x, uint32_t n)
{
    if (n <= 2) return x;
    int b = 32 - __clz(n - 1);
    b += b & 1;
    const int h = b >> 1;
    const uint32_t m = (1u << h) - 1u;
    do {
        uint32_t l = x >> h, r = x & m;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            uint32_t f = r * 0x9E3779B1u + 0x85EBCA77u * (uint32_t)(k + 1);
            f ^= f >> 15;
            f *= 0x2C1B3C6Du;
            f ^= f >> 12;
            const uint32_t t = r;
            r = l ^ (f & m);
            l = t;
        }
        x = (l << h) | r;
    } while (x >= n);
    return x;
}

__device__ __forceinline__ void scatter_atoms_body(const double *pos, const int32_t *iscat, const float *aocc,
                                                   int64_t n, int32_t nscat, const FoldSpec &fs, const PhaseGeom &g,
                                                   const int64_t *offs, int64_t nblk, const int64_t *ts,
                                                   uint64_t *ph0, uint64_t *du, uint64_t *dv, uint64_t *dw,
                                                   float *w, int32_t *idx, int64_t bx)
{
    __shared__ int32_t wcnt[32][MAXT];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < 32 * MAXT; k += blockDim.x) (&wcnt[0][0])[k] = 0;
    __syncthreads();
    int64_t i = bx * PREP_BLK + threadIdx.x;
    int t = eff_type(iscat, i, n, nscat, fs);
    unsigned same = __match_any_sync(0xffffffffu, t);
    int rank = __popc(same & ((1u << lane) - 1u));
    if (t && rank == 0) wcnt[wid][t] = __popc(same);
    __syncthreads();
    // exclusive prefix over warps, per type (one thread per type)
    if (threadIdx.x >= 1 && threadIdx.x <= nscat) {
        int tt = threadIdx.x, run = 0;
        for (int ww = 0; ww < 32; ww++) {
            int c = wcnt[ww][tt];
            wcnt[ww][tt] = run;
            run += c;
        }
    }
    __syncthreads();
    if (!t) return;
    // stable rank within the type, then the type's summation order
    const int64_t rk = offs[(int64_t)(t - 1) * nblk + bx] + wcnt[wid][t] + rank - ts[t - 1];
    const int64_t dst = ts[t - 1] + slot_perm((uint32_t)rk, (uint32_t)ts[nscat + t]);
    double x0 = pos[3 * i], x1 = pos[3 * i + 1], x2 = pos[3 * i + 2];
    if (fs.fold) {
        int64_t c = i / fs.ncatoms;
        int64_t ci = c % fs.icc[0];
        int64_t cj = (c / fs.icc[0]) % fs.icc[1];
        int64_t ck = c / ((int64_t)fs.icc[0] * fs.icc[1]);
        // xat = cr_pos - (icell-1) - cr_dim0 (fourier_sup.f90:1272-1281)
        x0 = __dsub_rn(__dsub_rn(x0, (double)ci), fs.dim0[0]);
        x1 = __dsub_rn(__dsub_rn(x1, (double)cj), fs.dim0[1]);
        x2 = __dsub_rn(__dsub_rn(x2, (double)ck), fs.dim0[2]);
    }
    PhaseOut o = atom_phase(g, x0, x1, x2);
    ph0[dst] = o.ph0;
    du[dst] = o.du;
    dv[dst] = o.dv;
    dw[dst] = o.dw;
    w[dst] = aocc ? aocc[i] : 1.0f;
    idx[dst] = (int32_t)i;
}

__global__ void k_scatter_atoms(const double *pos, const int32_t *iscat, const float *aocc,
                                int64_t n, int32_t nscat, FoldSpec fs, PhaseGeom g,
                                const int64_t *offs, int64_t nblk, const int64_t *ts, uint64_t *ph0,
                                uint64_t *du, uint64_t *dv, uint64_t *dw, float *w, int32_t *idx)
{
    scatter_atoms_body(pos, iscat, aocc, n, nscat, fs, g, offs, nblk, ts, ph0, du, dv, dw, w, idx, blockIdx.x);
}

size_t dgpu_prepare_region_bytes(int64_t natoms, int32_t nscat)
{
    const int64_t nblk = natoms > PREP_BLK ? dgpu_cdiv(natoms, PREP_BLK) : 1;
    const size_t cnt = ((size_t)(nblk * nscat) * sizeof(int32_t) + 255) & ~(size_t)255;
    const size_t off = ((size_t)(nblk * nscat) * sizeof(int64_t) + 255) & ~(size_t)255;
    return cnt + off + (((2 * MAXT + 4) * sizeof(int64_t) + 255) & ~(size_t)255);
}

PrepRegion dgpu_prepare_region(void *base, int64_t natoms, int32_t nscat)
{
    PrepRegion r;
    r.nblk = natoms > PREP_BLK ? dgpu_cdiv(natoms, PREP_BLK) : 1;
    const size_t cnt = ((size_t)(r.nblk * nscat) * sizeof(int32_t) + 255) & ~(size_t)255;
    const size_t off = ((size_t)(r.nblk * nscat) * sizeof(int64_t) + 255) & ~(size_t)255;
    r.counts = (int32_t *)base;
    r.offs = (int64_t *)((char *)base + cnt);
    r.d_ts = (int64_t *)((char *)base + cnt + off);
    return r;
}

int dgpu_prepare_count(dgpu_ctx *ctx, const int32_t *d_iscat, int64_t natoms, int32_t nscat, const FoldSpec &fs,
                       const PrepRegion &r)
{
    if (nscat < 1 || nscat >= MAXT)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "nscat=%d outside 1..%d", nscat, MAXT - 1);
    k_type_count<<<(unsigned)r.nblk, PREP_BLK, 0, ctx->stream>>>(d_iscat, natoms, nscat, fs, r.counts, r.nblk);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_scan_counts<<<1, 1024, 0, ctx->stream>>>(r.counts, r.nblk * nscat, r.offs, r.nblk, nscat, r.d_ts);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_prepare_scatter(dgpu_ctx *ctx, const double *d_pos, const int32_t *d_iscat, const float *d_aocc,
                         int64_t natoms, int32_t nscat, const PhaseGeom &g, const FoldSpec &fs, const PrepRegion &r,
                         int64_t total, DevBuf &ph0, DevBuf &du, DevBuf &dv, DevBuf &dw, DevBuf &w,
                         DevBuf *idx)
{
    DevBuf &ib = idx ? *idx : ctx->aidx;
    size_t cap = (size_t)(total > 0 ? total : 1);
    DGPU_CUDA(ctx, ph0.ensure(cap * 8));
    DGPU_CUDA(ctx, du.ensure(cap * 8));
    DGPU_CUDA(ctx, dv.ensure(cap * 8));
    DGPU_CUDA(ctx, dw.ensure(cap * 8));
    DGPU_CUDA(ctx, w.ensure(cap * 4));
    // padding slots: phase 0, weight 0
    DGPU_CUDA(ctx, cudaMemsetAsync(ph0.p, 0, cap * 8, ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(du.p, 0, cap * 8, ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(dv.p, 0, cap * 8, ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(dw.p, 0, cap * 8, ctx->stream));
    DGPU_CUDA(ctx, cudaMemsetAsync(w.p, 0, cap * 4, ctx->stream));
    DGPU_CUDA(ctx, ib.ensure(cap * 4));
    DGPU_CUDA(ctx, cudaMemsetAsync(ib.p, 0xFF, cap * 4, ctx->stream));   // padding: -1
    k_scatter_atoms<<<(unsigned)r.nblk, PREP_BLK, 0, ctx->stream>>>(
        d_pos, d_iscat, d_aocc, natoms, nscat, fs, g, r.offs, r.nblk, r.d_ts, ph0.as<uint64_t>(),
        du.as<uint64_t>(), dv.as<uint64_t>(), dw.as<uint64_t>(), w.as<float>(), ib.as<int32_t>());
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_prepare_atoms(dgpu_ctx *ctx, const double *d_pos, const int32_t *d_iscat,
                       const float *d_aocc, int64_t natoms, int32_t nscat, const PhaseGeom &g,
                       const FoldSpec &fs, DevBuf &ph0, DevBuf &du, DevBuf &dv, DevBuf &dw,
                       DevBuf &w, int64_t *h_type_start, DevBuf *idx)
{
    if (nscat < 1 || nscat >= MAXT)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "nscat=%d outside 1..%d", nscat, MAXT - 1);
    DGPU_CUDA(ctx, ctx->counts.ensure(dgpu_prepare_region_bytes(natoms, nscat)));
    const PrepRegion r = dgpu_prepare_region(ctx->counts.p, natoms, nscat);
    int rc = dgpu_prepare_count(ctx, d_iscat, natoms, nscat, fs, r);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaMemcpyAsync(h_type_start, r.d_ts, (2 * nscat + 1) * sizeof(int64_t),
                                   cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return dgpu_prepare_scatter(ctx, d_pos, d_iscat, d_aocc, natoms, nscat, g, fs, r, h_type_start[nscat], ph0, du,
                                dv, dw, w, idx);
}

__global__ void k_lattice(int64_t ncell, int32_t i0, int32_t i1, double d0, double d1, double d2,
                          PhaseGeom g, uint64_t *ph0, uint64_t *du, uint64_t *dv, uint64_t *dw,
                          float *w)
{
    int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncell) return;
    int64_t ii = c % i0, jj = (c / i0) % i1, kk = c / ((int64_t)i0 * i1);
    // four_getav LOT_OFF: xat = (ii,jj,kk) + cr_dim0 (fourier_sup.f90:2457-2466)
    double x0 = __dadd_rn((double)ii, d0), x1 = __dadd_rn((double)jj, d1), x2 = __dadd_rn((double)kk, d2);
    PhaseOut o = atom_phase(g, x0, x1, x2);
    ph0[c] = o.ph0;
    du[c] = o.du;
    dv[c] = o.dv;
    dw[c] = o.dw;
    w[c] = 1.0f;
}

int dgpu_prepare_lattice(dgpu_ctx *ctx, const int32_t icc[3], const double dim0[3],
                         const PhaseGeom &g, DevBuf &ph0, DevBuf &du, DevBuf &dv, DevBuf &dw,
                         DevBuf &w)
{
    int64_t ncell = (int64_t)icc[0] * icc[1] * icc[2];
    DGPU_CUDA(ctx, ph0.ensure(ncell * 8));
    DGPU_CUDA(ctx, du.ensure(ncell * 8));
    DGPU_CUDA(ctx, dv.ensure(ncell * 8));
    DGPU_CUDA(ctx, dw.ensure(ncell * 8));
    DGPU_CUDA(ctx, w.ensure(ncell * 4));
    k_lattice<<<(unsigned)dgpu_cdiv(ncell, 256), 256, 0, ctx->stream>>>(
        ncell, icc[0], icc[1], dim0[0], dim0[1], dim0[2], g, ph0.as<uint64_t>(),
        du.as<uint64_t>(), dv.as<uint64_t>(), dw.as<uint64_t>(), w.as<float>());
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

// ---------------------------------------------------------------------------
// tables

// istl(i,j,l) = NINT(sqrt(h.G*.h/4)/CFINC) with h rounded to REAL(4)
// istl of grid point p; e = eck(:,1), r = rten column-major
__device__ __forceinline__ void stltab_point(const double *e, const double *vi, int32_t n0, int32_t n1, int32_t n2,
                                             const double *r, int32_t *istl, int32_t *flag, int64_t p)
{
    int64_t np = (int64_t)n0 * n1 * n2;
    if (p >= np) return;
    int64_t i = p % n0, j = (p / n0) % n1, l = p / ((int64_t)n0 * n1);
    const double r00 = r[0], r10 = r[1], r20 = r[2], r01 = r[3], r11 = r[4], r21 = r[5], r02 = r[6], r12 = r[7],
                 r22 = r[8];
    double h[3];
    for (int k = 0; k < 3; k++) {
        double s = __dadd_rn(__dadd_rn(__dadd_rn(e[k], __dmul_rn(vi[k], (double)i)),
                                       __dmul_rn(vi[3 + k], (double)j)),
                             __dmul_rn(vi[6 + k], (double)l));
        h[k] = (double)__double2float_rn(s);
    }
    double t0 = __dadd_rn(__dadd_rn(__dmul_rn(r00, h[0]), __dmul_rn(r01, h[1])), __dmul_rn(r02, h[2]));
    double t1 = __dadd_rn(__dadd_rn(__dmul_rn(r10, h[0]), __dmul_rn(r11, h[1])), __dmul_rn(r12, h[2]));
    double t2 = __dadd_rn(__dadd_rn(__dmul_rn(r20, h[0]), __dmul_rn(r21, h[1])), __dmul_rn(r22, h[2]));
    double q = __dadd_rn(__dadd_rn(__dmul_rn(h[0], t0), __dmul_rn(h[1], t1)), __dmul_rn(h[2], t2));
    double q2 = q / 4.0;
    long long v = llround(__dmul_rn(__dsqrt_rn(q2), 1000.0));
    istl[p] = (int32_t)v;
    if (v > DGPU_CFPKT) atomicExch(flag, 1);
}

__global__ void k_stltab(double e0, double e1, double e2, PhaseGeom vg, int32_t n0, int32_t n1,
                         int32_t n2, double r00, double r10, double r20, double r01, double r11,
                         double r21, double r02, double r12, double r22, int32_t *istl,
                         int32_t *flag)
{
    const double e[3] = {e0, e1, e2}, r[9] = {r00, r10, r20, r01, r11, r21, r02, r12, r22};
    stltab_point(e, vg.vi, n0, n1, n2, r, istl, flag, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

// the table in ctx's buffer p already holds what key describes
static bool tab_cached(const dgpu_ctx::TabKey &t, const DevBuf &b, const void *p, const std::vector<double> &key)
{
    return t.p == p && b.p == p && t.cap == b.cap && t.k == key;
}

int dgpu_stltab_dev(dgpu_ctx *ctx, const double eck[3], const double vi[9], const int32_t num[3],
                    const double rten[9], int32_t *d_istl)
{
    // the context's own table for the same grid and metric: already there
    std::vector<double> key(eck, eck + 3);
    key.insert(key.end(), vi, vi + 9);
    key.insert(key.end(), rten, rten + 9);
    for (int k = 0; k < 3; k++) key.push_back((double)num[k]);
    if (tab_cached(ctx->stl_key, ctx->istl, d_istl, key)) return DGPU_OK;
    ctx->stl_key.p = nullptr;
    int64_t np = (int64_t)num[0] * num[1] * num[2];
    DGPU_CUDA(ctx, ctx->flag.ensure(64));
    int32_t *flag = ctx->flag.as<int32_t>();
    DGPU_CUDA(ctx, cudaMemsetAsync(flag, 0, 4, ctx->stream));
    PhaseGeom vg;
    memset(&vg, 0, sizeof(vg));
    memcpy(vg.vi, vi, sizeof(vg.vi));
    k_stltab<<<(unsigned)dgpu_cdiv(np, 256), 256, 0, ctx->stream>>>(
        eck[0], eck[1], eck[2], vg, num[0], num[1], num[2], rten[0], rten[1], rten[2], rten[3],
        rten[4], rten[5], rten[6], rten[7], rten[8], d_istl, flag);
    DGPU_CUDA(ctx, cudaGetLastError());
    int32_t hflag = 0;
    DGPU_CUDA(ctx, cudaMemcpyAsync(&hflag, flag, 4, cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (hflag)
        return dgpu_set_error(ctx, DGPU_ERR_STL_RANGE,
                              "sin(theta)/lambda beyond the form-factor table (istl > %d)", DGPU_CFPKT);
    if (d_istl == ctx->istl.as<int32_t>()) {
        ctx->stl_key.p = d_istl;
        ctx->stl_key.cap = ctx->istl.cap;
        ctx->stl_key.k = key;
    }
    return DGPU_OK;
}

struct FormCoef {
    double scat[MAXT * 11];
    double occ[MAXT], dw[MAXT], delfr[MAXT], delfi[MAXT];
};

// cfact(iq,t) = sb*(f+f') + i sb*f'' ; f = c + sum_i a_i exp(-b_i s^2)
__device__ __forceinline__ void formtab_entry(const FormCoef *fc, int32_t nscat, int32_t lxray, int32_t power,
                                              int32_t ano, int32_t ldbw, double2 *cfact, int64_t k)
{
    if (k >= (int64_t)nscat * DGPU_NTAB) return;
    int t = (int)(k / DGPU_NTAB) + 1, iq = (int)(k % DGPU_NTAB);
    double s = __dmul_rn((double)iq, DGPU_CFINC);
    double q2 = __dmul_rn(s, s);
    const double *sc = fc->scat + 11 * t;
    double f = sc[0];
    if (lxray)
        for (int i = 1; i <= power; i++) f = __dadd_rn(f, __dmul_rn(sc[2 * i - 1], exp(-__dmul_rn(sc[2 * i], q2))));
    double fp = ano ? fc->delfr[t] : 0.0, fpp = ano ? fc->delfi[t] : 0.0;
    double sb = ldbw ? __dmul_rn(exp(-__dmul_rn(fc->dw[t], q2)), fc->occ[t]) : fc->occ[t];
    cfact[k] = make_double2(__dmul_rn(sb, __dadd_rn(f, fp)), __dmul_rn(sb, fpp));
}

__global__ void k_formtab(const FormCoef *fc, int32_t nscat, int32_t lxray, int32_t power,
                          int32_t ano, int32_t ldbw, double2 *cfact)
{
    formtab_entry(fc, nscat, lxray, power, ano, ldbw, cfact, (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

int dgpu_formtab_dev(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, double2 *d_cfact)
{
    if (cr->nscat < 1 || cr->nscat >= MAXT)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "nscat=%d outside 1..%d", cr->nscat, MAXT - 1);
    FormCoef h;
    memset(&h, 0, sizeof(h));
    for (int t = 0; t <= cr->nscat; t++) {
        for (int i = 0; i < 11; i++) h.scat[11 * t + i] = cr->scat[11 * t + i];
        h.occ[t] = cr->occ[t];
        h.dw[t] = cr->dw[t];
        h.delfr[t] = cr->delfr ? cr->delfr[t] : 0.0;
        h.delfi[t] = cr->delfi ? cr->delfi[t] : 0.0;
    }
    const int32_t ldbw = op->ldbw && !cr->is_anis;
    std::vector<double> key(reinterpret_cast<const double *>(&h),
                            reinterpret_cast<const double *>(&h) + (sizeof(h) / sizeof(double)));
    key.push_back(cr->nscat);
    key.push_back(op->lxray);
    key.push_back(op->power);
    key.push_back(op->ano);
    key.push_back(ldbw);
    if (tab_cached(ctx->cf_key, ctx->cfact, d_cfact, key)) return DGPU_OK;
    ctx->cf_key.p = nullptr;
    DGPU_CUDA(ctx, ctx->stats.ensure(sizeof(FormCoef)));
    FormCoef *d = ctx->stats.as<FormCoef>();
    DGPU_CUDA(ctx, cudaMemcpyAsync(d, &h, sizeof(h), cudaMemcpyHostToDevice, ctx->stream));
    int64_t n = (int64_t)cr->nscat * DGPU_NTAB;
    k_formtab<<<(unsigned)dgpu_cdiv(n, 256), 256, 0, ctx->stream>>>(d, cr->nscat, op->lxray, op->power,
                                                                      op->ano, ldbw, d_cfact);
    DGPU_CUDA(ctx, cudaGetLastError());
    // the coefficient block lives in ctx->stats: finish before it is reused
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (d_cfact == ctx->cfact.as<double2>()) {
        ctx->cf_key.p = d_cfact;
        ctx->cf_key.cap = ctx->cfact.cap;
        ctx->cf_key.k = key;
    }
    return DGPU_OK;
}

__global__ void k_increments(const double *xat, int64_t n, PhaseGeom g, int64_t *out)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    double x0 = xat[k], x1 = xat[n + k], x2 = xat[2 * n + k];
    out[0 * n + k] = inc22(dot3_nc(g.vi + 0, x0, x1, x2));
    out[1 * n + k] = inc22(dot3_nc(g.vi + 3, x0, x1, x2));
    out[2 * n + k] = inc22(dot3_nc(g.vi + 6, x0, x1, x2));
    out[3 * n + k] = inc22(dot3_nc(g.off + 0, x0, x1, x2));
    out[4 * n + k] = inc22(dot3_nc(g.off + 3, x0, x1, x2));
    out[5 * n + k] = inc22(dot3_nc(g.off + 6, x0, x1, x2));
}

int dgpu_increments_dev(dgpu_ctx *ctx, const double *d_xat, int64_t nxat, const double uin[3],
                        const double vin[3], const double win[3], const double off[9],
                        int64_t *d_out)
{
    PhaseGeom g;
    memset(&g, 0, sizeof(g));
    for (int k = 0; k < 3; k++) {
        g.vi[k] = uin[k];
        g.vi[3 + k] = vin[k];
        g.vi[6 + k] = win[k];
    }
    memcpy(g.off, off, sizeof(g.off));
    if (nxat > 0) {
        k_increments<<<(unsigned)dgpu_cdiv(nxat, 256), 256, 0, ctx->stream>>>(d_xat, nxat, g, d_out);
        DGPU_CUDA(ctx, cudaGetLastError());
    }
    return DGPU_OK;
}

// ---------------------------------------------------------------------------
// Enqueue-only variants (no host synchronisation; usable under stream capture).
// counts: int32[nblk*nscat], offs: int64[nblk*nscat], ts_dev: int64[2*nscat+1]
// scratch; the phase arrays receive the atoms at the type ranges the host
// computed with the same padding rule (dgpu_type_ranges).
void dgpu_type_ranges(const int32_t *iscat, int64_t n, int32_t nscat, int64_t *ts)
{
    int64_t cnt[MAXT] = {0};
    for (int64_t i = 0; i < n; i++)
        if (iscat[i] >= 1 && iscat[i] <= nscat) cnt[iscat[i]]++;
    int64_t c = 0;
    for (int t = 0; t < nscat; t++) {
        c = (c + TYPE_ALIGN - 1) / TYPE_ALIGN * TYPE_ALIGN;
        ts[t] = c;
        ts[nscat + 1 + t] = cnt[t + 1];
        c += cnt[t + 1];
    }
    ts[nscat] = (c + TYPE_ALIGN - 1) / TYPE_ALIGN * TYPE_ALIGN;
}

int64_t dgpu_prepare_blocks(int64_t natoms) { return dgpu_cdiv(natoms > 0 ? natoms : 1, PREP_BLK); }

int dgpu_prepare_async(dgpu_ctx *ctx, const double *d_pos, const int32_t *d_iscat, const float *d_aocc,
                       int64_t natoms, int32_t nscat, const PhaseGeom &g, int32_t *counts, int64_t *offs,
                       int64_t *ts_dev, uint64_t *ph0, uint64_t *du, uint64_t *dv, uint64_t *dw, float *w,
                       int32_t *idx)
{
    const int64_t nblk = dgpu_prepare_blocks(natoms);
    FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
    k_type_count<<<(unsigned)nblk, PREP_BLK, 0, ctx->stream>>>(d_iscat, natoms, nscat, nofold, counts, nblk);
    k_scan_counts<<<1, 1024, 0, ctx->stream>>>(counts, nblk * nscat, offs, nblk, nscat, ts_dev);
    k_scatter_atoms<<<(unsigned)nblk, PREP_BLK, 0, ctx->stream>>>(d_pos, d_iscat, d_aocc, natoms, nscat, nofold, g,
                                                                  offs, nblk, ts_dev, ph0, du, dv, dw, w, idx);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

// ---------------------------------------------------------------------------
// member-indexed launches (the batch): member blockIdx.y

__global__ void __launch_bounds__(PREP_BLK) k_type_count_m(const PrepMember *__restrict__ M)
{
    const PrepMember &m = M[blockIdx.y];
    if ((int64_t)blockIdx.x >= m.nblk) return;
    const FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
    type_count_body(m.iscat, m.n, m.nscat, nofold, m.counts, m.nblk, blockIdx.x);
}

__global__ void k_scan_counts_m(const PrepMember *__restrict__ M)
{
    const PrepMember &m = M[blockIdx.x];
    scan_counts_body(m.counts, m.offs, m.nblk, m.nscat, m.ts);
}

__global__ void __launch_bounds__(PREP_BLK) k_scatter_atoms_m(const PrepMember *__restrict__ M)
{
    const PrepMember &m = M[blockIdx.y];
    if ((int64_t)blockIdx.x >= m.nblk) return;
    const FoldSpec nofold = {0, 1, {1, 1, 1}, {0, 0, 0}, nullptr};
    scatter_atoms_body(m.pos, m.iscat, m.aocc, m.n, m.nscat, nofold, m.g, m.offs, m.nblk, m.ts, m.ph0, m.du, m.dv,
                       m.dw, m.w, m.idx, blockIdx.x);
}

__global__ void k_stltab_m(const PrepMember *__restrict__ M, int32_t *flag)
{
    const PrepMember &m = M[blockIdx.y];
    stltab_point(m.g.eck, m.g.vi, m.num[0], m.num[1], m.num[2], m.rten, m.istl, flag,
                 (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

__global__ void k_formtab_m(const PrepMember *__restrict__ M, int32_t lxray, int32_t power, int32_t ano)
{
    const PrepMember &m = M[blockIdx.y];
    formtab_entry((const FormCoef *)m.coef, m.ncf, lxray, power, ano, m.ldbw_cf, m.cfact,
                  (int64_t)blockIdx.x * blockDim.x + threadIdx.x);
}

int dgpu_prepare_members(dgpu_ctx *ctx, const PrepMember *d_m, int32_t nc, int64_t max_nblk)
{
    if (nc < 1) return DGPU_OK;
    if (nc > 65535) return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "more than 65535 batch members");
    const dim3 gp((unsigned)max_nblk, (unsigned)nc);
    k_type_count_m<<<gp, PREP_BLK, 0, ctx->stream>>>(d_m);
    k_scan_counts_m<<<(unsigned)nc, 1024, 0, ctx->stream>>>(d_m);
    k_scatter_atoms_m<<<gp, PREP_BLK, 0, ctx->stream>>>(d_m);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_tables_members(dgpu_ctx *ctx, const PrepMember *d_m, int32_t nc, int64_t max_np, int32_t max_nscat,
                        const dgpu_opts *op, int32_t *flag)
{
    if (nc < 1) return DGPU_OK;
    if (nc > 65535) return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "more than 65535 batch members");
    k_stltab_m<<<dim3((unsigned)dgpu_cdiv(max_np, 256), (unsigned)nc), 256, 0, ctx->stream>>>(d_m, flag);
    k_formtab_m<<<dim3((unsigned)dgpu_cdiv((int64_t)max_nscat * DGPU_NTAB, 256), (unsigned)nc), 256, 0,
                  ctx->stream>>>(d_m, op->lxray, op->power, op->ano);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_stltab_async(dgpu_ctx *ctx, const double eck[3], const double vi[9], const int32_t num[3],
                      const double rten[9], int32_t *d_istl, int32_t *d_flag)
{
    const int64_t np = (int64_t)num[0] * num[1] * num[2];
    PhaseGeom vg;
    memset(&vg, 0, sizeof(vg));
    memcpy(vg.vi, vi, sizeof(vg.vi));
    k_stltab<<<(unsigned)dgpu_cdiv(np, 256), 256, 0, ctx->stream>>>(
        eck[0], eck[1], eck[2], vg, num[0], num[1], num[2], rten[0], rten[1], rten[2], rten[3], rten[4], rten[5],
        rten[6], rten[7], rten[8], d_istl, d_flag);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

size_t dgpu_formcoef_bytes() { return sizeof(FormCoef); }

void dgpu_formcoef_fill(const dgpu_crystal *cr, void *host)
{
    FormCoef *h = (FormCoef *)host;
    memset(h, 0, sizeof(FormCoef));
    for (int t = 0; t <= cr->nscat && t < MAXT; t++) {
        for (int i = 0; i < 11; i++) h->scat[11 * t + i] = cr->scat[11 * t + i];
        h->occ[t] = cr->occ[t];
        h->dw[t] = cr->dw[t];
        h->delfr[t] = cr->delfr ? cr->delfr[t] : 0.0;
        h->delfi[t] = cr->delfi ? cr->delfi[t] : 0.0;
    }
}

int dgpu_formtab_async(dgpu_ctx *ctx, const void *d_coef, int32_t nscat, const dgpu_opts *op, double2 *d_cfact)
{
    const int64_t n = (int64_t)nscat * DGPU_NTAB;
    k_formtab<<<(unsigned)dgpu_cdiv(n, 256), 256, 0, ctx->stream>>>((const FormCoef *)d_coef, nscat, op->lxray,
                                                                      op->power, op->ano, op->ldbw, d_cfact);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}
