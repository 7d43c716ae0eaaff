// Tensor-core adjoint: the per-atom sums of the chi^2 gradient
//   T0_j  = sum_h Q_t(h) exp(2 pi i phi_j(h))
//   T_a,j = sum_h n_a(h) Q_t(h) exp(2 pi i phi_j(h))     (a = grid axis)
// (the same sums as k_adj_atoms in k_adjoint.cu; there the derivation).
//
// The Friedel box is cut into one column axis ac (ncols points) and the two
// row axes ra, rb (rows rg = nb * fra + na).  With the exact phase split
//   phi_j = [ph0_j + na d_ra,j + nb d_rb,j] + n_c d_ac,j
// the sums factor through a GEMM over the columns:
//   X[j, rg]  = sum_c V'[j, c] Q[rg, c],      V' = exp(2 pi i n_c d_ac,j)
//   Xc[j, rg] = sum_c n_c V'[j, c] Q[rg, c]
//   T0_j += U'[rg, j] X[j, rg],  T_ra,j += na Im(U' X),  T_rb,j += nb Im(U' X),
//   T_ac,j += Im(U' Xc),         U' = exp(2 pi i (ph0 + na d_ra + nb d_rb)).
// X and Xc run on tcgen05 with the atoms on the 128 TMEM lanes (M = 128 atoms
// of one type), 64 grid rows per MMA (N = 2 x 64: Re | Im through B rows
// [Qr; Qi; -Qr]) and K = grid columns, in the same fp16 hi/lo split
// (three products) as the forward engine; all three products of a row tile
// go to one accumulator (24 MMAs per 64 columns).  Each drain thread owns one
// atom: it walks the rows of the tile with the recurrence
// U' <- U' exp(2 pi i d_ra) (restarting from the exact phase where nb
// changes) and keeps its five sums in registers; there is no reduction across
// lanes.
//
// Q (FP32 complex on the box, per type) is scaled by a power of two so that
// its largest component lies in [2^13, 2^14) and stored once per launch as
// bulk-copy images of 64 rows x 32 columns ([Qr; Qi; -Qr], hi then lo,
// 64-byte-swizzled K-major rows); V' and n_c V' (the A operands of one atom
// tile, 64 columns) are generated in shared memory and stay there for all row
// tiles of the work item.
//
// Warp roles (288 threads): warps 0-3 generate the A operands (and thread 0
// issues the Q copies), warp 4 issues the MMAs, warps 5-8 drain TMEM.  All
// waits are bounded; producers leave their loops together (barrier with an
// OR over failures); bulk copies in flight are awaited before exit.
#include <math.h>

#include "dgpu_internal.h"
#include "tc_ptx.cuh"

#define AT_M 128                                 // atoms per tile (TMEM lanes)
#define AT_R 64                                  // grid rows per row tile
#define AT_KS 32                                 // grid columns per Q stage (two MMA K-steps)
#define AT_KC 64                                 // grid columns per K chunk (A operands resident)
#define AT_QSLOTS 3
#define AT_PROD_WARPS 4
#define AT_PROD_THREADS (AT_PROD_WARPS * 32)
#define AT_MMA_WARP 4
#define AT_THREADS (9 * 32)
#define AT_SUB_BYTES (AT_M * AT_KS * 2)          // one A part of one 32-column block: 8 KB
#define AT_A_BYTES (2 * 4 * 2 * AT_SUB_BYTES)    // 2 variants x 4 parts x 2 blocks: 128 KB
#define AT_QH_BYTES (3 * AT_R * AT_KS * 2)       // [Qr; Qi; -Qr] of one stage, hi or lo: 12 KB
#define AT_Q_BYTES (2 * AT_QH_BYTES)
#define AT_BAR_BYTES 256
#define AT_SMEM (AT_A_BYTES + AT_QSLOTS * AT_Q_BYTES + AT_BAR_BYTES)
#define AT_V_SCALE 4096.0f

// max |component| of Q over all types (bits of a non-negative float)
__global__ void k_adjtc_qmax(const float2 *__restrict__ Q, int64_t n, uint32_t *__restrict__ out)
{
    float m = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 q = Q[i];
        m = fmaxf(m, fmaxf(fabsf(q.x), fabsf(q.y)));
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(out, __float_as_uint(m));
}

// power-of-two exponent that brings the largest Q component to [2^13, 2^14)
__device__ __forceinline__ int adj_qexp(const uint32_t *qmax)
{
    const float m = __uint_as_float(*qmax);
    if (!(m > 0.f) || !isfinite(m)) return 0;
    int e;
    frexpf(m, &e);                 // m = f 2^e, f in [0.5, 1)
    return 14 - e;
}

// Q images: one block per (type, row tile, 32-column stage); thread unit =
// (row r, column quad cq).  Rows and columns outside the box are zero.
__device__ __forceinline__ void adjtc_qimg_block(const float2 *__restrict__ Q, const AdjTcGeom &g,
                                                 const uint32_t *__restrict__ qmax, uint8_t *__restrict__ img,
                                                 int64_t b)
{
    const int sc = (int)(b % g.nstage);
    const int rt = (int)((b / g.nstage) % g.rtiles);
    const int t = (int)(b / ((int64_t)g.nstage * g.rtiles));
    const float scale = ldexpf(1.f, adj_qexp(qmax));
    uint8_t *im = img + b * AT_Q_BYTES;
    const uint32_t blk = (AT_R / 8) * TC_SBO;    // 64 rows further
    for (int u = threadIdx.x; u < AT_R * 8; u += blockDim.x) {
        const int r = u >> 3, cq = u & 7;
        const int64_t rg = (int64_t)rt * AT_R + r;
        float xr[4], xi[4];
#pragma unroll
        for (int e = 0; e < 4; e++) {
            const int c = sc * AT_KS + 4 * cq + e;
            xr[e] = 0.f;
            xi[e] = 0.f;
            if (rg < g.rows && c < g.ncols) {
                const int64_t pb = (rg % g.fra) * g.sra + (rg / g.fra) * g.srb + (int64_t)c * g.sac;
                const float2 q = Q[(int64_t)t * g.pbox + pb];
                xr[e] = q.x * scale;
                xi[e] = q.y * scale;
            }
        }
        uint2 rh, rl, ih, il;
        split4<false>(xr[0], xr[1], xr[2], xr[3], rh, rl);
        split4<false>(xi[0], xi[1], xi[2], xi[3], ih, il);
        uint8_t *d = im + sw_off(r, cq >> 1) + (cq & 1) * 8;
        *reinterpret_cast<uint2 *>(d) = rh;
        *reinterpret_cast<uint2 *>(d + AT_QH_BYTES) = rl;
        *reinterpret_cast<uint2 *>(d + blk) = ih;
        *reinterpret_cast<uint2 *>(d + blk + AT_QH_BYTES) = il;
        *reinterpret_cast<uint2 *>(d + 2 * blk) = make_uint2(rh.x ^ 0x80008000u, rh.y ^ 0x80008000u);
        *reinterpret_cast<uint2 *>(d + 2 * blk + AT_QH_BYTES) = make_uint2(rl.x ^ 0x80008000u, rl.y ^ 0x80008000u);
    }
}

__global__ void __launch_bounds__(256) k_adjtc_qimg(const float2 *__restrict__ Q, AdjTcGeom g,
                                                    const uint32_t *__restrict__ qmax, uint8_t *__restrict__ img)
{
    adjtc_qimg_block(Q, g, qmax, img, blockIdx.x);
}

// exp(2 pi i turn) for a 64-bit fixed-point turn to about one ulp: a float
// part for sincospif and the remainder to first order
__device__ __forceinline__ float2 phasor_accurate(uint64_t turn)
{
    const double x = (double)(int64_t)turn * 0x1p-63;      // turns x 2, in [-1, 1]
    const float xf = (float)x;
    const float dth = (float)((x - (double)xf) * 3.141592653589793);
    float s, c;
    sincospif(xf, &s, &c);
    return make_float2(fmaf(-s, dth, c), fmaf(c, dth, s));
}

// One launch: its work items, and the problem (geometry, atoms, Q images,
// gradient) of each -- p0 for a single problem, or probs[item.prob] in
// device memory for the members of a batch.
struct AdjTcLaunch {
    const AdjItem *items;
    int64_t nitems;
    const AdjTcProb *probs;
    AdjTcProb p0;
    int32_t *err;
};

// barrier among the producer warps, OR of `stop` over them
__device__ __forceinline__ bool adj_prod_sync(bool stop)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)stop), "n"(AT_PROD_THREADS)
        : "memory");
    return r != 0;
}

__device__ __forceinline__ uint32_t adj_a_off(int v, int part, int blk)
{
    return (uint32_t)(((v * 4 + part) * 2 + blk) * AT_SUB_BYTES);
}

// A operands of one atom tile: row m = atom a, the 64 columns of chunk kc:
// V' (x 2^12) and n_c V' (x 2^ec), hi and lo of real and imaginary parts.
// Each 32-column block starts from the exact phase, then steps by
// exp(2 pi i d_ac).
__device__ __forceinline__ void adj_gen_a(uint8_t *A, int m, bool valid, uint64_t dac, int c0, int ncols, int ec)
{
    const float2 step = valid ? phasor_accurate(dac) : make_float2(1.f, 0.f);
    const float sc = ldexpf(1.f, ec);
    for (int blk = 0; blk < 2; blk++) {
        const int cb0 = c0 + blk * AT_KS;
        float2 x = valid ? phasor_fast((uint64_t)(uint32_t)cb0 * dac) : make_float2(0.f, 0.f);
        x = make_float2(x.x * AT_V_SCALE, x.y * AT_V_SCALE);
        for (int cq = 0; cq < AT_KS / 4; cq++) {
            float vr[4], vi[4], wr[4], wi[4];
#pragma unroll
            for (int e = 0; e < 4; e++) {
                const int c = cb0 + 4 * cq + e;
                const bool in = c < ncols;
                const float n = (float)c * sc * (1.f / AT_V_SCALE);
                vr[e] = in ? x.x : 0.f;
                vi[e] = in ? x.y : 0.f;
                wr[e] = in ? x.x * n : 0.f;
                wi[e] = in ? x.y * n : 0.f;
                x = cmulf(x, step);
            }
            const uint32_t o = sw_off(m, cq >> 1) + (cq & 1) * 8;
            uint2 h, l;
            split4<false>(vr[0], vr[1], vr[2], vr[3], h, l);
            *reinterpret_cast<uint2 *>(A + adj_a_off(0, 0, blk) + o) = h;
            *reinterpret_cast<uint2 *>(A + adj_a_off(0, 1, blk) + o) = l;
            split4<false>(vi[0], vi[1], vi[2], vi[3], h, l);
            *reinterpret_cast<uint2 *>(A + adj_a_off(0, 2, blk) + o) = h;
            *reinterpret_cast<uint2 *>(A + adj_a_off(0, 3, blk) + o) = l;
            split4<false>(wr[0], wr[1], wr[2], wr[3], h, l);
            *reinterpret_cast<uint2 *>(A + adj_a_off(1, 0, blk) + o) = h;
            *reinterpret_cast<uint2 *>(A + adj_a_off(1, 1, blk) + o) = l;
            split4<false>(wi[0], wi[1], wi[2], wi[3], h, l);
            *reinterpret_cast<uint2 *>(A + adj_a_off(1, 2, blk) + o) = h;
            *reinterpret_cast<uint2 *>(A + adj_a_off(1, 3, blk) + o) = l;
        }
    }
}

__device__ __forceinline__ int adj_nks(const AdjTcGeom &g, int kc)
{
    const int cols = min(AT_KC, g.ncols - kc * AT_KC);
    return (cols + AT_KS - 1) / AT_KS;
}

__global__ void __launch_bounds__(AT_THREADS, 1) k_adjtc(const AdjTcLaunch L)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    uint8_t *Asm = smem;
    uint8_t *Qsm = smem + AT_A_BYTES;
    uint64_t *bars = reinterpret_cast<uint64_t *>(Qsm + AT_QSLOTS * AT_Q_BYTES);
    uint64_t *afull = bars, *aempty = bars + 1;
    uint64_t *qfull = bars + 2, *qempty = qfull + AT_QSLOTS;
    uint64_t *xfull = qempty + AT_QSLOTS, *xempty = xfull + 2;
    uint64_t *drain = xempty + 2;
    uint32_t *tbase = reinterpret_cast<uint32_t *>(drain + 1);
    volatile int32_t *err = L.err;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    auto prob = [&](const AdjItem &I) -> const AdjTcProb & { return L.probs ? L.probs[I.prob] : L.p0; };

    if (threadIdx.x == 0) {
        mbar_init(afull, AT_PROD_WARPS);
        mbar_init(aempty, 1);
        for (int s = 0; s < AT_QSLOTS; s++) {
            mbar_init(&qfull[s], 1);
            mbar_init(&qempty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&xfull[b], 1);
            mbar_init(&xempty[b], 4);
        }
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == AT_MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase)),
                     "r"(512)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tbase;

    if (warp < AT_PROD_WARPS) {
        // ------------------------------------------------------------ producers
        const int tid = threadIdx.x;
        uint32_t qnext = 0, qland = 0, nit = 0;
        bool ok = true;
        for (int64_t item = blockIdx.x; item < L.nitems; item += gridDim.x) {
            const AdjItem I = L.items[item];
            const AdjTcProb &P = prob(I);
            const AdjTcGeom &G = P.g;
            // the MMAs of the previous item are done with the A operands
            if (tid == 0 && ok && nit > 0) ok = mbar_wait(aempty, (nit - 1) & 1, err, 21);
            if (adj_prod_sync(!ok)) break;
            const int64_t a = I.a0 + tid;
            const bool valid = a < I.a_end;
            adj_gen_a(Asm, tid, valid, valid ? P.dac[a] : 0ull, I.kc * AT_KC, G.ncols, G.ec);
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(afull);
            // thread 0 streams the Q stages of the item through the ring
            if (tid == 0 && ok) {
                const int nks = adj_nks(G, I.kc);
                for (int rt = I.rt0; rt < I.rt1 && ok; rt++)
                    for (int s = 0; s < nks && ok; s++) {
                        const int slot = (int)(qnext % AT_QSLOTS);
                        if (qnext >= AT_QSLOTS) {
                            ok = mbar_wait(&qempty[slot], ((qnext / AT_QSLOTS) - 1) & 1, err, 22);
                            if (!ok) break;
                            qland = qnext - AT_QSLOTS + 1;
                        }
                        const int64_t im =
                            ((int64_t)I.t * G.rtiles + rt) * G.nstage + (int64_t)I.kc * (AT_KC / AT_KS) + s;
                        mbar_arrive_tx(&qfull[slot], AT_Q_BYTES);
                        bulk_g2s(Qsm + (size_t)slot * AT_Q_BYTES, P.qimg + im * AT_Q_BYTES, AT_Q_BYTES, &qfull[slot]);
                        qnext++;
                    }
            }
            nit++;
        }
        // let this thread's bulk copies in flight land before the CTA can exit
        if (tid == 0)
            for (uint32_t x = qland; x < qnext; x++) mbar_wait_quiet(&qfull[x % AT_QSLOTS], (x / AT_QSLOTS) & 1);
    } else if (warp == AT_MMA_WARP) {
        // ------------------------------------------------------------ MMA issuer
        // Lane 0 alone waits, issues and commits; the other lanes join it at
        // the end, so that no warp-wide step sits between two stages.
        // D = 128 atoms x 128 (Re | Im of 64 rows), f32; A and B fp16
        bool issued = false;
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | ((uint32_t)(128 >> 3) << 17) | ((uint32_t)(AT_M >> 4) << 24);
            const uint32_t idesc_neg = idesc | (1u << 13);
            uint32_t qn = 0, nrt = 0, nit = 0;
            bool ok = true;
            for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
                const AdjItem I = L.items[item];
                const AdjTcProb &P = prob(I);
                const AdjTcGeom &G = P.g;
                const int nks = adj_nks(G, I.kc);
                if (!mbar_wait(afull, nit & 1, err, 23)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                for (int rt = I.rt0; rt < I.rt1 && ok; rt++, nrt++) {
                    const int b = (int)(nrt & 1);
                    const uint32_t use = nrt >> 1;
                    if (use > 0 && !mbar_wait(&xempty[b], (use - 1) & 1, err, 24)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t dX = tmem + 256u * b, dXc = dX + 128u;
                    for (int s = 0; s < nks; s++, qn++) {
                        const int slot = (int)(qn % AT_QSLOTS);
                        if (!mbar_wait(&qfull[slot], (qn / AT_QSLOTS) & 1, err, 25)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t A = smem_u32(Asm), Bh = smem_u32(Qsm) + slot * AT_Q_BYTES;
                        const uint32_t Bl = Bh + AT_QH_BYTES, b2 = (AT_R / 8) * TC_SBO;
#pragma unroll
                        for (int kk = 0; kk < AT_KS / 16; kk++) {
                            const uint32_t ko = kk * 32;
                            const uint64_t b1h = sdesc(Bh + ko), b2h = sdesc(Bh + b2 + ko);
                            const uint64_t b1l = sdesc(Bl + ko), b2l = sdesc(Bl + b2 + ko);
                            const uint32_t acc = (s > 0 || kk > 0) ? 1u : 0u;
#pragma unroll
                            for (int v = 0; v < 2; v++) {
                                const uint32_t d = v ? dXc : dX;
                                const uint64_t arh = sdesc(A + adj_a_off(v, 0, s) + ko);
                                const uint64_t arl = sdesc(A + adj_a_off(v, 1, s) + ko);
                                const uint64_t aih = sdesc(A + adj_a_off(v, 2, s) + ko);
                                const uint64_t ail = sdesc(A + adj_a_off(v, 3, s) + ko);
                                mma_f16(d, arh, b1h, idesc, acc);
                                mma_f16(d, aih, b2h, idesc_neg, 1u);
                                mma_f16(d, arh, b1l, idesc, 1u);
                                mma_f16(d, aih, b2l, idesc_neg, 1u);
                                mma_f16(d, arl, b1h, idesc, 1u);
                                mma_f16(d, ail, b2h, idesc_neg, 1u);
                            }
                        }
                        mma_commit(&qempty[slot]);
                        issued = true;
                    }
                    if (!ok) break;
                    mma_commit(&xfull[b]);
                }
                if (!ok) break;
                mma_commit(aempty);
                nit++;
            }
            // no MMA of this CTA may still run when TMEM is freed
            if (issued) {
                mma_commit(drain);
                mbar_wait_quiet(drain, 0);
            }
        }
        __syncwarp();
        tc_fence_before();
    } else {
        // ------------------------------------------------------------ drain: one atom per thread
        const int q = warp & 3;
        const int m = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        uint32_t nrt = 0;
        bool ok = true;
        for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
            const AdjItem I = L.items[item];
            const AdjTcProb &P = prob(I);
            const AdjTcGeom &G = P.g;
            const int64_t a = I.a0 + m;
            const bool valid = a < I.a_end;
            const int eq = adj_qexp(P.qmax);
            const float sx = ldexpf(1.f, -(12 + eq)), sc = ldexpf(1.f, -(G.ec + eq));
            const uint64_t p0 = valid ? P.ph0[a] : 0ull, d0 = valid ? P.dra[a] : 0ull, d1 = valid ? P.drb[a] : 0ull;
            const float2 step = valid ? phasor_accurate(d0) : make_float2(1.f, 0.f);
            float t0r = 0.f, t0i = 0.f, tra = 0.f, trb = 0.f, tac = 0.f;
            // (na, nb) of the first row of each row tile, advanced by AT_R rows per tile
            int64_t na_t = ((int64_t)I.rt0 * AT_R) % G.fra, nb_t = ((int64_t)I.rt0 * AT_R) / G.fra;
            for (int rt = I.rt0; rt < I.rt1; rt++, nrt++) {
                const int b = (int)(nrt & 1);
                if (!__shfl_sync(0xffffffffu, lane == 0 ? mbar_wait(&xfull[b], (nrt >> 1) & 1, err, 26) : true, 0)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const int64_t rg0 = (int64_t)rt * AT_R;
                uint32_t na = (uint32_t)na_t, nb = (uint32_t)nb_t;
                na_t += AT_R;
                while (na_t >= G.fra) {
                    na_t -= G.fra;
                    nb_t++;
                }
                float2 u = valid ? phasor_fast(p0 + (uint64_t)na * d0 + (uint64_t)nb * d1) : make_float2(0.f, 0.f);
                const uint32_t tb = tmem + lane_off + 256u * b;
                for (int c16 = 0; c16 < AT_R / 16; c16++) {
                    uint32_t xr[16], xi[16], cr[16], ci[16];
                    tmem_ld16(tb + (uint32_t)(c16 * 16), xr);
                    tmem_ld16(tb + 64u + (uint32_t)(c16 * 16), xi);
                    tmem_ld16(tb + 128u + (uint32_t)(c16 * 16), cr);
                    tmem_ld16(tb + 192u + (uint32_t)(c16 * 16), ci);
                    tmem_wait_ld();
                    const int64_t rgc = rg0 + c16 * 16;
                    const int kmax = (int)min((int64_t)16, G.rows - rgc);
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        if (k >= kmax) break;
                        const float Xr = __uint_as_float(xr[k]), Xi = __uint_as_float(xi[k]);
                        const float Cr = __uint_as_float(cr[k]), Ci = __uint_as_float(ci[k]);
                        const float zr = fmaf(u.x, Xr, -u.y * Xi), zi = fmaf(u.x, Xi, u.y * Xr);
                        t0r += zr;
                        t0i += zi;
                        tra = fmaf((float)na, zi, tra);
                        trb = fmaf((float)nb, zi, trb);
                        tac += fmaf(u.x, Ci, u.y * Cr);
                        if (++na == (uint32_t)G.fra) {          // next nb: restart from the exact phase
                            na = 0;
                            nb++;
                            u = valid ? phasor_fast(p0 + (uint64_t)nb * d1) : make_float2(0.f, 0.f);
                        } else {
                            u = cmulf(u, step);
                        }
                    }
                }
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&xempty[b]);
            }
            if (!ok) break;
            const int32_t o = valid ? P.aidx[a] : -1;
            if (o >= 0) {
                const double T0r = (double)t0r * sx, T0i = (double)t0i * sx;
                const double Tra = (double)tra * sx, Trb = (double)trb * sx, Tac = (double)tac * sc;
                const double wj = (double)P.w[a], zpi = 6.283185307179586476925286766559;
                if (P.gocc) atomicAdd(&P.gocc[o], T0r);
                if (P.gpos)
#pragma unroll
                    for (int k = 0; k < 3; k++) {
                        const double s = G.eck[k] * T0i + G.vi[3 * G.ra + k] * Tra + G.vi[3 * G.rb + k] * Trb +
                                         G.vi[3 * G.ac + k] * Tac;
                        atomicAdd(&P.gpos[3 * (int64_t)o + k], -zpi * wj * s);
                    }
            }
        }
    }
    __syncthreads();
    if (warp == AT_MMA_WARP) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(512) : "memory");
    }
}

// ---------------------------------------------------------------------------
// Relative cost of a column axis: row tiles x (MMA time of the column stages
// of each chunk, at least the drain time of one row tile).
static double adjtc_cost(const int32_t f[3], int ac)
{
    const int64_t rows = (int64_t)f[0] * f[1] * f[2] / f[ac];
    const double rtiles = (double)dgpu_cdiv(rows, AT_R);
    double c = 0.0;
    for (int c0 = 0; c0 < f[ac]; c0 += AT_KC) {
        const int nks = (int)dgpu_cdiv(f[ac] - c0 < AT_KC ? f[ac] - c0 : AT_KC, AT_KS);
        c += nks * 1.0 > 1.4 ? nks * 1.0 : 1.4;        // one stage ~ 1, one row-tile drain ~ 1.4
    }
    return rtiles * c;
}

void dgpu_adjtc_plan(dgpu_ctx *ctx, const BoxSpec &box, const dgpu_grid *grid, int32_t nscat, const int64_t *ts,
                     AdjTcPlan &plan)
{
    AdjTcGeom &g = plan.g;
    memset(&g, 0, sizeof(g));
    for (int k = 0; k < 3; k++) {
        g.f[k] = box.f[k];
        g.eck[k] = grid->eck[k];
    }
    memcpy(g.vi, grid->vi, sizeof(g.vi));
    int ac = 0;
    double best = 1e300;
    for (int a = 0; a < 3; a++) {
        const double c = adjtc_cost(g.f, a);
        if (c < best * (1 - 1e-9)) {
            best = c;
            ac = a;
        }
    }
    g.ac = ac;
    const int o1 = ac == 0 ? 1 : 0, o2 = 3 - ac - o1;
    g.ra = g.f[o2] > g.f[o1] ? o2 : o1;
    g.rb = 3 - ac - g.ra;
    g.fra = g.f[g.ra];
    g.frb = g.f[g.rb];
    g.ncols = g.f[ac];
    g.rows = (int64_t)g.fra * g.frb;
    const int64_t stride[3] = {1, (int64_t)g.f[0], (int64_t)g.f[0] * g.f[1]};
    g.sra = stride[g.ra];
    g.srb = stride[g.rb];
    g.sac = stride[g.ac];
    g.pbox = (int64_t)g.f[0] * g.f[1] * g.f[2];
    g.rtiles = (int32_t)dgpu_cdiv(g.rows, AT_R);
    g.nstage = (int32_t)dgpu_cdiv(g.ncols, AT_KC) * (AT_KC / AT_KS);
    int lg = 0;
    while ((1 << lg) < g.ncols) lg++;
    g.ec = 14 - lg;                                // n_c < ncols <= 2^lg
    const int kch = (int)dgpu_cdiv(g.ncols, AT_KC);
    // work items: atom tiles x column chunks x row parts
    int64_t tiles = 0;
    for (int t = 0; t < nscat; t++) tiles += dgpu_cdiv(ts[t + 1] - ts[t], AT_M);
    int64_t rp = tiles * kch > 0 ? dgpu_cdiv((int64_t)4 * ctx->nsm, tiles * kch) : 1;
    if (rp > g.rtiles) rp = g.rtiles;
    if (rp < 1) rp = 1;
    plan.items.clear();
    for (int t = 0; t < nscat; t++)
        for (int64_t a0 = ts[t]; a0 < ts[t + 1]; a0 += AT_M)
            for (int kc = 0; kc < kch; kc++)
                for (int64_t p = 0; p < rp; p++) {
                    AdjItem it;
                    it.a0 = a0;
                    it.a_end = ts[t + 1];
                    it.t = t;
                    it.kc = kc;
                    it.rt0 = (int32_t)(g.rtiles * p / rp);
                    it.rt1 = (int32_t)(g.rtiles * (p + 1) / rp);
                    if (it.rt1 > it.rt0) plan.items.push_back(it);
                }
    plan.nimg = (int64_t)nscat * g.rtiles * g.nstage;
    plan.nscat = nscat;
    // once per context (and device), outside any stream capture
    if (!ctx->adj_attr &&
        cudaFuncSetAttribute(k_adjtc, cudaFuncAttributeMaxDynamicSharedMemorySize, AT_SMEM) == cudaSuccess)
        ctx->adj_attr = true;
}

size_t dgpu_adjtc_img_bytes(const AdjTcPlan &plan) { return (size_t)plan.nimg * AT_Q_BYTES; }

int dgpu_adjtc_enqueue(dgpu_ctx *ctx, const AdjTcPlan &plan, const AdjItem *d_items, uint8_t *d_img,
                       uint32_t *d_qmax, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv,
                       const uint64_t *dw, const float *w, const int32_t *aidx, const float2 *Q, double *gpos,
                       double *gocc, int32_t *err)
{
    if (plan.items.empty()) return DGPU_OK;
    const AdjTcGeom &g = plan.g;
    DGPU_CUDA(ctx, cudaMemsetAsync(d_qmax, 0, sizeof(uint32_t), ctx->stream));
    k_adjtc_qmax<<<4 * ctx->nsm, 256, 0, ctx->stream>>>(Q, (int64_t)plan.nscat * g.pbox, d_qmax);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_adjtc_qimg<<<(unsigned)plan.nimg, 256, 0, ctx->stream>>>(Q, g, d_qmax, d_img);
    DGPU_CUDA(ctx, cudaGetLastError());
    AdjTcLaunch L;
    L.items = d_items;
    L.nitems = (int64_t)plan.items.size();
    L.probs = nullptr;
    dgpu_adjtc_prob(plan, ph0, du, dv, dw, w, aidx, Q, d_img, d_qmax, gpos, gocc, L.p0);
    L.err = err;
    const int grid_n = (int)(L.nitems < ctx->nsm ? L.nitems : ctx->nsm);
    k_adjtc<<<grid_n, AT_THREADS, AT_SMEM, ctx->stream>>>(L);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

void dgpu_adjtc_prob(const AdjTcPlan &plan, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv,
                     const uint64_t *dw, const float *w, const int32_t *aidx, const float2 *Q, uint8_t *img,
                     uint32_t *qmax, double *gpos, double *gocc, AdjTcProb &P)
{
    const uint64_t *dd[3] = {du, dv, dw};
    P.g = plan.g;
    P.ph0 = ph0;
    P.dra = dd[plan.g.ra];
    P.drb = dd[plan.g.rb];
    P.dac = dd[plan.g.ac];
    P.w = w;
    P.aidx = aidx;
    P.Q = Q;
    P.qimg = img;
    P.qmax = qmax;
    P.gpos = gpos;
    P.gocc = gocc;
    P.nimg = plan.nimg;
    P.nscat = plan.nscat;
}

// member-indexed Q scale and Q images of a batch (member blockIdx.y)
#define ADJ_QMAX_BLOCKS 64
__global__ void k_adjtc_qmax_m(const AdjTcProb *__restrict__ M)
{
    const AdjTcProb &m = M[blockIdx.y];
    const int64_t n = (int64_t)m.nscat * m.g.pbox;
    float v = 0.f;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)ADJ_QMAX_BLOCKS * blockDim.x) {
        const float2 q = m.Q[i];
        v = fmaxf(v, fmaxf(fabsf(q.x), fabsf(q.y)));
    }
    for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0 && v > 0.f) atomicMax(m.qmax, __float_as_uint(v));
}

__global__ void __launch_bounds__(256) k_adjtc_qimg_m(const AdjTcProb *__restrict__ M)
{
    const AdjTcProb &m = M[blockIdx.y];
    if ((int64_t)blockIdx.x >= m.nimg) return;
    adjtc_qimg_block(m.Q, m.g, m.qmax, m.qimg, blockIdx.x);
}

int dgpu_adjtc_members(dgpu_ctx *ctx, const AdjTcProb *d_probs, int32_t nc, int64_t max_nimg, const AdjItem *d_items,
                       int64_t nitems, int32_t *err)
{
    if (nc < 1 || nitems < 1) return DGPU_OK;
    k_adjtc_qmax_m<<<dim3(ADJ_QMAX_BLOCKS, (unsigned)nc), 256, 0, ctx->stream>>>(d_probs);
    k_adjtc_qimg_m<<<dim3((unsigned)max_nimg, (unsigned)nc), 256, 0, ctx->stream>>>(d_probs);
    DGPU_CUDA(ctx, cudaGetLastError());
    AdjTcLaunch L;
    memset(&L, 0, sizeof(L));
    L.items = d_items;
    L.nitems = nitems;
    L.probs = d_probs;
    L.err = err;
    if (!ctx->adj_attr &&
        cudaFuncSetAttribute(k_adjtc, cudaFuncAttributeMaxDynamicSharedMemorySize, AT_SMEM) == cudaSuccess)
        ctx->adj_attr = true;
    const int grid_n = (int)(nitems < ctx->nsm ? nitems : ctx->nsm);
    k_adjtc<<<grid_n, AT_THREADS, AT_SMEM, ctx->stream>>>(L);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_adjtc_sums(dgpu_ctx *ctx, const BoxSpec &box, const dgpu_grid *grid, int32_t nscat, const int64_t *ts,
                    const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw, const float *w,
                    const int32_t *aidx, const float2 *Q, double *gpos, double *gocc)
{
    if (nscat < 1 || nscat > 64) return dgpu_set_error(ctx, DGPU_ERR_ARG, "nscat=%d", nscat);
    AdjTcPlan plan;
    dgpu_adjtc_plan(ctx, box, grid, nscat, ts, plan);
    if (plan.items.empty()) return DGPU_OK;
    const size_t ibytes = ((size_t)plan.items.size() * sizeof(AdjItem) + 255) & ~(size_t)255;
    DGPU_CUDA(ctx, ctx->adj_qimg.ensure(dgpu_adjtc_img_bytes(plan)));
    DGPU_CUDA(ctx, ctx->adj_items.ensure(ibytes + 256));
    uint32_t *qmax = reinterpret_cast<uint32_t *>(ctx->adj_items.as<uint8_t>() + ibytes);
    DGPU_CUDA(ctx, cudaMemcpyAsync(ctx->adj_items.p, plan.items.data(), plan.items.size() * sizeof(AdjItem),
                                   cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, ctx->flag.ensure(64));
    int32_t *err = ctx->flag.as<int32_t>() + 10;
    DGPU_CUDA(ctx, cudaMemsetAsync(err, 0, sizeof(int32_t), ctx->stream));
    int rc = dgpu_adjtc_enqueue(ctx, plan, ctx->adj_items.as<AdjItem>(), ctx->adj_qimg.as<uint8_t>(), qmax, ph0, du,
                                dv, dw, w, aidx, Q, gpos, gocc, err);
    if (rc) return rc;
    // the item table must outlive its copy; the error flag is read here
    int32_t herr = 0;
    DGPU_CUDA(ctx, cudaMemcpyAsync(&herr, err, sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr) return dgpu_set_error(ctx, DGPU_ERR_TIMEOUT, "tensor-core adjoint wait gave up (site %d)", herr);
    return DGPU_OK;
}
