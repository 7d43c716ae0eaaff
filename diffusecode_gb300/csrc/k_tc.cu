// Tensor-core engine: the type sums as a split-precision complex GEMM on
// tcgen05 (sm_100 family), accumulators in TMEM.
//
// For the computed box, one grid axis ac is the GEMM's N dimension
// ("columns") and the other two, flattened, its M dimension ("rows").  The
// phase of point (row r, column c) and atom j splits exactly:
//     phase = [ph0_j + n_ra(r) d_ra,j + n_rb(r) d_rb,j] + [n_ac(c) d_ac,j]
// so  S(r,c) = sum_j U[r,j] V[j,c]  with  U = w_j exp(2 pi i A-phase),
// V = exp(2 pi i B-phase); K = the atoms of one type (a slice of them per
// work item).  Each CTA generates its U (128 rows) and V (N columns) tiles
// for KA = 32 atoms per stage directly in shared memory from the 64-bit
// fixed-point phases (no operand traffic in HBM), splits every FP32 phasor
// value into fp16 (or bf16) hi + lo, and issues per 16 atoms the 12 MMAs
//     Re += Ur Vr^T - Ui Vi^T ,  Im += Ur Vi^T + Ui Vr^T
// for the split products (hi,hi), (hi,lo), (lo,hi).
//
// Accumulation.  Every MMA truncates its FP32 accumulator by about one ulp,
// so the error of one TMEM accumulator grows with the number of MMAs chained
// into it.  The large (hi,hi) products therefore go to a "main" accumulator
// that is drained every `flush` stages (flush*32 atoms) into the work item's
// FP32 partial in global memory (round-to-nearest adds on CUDA cores, the
// partial stays in L2), and the small (hi,lo)+(lo,hi) corrections go to a
// separate accumulator drained once per work item.  With nbuf = 2 the main
// accumulator is double-buffered so the drain overlaps the next chunk.  The
// combine kernel adds the K slices of all work items in FP64.
//
// Warp roles (416 threads): warps 0-7 produce operand stages, warp 8 owns
// TMEM and issues the MMAs (one elected lane), warps 9-12 drain TMEM.  All
// waits are bounded (globaltimer); a wait that gives up sets an error flag,
// the CTA stops issuing, waits for its own MMAs, frees TMEM and returns.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8x8 fp16 core matrices of 128 contiguous bytes, LBO = 128 B between
// K-adjacent core matrices, SBO = (KA/8)*128 B between 8-row groups.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "dgpu_internal.h"

#define TC_KA 32
#define TC_M 128
#define TC_PROD_WARPS 8
#define TC_MMA_WARP 8
#define TC_EPI_WARP0 9
#define TC_THREADS (13 * 32)
#define TC_PROD_THREADS (TC_PROD_WARPS * 32)
#define TC_A_BYTES (TC_M * TC_KA * 2)          // one operand (e.g. Ur_hi): 8 KB
#define TC_SBO ((TC_KA / 8) * 128)
#define TC_LBO 128
#define TC_TIMEOUT_NS 2000000000ull            // 2 s per wait
// phase data of one 32-atom group in shared memory: ph0, d_ra, d_rb, d_ac (u64), w (f32)
#define TC_ATOM_SLOT (TC_KA * 4 * 8 + TC_KA * 4)
#define TC_BAR_BYTES 256
#ifndef TC_FLUSH_STAGES
#define TC_FLUSH_STAGES 4                      // 128 atoms per drain of the main accumulator
#endif

// ---------------------------------------------------------------------------
// PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ uint64_t gtimer()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// bounded wait: false if the error flag is up or the wait timed out
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int32_t *err, int code)
{
    if (mbar_try(bar, parity)) return true;
    uint64_t t0 = gtimer();
    for (uint32_t it = 1;; ++it) {
        if (mbar_try(bar, parity)) return true;
        if ((it & 63) == 0) {
            if (*err) return false;
            if (gtimer() - t0 > TC_TIMEOUT_NS) {
                atomicCAS((int32_t *)err, 0, code);
                return false;
            }
        }
    }
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
// barrier among the producer warps only
__device__ __forceinline__ void producers_sync() { asm volatile("bar.sync 1, %0;" ::"n"(TC_PROD_THREADS) : "memory"); }

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((TC_LBO >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((TC_SBO >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;          // descriptor version of the sm_100 family; no swizzle
    return d;
}

__device__ __forceinline__ void mma_f16(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// ---------------------------------------------------------------------------
// operand generation

// exp(2 pi i phase) from the top 32 bits of a 64-bit fixed-point turn
__device__ __forceinline__ void phasor(uint64_t ph, float &c, float &s)
{
#ifdef TC_PHASOR_ACCURATE
    sincospif((float)(int32_t)(ph >> 32) * 4.656612873077393e-10f, &s, &c);
#else
    float ang = (float)(int32_t)(ph >> 32) * 1.4629180792671596e-09f;   // 2 pi / 2^32
    __sincosf(ang, &s, &c);
#endif
}

__device__ __forceinline__ uint32_t pack2(float a, float b, bool bf)
{
    if (bf) {
        __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&v);
    }
    __half2 v = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}

__device__ __forceinline__ float2 unpack2(uint32_t u, bool bf)
{
    if (bf) {
        __nv_bfloat162 v = *reinterpret_cast<__nv_bfloat162 *>(&u);
        return __bfloat1622float2(v);
    }
    __half2 v = *reinterpret_cast<__half2 *>(&u);
    return __half22float2(v);
}

// 8 values -> hi (rounded) and lo (remainder x 2^12, rounded), 16 bytes each.
// hi is zero or a normal number; the remainder is scaled by 2^12 so that it
// stays normal in fp16 as well (tensor-core inputs below 2^-14 would
// otherwise lose their bits); the correction accumulator, which only ever
// receives products with one lo factor, is scaled back by 2^-12.
#define TC_LO_SCALE 4096.0f
#define TC_LO_UNSCALE (1.0f / 4096.0f)
__device__ __forceinline__ void split8(const float (&v)[8], uint4 &hi, uint4 &lo, bool bf)
{
    uint32_t h[4], l[4];
#pragma unroll
    for (int k = 0; k < 4; k++) {
        const float x0 = v[2 * k], x1 = v[2 * k + 1];
        const float y0 = fabsf(x0) < 6.103515625e-05f ? 0.f : x0;     // 2^-14: smallest normal fp16
        const float y1 = fabsf(x1) < 6.103515625e-05f ? 0.f : x1;
        h[k] = pack2(y0, y1, bf);
        float2 b = unpack2(h[k], bf);
        l[k] = pack2((x0 - b.x) * TC_LO_SCALE, (x1 - b.y) * TC_LO_SCALE, bf);
    }
    hi = make_uint4(h[0], h[1], h[2], h[3]);
    lo = make_uint4(l[0], l[1], l[2], l[3]);
}

// byte offset of (row, k-group) in one operand of the canonical layout
__device__ __forceinline__ uint32_t core_off(int row, int q) { return (row >> 3) * TC_SBO + q * TC_LBO + (row & 7) * 16; }

__device__ __forceinline__ void decode_item(const TcProblem &g, int64_t item, int &t, int &ks, int &nt, int &mt)
{
    mt = (int)(item % g.m_tiles);
    int64_t r = item / g.m_tiles;
    nt = (int)(r % g.n_tiles);
    r /= g.n_tiles;
    ks = (int)(r % g.nslice);
    t = (int)(r / g.nslice);
}

__global__ void __launch_bounds__(TC_THREADS, 1) k_tc(const TcLaunch L)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int S = L.stages;
    const int NM = L.Nmax;
    const uint32_t b_bytes = (uint32_t)NM * TC_KA * 2;     // one B operand
    const uint32_t stage_bytes = 4 * TC_A_BYTES + 4 * b_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)S * stage_bytes);
    uint64_t *empty = full + S;
    uint64_t *mfull = empty + S;      // [2] main accumulator b ready
    uint64_t *mempty = mfull + 2;     // [2] main accumulator b drained
    uint64_t *cfull = mempty + 2;     // correction accumulator ready (end of item)
    uint64_t *cempty = cfull + 1;     // correction accumulator drained
    uint64_t *drain = cempty + 1;
    uint32_t *tbase = reinterpret_cast<uint32_t *>(drain + 1);
    uint8_t *aslot = smem + (size_t)S * stage_bytes + TC_BAR_BYTES;   // 2 x TC_ATOM_SLOT
    volatile int32_t *err = L.err;
    const bool bf = L.bf16 != 0;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], TC_PROD_THREADS);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&mfull[b], 1);
            mbar_init(&mempty[b], 4 * 32);
        }
        mbar_init(cfull, 1);
        mbar_init(cempty, 4 * 32);
        mbar_init(drain, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == TC_MMA_WARP) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(tbase)),
                     "r"(L.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tbase;

    if (warp < TC_PROD_WARPS) {
        // ------------------------------------------------------------ producers
        // Atom groups are complete (type ranges padded to 32 atoms with zero
        // weight).  Their phase data is staged in shared memory with
        // cp.async, one group ahead of the generation.
        const int tid = threadIdx.x;
        uint32_t it = 0;
        bool ok = true;
        auto issue = [&](const TcProblem &P, int slot, int64_t ab) {
            uint8_t *dst = aslot + slot * TC_ATOM_SLOT;
            if (tid < 64) {            // 4 arrays x 16 chunks of 16 B
                const int arr = tid >> 4, ch = tid & 15;
                const uint64_t *src = arr == 0 ? P.ph0 : arr == 1 ? P.dra : arr == 2 ? P.drb : P.dac;
                cp_async16(dst + arr * (TC_KA * 8) + ch * 16, src + ab + ch * 2);
            } else if (tid < 72) {     // weights: 8 chunks
                const int ch = tid - 64;
                cp_async16(dst + 4 * TC_KA * 8 + ch * 16, P.w + ab + ch * 4);
            }
            cp_async_commit();
        };
        for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
            const TcProblem &g = L.probs[L.item_prob[item]];
            const int N = g.N;
            int t, ks, nt, mt;
            decode_item(g, item - g.item0, t, ks, nt, mt);
            const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
            const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
            const int64_t cnt = a1 > a0 ? a1 - a0 : 0;
            const int nst = (int)(cnt / TC_KA);
            if (nst == 0) continue;
            producers_sync();               // previous item's slots are free
            issue(g, 0, a0);
            for (int st = 0; st < nst; st++, it++) {
                const int s = it % S;
                if (st + 1 < nst) {
                    issue(g, (st + 1) & 1, a0 + (int64_t)(st + 1) * TC_KA);
                    cp_async_wait1();
                } else {
                    cp_async_wait0();
                }
                producers_sync();           // group st staged for everybody
                if (it >= (uint32_t)S && !mbar_wait(&empty[s], ((it / S) - 1) & 1, err, 1)) { ok = false; break; }
                const uint8_t *as = aslot + (st & 1) * TC_ATOM_SLOT;
                const uint64_t *s_ph0 = reinterpret_cast<const uint64_t *>(as);
                const uint64_t *s_dra = s_ph0 + TC_KA, *s_drb = s_dra + TC_KA, *s_dac = s_drb + TC_KA;
                const float *s_w = reinterpret_cast<const float *>(s_dac + TC_KA);
                uint8_t *A = smem + (size_t)s * stage_bytes;
                uint8_t *B = A + 4 * TC_A_BYTES;
                const int units = 4 * TC_M + 4 * N;
                for (int u = tid; u < units; u += TC_PROD_THREADS) {
                    float re[8], im[8];
                    uint32_t off;
                    uint8_t *base;
                    uint32_t ostride;
                    if (u < 4 * TC_M) {
                        const int r = u % TC_M, q = u / TC_M;
                        const int64_t rg = (int64_t)mt * TC_M + r;
                        const bool rv = rg < g.nrows;
                        const uint32_t na = rv ? (uint32_t)(rg % g.fra) : 0u;
                        const uint32_t nb = rv ? (uint32_t)(rg / g.fra) : 0u;
                        const float wr = rv ? 1.f : 0.f;
#pragma unroll
                        for (int e = 0; e < 8; e++) {
                            const int k = q * 8 + e;
                            const uint64_t ph = s_ph0[k] + na * s_dra[k] + nb * s_drb[k];
                            float c, sn;
                            phasor(ph, c, sn);
                            const float wj = s_w[k] * wr;
                            re[e] = wj * c;
                            im[e] = wj * sn;
                        }
                        off = core_off(r, q);
                        base = A;
                        ostride = TC_A_BYTES;
                    } else {
                        const int v = u - 4 * TC_M;
                        const int c = v % N, q = v / N;
                        const int64_t cg = (int64_t)nt * N + c;
                        const float wc = cg < g.ncols ? 1.f : 0.f;
                        const uint32_t nc = (uint32_t)cg;
#pragma unroll
                        for (int e = 0; e < 8; e++) {
                            float cs, sn;
                            phasor(nc * s_dac[q * 8 + e], cs, sn);
                            re[e] = cs * wc;
                            im[e] = sn * wc;
                        }
                        off = core_off(c, q);
                        base = B;
                        ostride = b_bytes;
                    }
                    uint4 hr, lr, hi_, li;
                    split8(re, hr, lr, bf);
                    split8(im, hi_, li, bf);
                    *reinterpret_cast<uint4 *>(base + 0 * ostride + off) = hr;   // real hi
                    *reinterpret_cast<uint4 *>(base + 1 * ostride + off) = lr;   // real lo
                    *reinterpret_cast<uint4 *>(base + 2 * ostride + off) = hi_;  // imag hi
                    *reinterpret_cast<uint4 *>(base + 3 * ostride + off) = li;   // imag lo
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_arrive(&full[s]);
            }
            cp_async_wait0();
        }
    } else if (warp == TC_MMA_WARP) {
        // ------------------------------------------------------------ MMA issuer
        const uint32_t fmt = bf ? 1u : 0u;
        const uint32_t c_re = tmem, c_im = tmem + (uint32_t)NM;  // correction accumulator
        uint32_t it = 0, nitem = 0, nchunk = 0;
        bool ok = true, issued = false;
        for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
            const TcProblem &g = L.probs[L.item_prob[item]];
            const int N = g.N;
            int t, ks, nt, mt;
            decode_item(g, item - g.item0, t, ks, nt, mt);
            const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
            const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
            const int64_t cnt = a1 > a0 ? a1 - a0 : 0;
            const int nst = (int)((cnt + TC_KA - 1) / TC_KA);
            if (nst == 0) continue;
            const uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) |
                                   ((uint32_t)(TC_M >> 4) << 24);
            const uint32_t idesc_neg = idesc | (1u << 13);     // negate A: the -Ui Vi^T products
            // the correction accumulator restarts with this item: previous one drained?
            if (nitem > 0 && !mbar_wait(cempty, (nitem - 1) & 1, err, 2)) { ok = false; break; }
            for (int st0 = 0; st0 < nst && ok; st0 += L.flush, nchunk++) {
                const int b = (int)(nchunk % L.nbuf);
                const uint32_t use = nchunk / L.nbuf;
                if (use > 0 && !mbar_wait(&mempty[b], (use - 1) & 1, err, 6)) { ok = false; break; }
                tc_fence_after();
                const uint32_t m_re = tmem + 2u * NM * (1u + (uint32_t)b), m_im = m_re + (uint32_t)NM;
                const int st1 = min(nst, st0 + L.flush);
                for (int st = st0; st < st1; st++, it++) {
                    const int s = it % S;
                    if (!mbar_wait(&full[s], (it / S) & 1, err, 3)) { ok = false; break; }
                    tc_fence_after();
                    if (lane == 0) {
                        const uint32_t A = smem_u32(smem + (size_t)s * stage_bytes);
                        const uint32_t B = A + 4 * TC_A_BYTES;
#pragma unroll
                        for (int kk = 0; kk < TC_KA / 16; kk++) {
                            const uint32_t ko = kk * 2 * TC_LBO;
                            const uint64_t arh = sdesc(A + 0 * TC_A_BYTES + ko), arl = sdesc(A + 1 * TC_A_BYTES + ko);
                            const uint64_t aih = sdesc(A + 2 * TC_A_BYTES + ko), ail = sdesc(A + 3 * TC_A_BYTES + ko);
                            const uint64_t brh = sdesc(B + 0 * b_bytes + ko), brl = sdesc(B + 1 * b_bytes + ko);
                            const uint64_t bih = sdesc(B + 2 * b_bytes + ko), bil = sdesc(B + 3 * b_bytes + ko);
                            const uint32_t am = (st > st0 || kk > 0) ? 1u : 0u;   // main restarts per chunk
                            const uint32_t ac = (st > 0 || kk > 0) ? 1u : 0u;     // correction per item
                            // main: (hi,hi)
                            mma_f16(m_re, arh, brh, idesc, am);
                            mma_f16(m_re, aih, bih, idesc_neg, 1u);
                            mma_f16(m_im, arh, bih, idesc, am);
                            mma_f16(m_im, aih, brh, idesc, 1u);
                            // corrections: (hi,lo) and (lo,hi)
                            mma_f16(c_re, arh, brl, idesc, ac);
                            mma_f16(c_re, aih, bil, idesc_neg, 1u);
                            mma_f16(c_re, arl, brh, idesc, 1u);
                            mma_f16(c_re, ail, bih, idesc_neg, 1u);
                            mma_f16(c_im, arh, bil, idesc, ac);
                            mma_f16(c_im, aih, brl, idesc, 1u);
                            mma_f16(c_im, arl, bih, idesc, 1u);
                            mma_f16(c_im, ail, brh, idesc, 1u);
                        }
                        mma_commit(&empty[s]);
                        issued = true;
                    }
                    __syncwarp();
                }
                if (!ok) break;
                if (lane == 0) mma_commit(&mfull[b]);
                __syncwarp();
            }
            if (!ok) break;
            if (lane == 0) mma_commit(cfull);
            __syncwarp();
            nitem++;
        }
        // make sure no MMA of this CTA is still running before TMEM is freed
        if (lane == 0 && issued) mma_commit(drain);
        __syncwarp();
        if (__shfl_sync(0xffffffffu, issued ? 1 : 0, 0)) mbar_wait(drain, 0, err, 4);
        tc_fence_before();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;                       // TMEM lane quadrant of this warp
        const int r = q * 32 + lane;
        uint32_t nitem = 0, nchunk = 0;
        bool ok = true;
        for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
            const TcProblem &g = L.probs[L.item_prob[item]];
            const int N = g.N;
            int t, ks, nt, mt;
            decode_item(g, item - g.item0, t, ks, nt, mt);
            const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
            const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
            const int64_t cnt = a1 > a0 ? a1 - a0 : 0;
            const int nst = (int)((cnt + TC_KA - 1) / TC_KA);
            const int64_t rg = (int64_t)mt * TC_M + r;
            const bool rv = rg < g.nrows;
            const int64_t prow = rv ? (rg % g.fra) * g.sra + (rg / g.fra) * g.srb : 0;
            float2 *out = g.part + ((int64_t)t * g.nslice + ks) * g.pbox + prow;
            const int64_t cbase0 = (int64_t)nt * N;
            if (nst == 0) {
                if (rv)
                    for (int c = 0; c < N && cbase0 + c < g.ncols; c++) out[(cbase0 + c) * g.sac] = make_float2(0.f, 0.f);
                continue;
            }
            // main accumulator, one chunk at a time: first chunk stores, later chunks add
            for (int st0 = 0; st0 < nst; st0 += L.flush, nchunk++) {
                const int b = (int)(nchunk % L.nbuf);
                if (!mbar_wait(&mfull[b], (nchunk / L.nbuf) & 1, err, 5)) { ok = false; break; }
                tc_fence_after();
                const uint32_t col0 = 2u * NM * (1u + (uint32_t)b);
                for (int c0 = 0; c0 < N; c0 += 16) {
                    uint32_t vr[16], vi[16];
                    const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + col0 + (uint32_t)c0;
                    tmem_ld16(ta, vr);
                    tmem_ld16(ta + (uint32_t)NM, vi);
                    tmem_wait_ld();
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        const int64_t cg = cbase0 + c0 + k;
                        if (rv && cg < g.ncols) {
                            float2 v = make_float2(__uint_as_float(vr[k]), __uint_as_float(vi[k]));
                            float2 *o = out + cg * g.sac;
                            if (st0 > 0) {
                                float2 old = *o;
                                v.x += old.x;
                                v.y += old.y;
                            }
                            *o = v;
                        }
                    }
                }
                tc_fence_before();
                mbar_arrive(&mempty[b]);
            }
            if (!ok) break;
            // correction accumulator of the item
            if (!mbar_wait(cfull, nitem & 1, err, 7)) { ok = false; break; }
            tc_fence_after();
            for (int c0 = 0; c0 < N; c0 += 16) {
                uint32_t vr[16], vi[16];
                const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0;
                tmem_ld16(ta, vr);
                tmem_ld16(ta + (uint32_t)NM, vi);
                tmem_wait_ld();
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    const int64_t cg = cbase0 + c0 + k;
                    if (rv && cg < g.ncols) {
                        float2 *o = out + cg * g.sac;
                        float2 old = *o;
                        *o = make_float2(fmaf(__uint_as_float(vr[k]), TC_LO_UNSCALE, old.x),
                                         fmaf(__uint_as_float(vi[k]), TC_LO_UNSCALE, old.y));
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(cempty);
            nitem++;
        }
    }
    __syncthreads();
    if (warp == TC_MMA_WARP) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L.tmem_cols)
                     : "memory");
    }
}

// ---------------------------------------------------------------------------
bool dgpu_tc_available(dgpu_ctx *ctx)
{
    static int cached = -1;
    if (cached < 0) {
        cudaDeviceProp p;
        cached = (cudaGetDeviceProperties(&p, ctx->device) == cudaSuccess && p.major == 10) ? 1 : 0;
    }
    return cached == 1;
}

static uint32_t pow2_cols(int n)
{
    uint32_t c = 32;
    while (c < (uint32_t)n) c <<= 1;
    return c;
}

// padded MMA area of a column axis / tile width
static double tc_area(const BoxSpec &box, int a, int N)
{
    const int64_t npts = (int64_t)box.f[0] * box.f[1] * box.f[2];
    const int nc = box.f[a];
    if (nc < 2 && npts != nc) return -1.0;
    return (double)dgpu_cdiv(nc, N) * N * dgpu_cdiv(npts / nc, TC_M) * TC_M;
}

// Geometry of one problem for a column axis, tile width and slicing.
static void tc_problem(dgpu_ctx *ctx, const TcInput &in, const dgpu_opts *op, int axis, int N, int slice_mult,
                       TcProblem &g)
{
    memset(&g, 0, sizeof(g));
    const BoxSpec &box = in.box;
    for (int k = 0; k < 3; k++) g.f[k] = box.f[k];
    g.ac = axis;
    g.ra = axis == 0 ? 1 : 0;
    g.rb = 3 - axis - g.ra;
    g.ncols = box.f[axis];
    g.fra = box.f[g.ra];
    const int64_t stride[3] = {1, (int64_t)box.f[0], (int64_t)box.f[0] * box.f[1]};
    g.sra = stride[g.ra];
    g.srb = stride[g.rb];
    g.sac = stride[axis];
    g.nrows = box.f[g.ra] * box.f[g.rb];
    g.N = N;
    g.n_tiles = (int32_t)dgpu_cdiv(g.ncols, N);
    g.m_tiles = (int32_t)dgpu_cdiv(g.nrows, TC_M);
    g.pbox = (int64_t)box.f[0] * box.f[1] * box.f[2];
    g.ntype = in.ntype;
    int64_t maxn = 0;
    for (int t = 0; t < in.ntype; t++) {
        g.ts[t] = in.ts[t];
        const int64_t n = in.ts[t + 1] - in.ts[t];
        maxn = n > maxn ? n : maxn;
    }
    g.ts[in.ntype] = in.ts[in.ntype];
    // K slices: about slice_mult work items per SM, or tc_kslice atoms each when given
    const int64_t tiles = (int64_t)g.m_tiles * g.n_tiles * in.ntype;
    int64_t nsl;
    if (op->tc_kslice > 0) {
        nsl = dgpu_cdiv(maxn, op->tc_kslice);
    } else {
        nsl = dgpu_cdiv((int64_t)slice_mult * ctx->nsm, tiles);
        if (nsl > 1 && dgpu_cdiv(maxn, nsl) < 2048) nsl = dgpu_cdiv(maxn, 2048);
    }
    if (nsl < 1) nsl = 1;
    g.slice_len = dgpu_cdiv(dgpu_cdiv(maxn > 0 ? maxn : 1, nsl), TC_KA) * TC_KA;
    g.nslice = (int32_t)dgpu_cdiv(maxn > 0 ? maxn : 1, g.slice_len);
    g.nitems = tiles * g.nslice;
    const uint64_t *dd[3] = {in.du, in.dv, in.dw};
    g.ph0 = in.ph0;
    g.dra = dd[g.ra];
    g.drb = dd[g.rb];
    g.dac = dd[axis];
    g.w = in.w;
}

int dgpu_tc_plan(dgpu_ctx *ctx, int nprob, const TcInput *in, const dgpu_opts *op, int N, int slice_mult,
                 TcPlan &plan, DevBuf &part, DevBuf &desc)
{
    plan.probs.assign(nprob, TcProblem());
    plan.part_off.assign(nprob, 0);
    plan.nslice.assign(nprob, 0);
    int64_t items = 0, elems = 0;
    for (int p = 0; p < nprob; p++) {
        int axis = in[p].axis;
        if (axis < 0) {
            double best = 1e300;
            for (int a = 0; a < 3; a++) {
                const double ar = tc_area(in[p].box, a, N);
                if (ar >= 0 && ar < best * (1 - 1e-9)) { best = ar; axis = a; }
            }
        }
        if (axis < 0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "no tensor-core tile fits the box");
        TcProblem &g = plan.probs[p];
        tc_problem(ctx, in[p], op, axis, N, slice_mult, g);
        g.item0 = items;
        items += g.nitems;
        plan.part_off[p] = elems;
        plan.nslice[p] = g.nslice;
        elems += (int64_t)g.ntype * g.nslice * g.pbox;
    }
    plan.item_prob.resize(items);
    for (int p = 0; p < nprob; p++)
        for (int64_t i = 0; i < plan.probs[p].nitems; i++) plan.item_prob[plan.probs[p].item0 + i] = p;
    DGPU_CUDA(ctx, part.ensure((size_t)(elems > 0 ? elems : 1) * sizeof(float2)));
    for (int p = 0; p < nprob; p++) plan.probs[p].part = part.as<float2>() + plan.part_off[p];
    const size_t pbytes = ((size_t)nprob * sizeof(TcProblem) + 255) & ~(size_t)255;
    DGPU_CUDA(ctx, desc.ensure(pbytes + (size_t)items * sizeof(int32_t) + 256));
    DGPU_CUDA(ctx, cudaMemcpyAsync(desc.p, plan.probs.data(), (size_t)nprob * sizeof(TcProblem),
                                   cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync((char *)desc.p + pbytes, plan.item_prob.data(), (size_t)items * sizeof(int32_t),
                                   cudaMemcpyHostToDevice, ctx->stream));
    // the host vectors must outlive the copies
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    TcLaunch &L = plan.L;
    L.probs = (const TcProblem *)desc.p;
    L.item_prob = (const int32_t *)((char *)desc.p + pbytes);
    L.nitems = items;
    L.Nmax = N;
    L.nbuf = 6 * N <= 512 ? 2 : 1;
    L.flush = op->tc_flush > 0 ? (int32_t)dgpu_cdiv(op->tc_flush, TC_KA) : TC_FLUSH_STAGES;
    L.bf16 = op->split == DGPU_SPLIT_BF16;
    const uint32_t stage_bytes = 4 * TC_A_BYTES + 4u * N * TC_KA * 2;
    const uint32_t bar_bytes = TC_BAR_BYTES + 2 * TC_ATOM_SLOT;
    const int stages = (int)((200 * 1024 - bar_bytes) / stage_bytes);
    L.stages = stages > 4 ? 4 : stages;
    L.tmem_cols = pow2_cols(2 * N * (1 + L.nbuf));
    if (L.stages < 2 || L.tmem_cols > 512) return dgpu_set_error(ctx, DGPU_ERR_ARG, "tile does not fit");
    plan.smem = (size_t)L.stages * stage_bytes + bar_bytes;
    static bool attr_set = false;     // set once, outside any stream capture
    if (!attr_set) {
        DGPU_CUDA(ctx, cudaFuncSetAttribute(k_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        attr_set = true;
    }
    DGPU_CUDA(ctx, ctx->flag.ensure(64));
    L.err = ctx->flag.as<int32_t>() + 8;
    return DGPU_OK;
}

int dgpu_tc_launch(dgpu_ctx *ctx, const TcPlan &plan)
{
    DGPU_CUDA(ctx, cudaMemsetAsync(plan.L.err, 0, sizeof(int32_t), ctx->stream));
    if (plan.L.nitems < 1) return DGPU_OK;
    const int grid = (int)(plan.L.nitems < ctx->nsm ? plan.L.nitems : ctx->nsm);
    k_tc<<<grid, TC_THREADS, plan.smem, ctx->stream>>>(plan.L);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

int dgpu_tc_check(dgpu_ctx *ctx)
{
    int32_t herr = 0;
    DGPU_CUDA(ctx, cudaMemcpyAsync(&herr, ctx->flag.as<int32_t>() + 8, sizeof(int32_t), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (herr) return dgpu_set_error(ctx, DGPU_ERR_TIMEOUT, "tensor-core kernel wait gave up (site %d)", herr);
    return DGPU_OK;
}

// Candidate configurations: every column axis and tile width whose padded
// MMA area is within 25% of the smallest, at two slicings.
static void tc_candidates(const BoxSpec &box, int want_n, TcChoice *out, int &n)
{
    double best = 1e300;
    for (int a = 0; a < 3; a++)
        for (int N = 16; N <= 128; N += 16) {
            if ((want_n && N != want_n) || (!want_n && N < 48)) continue;
            const double ar = tc_area(box, a, N);
            if (ar >= 0 && ar < best) best = ar;
        }
    n = 0;
    for (int a = 0; a < 3; a++)
        for (int N = 16; N <= 128; N += 16) {
            if ((want_n && N != want_n) || (!want_n && N < 48)) continue;
            const double ar = tc_area(box, a, N);
            if (ar < 0 || ar > 1.25 * best) continue;
            for (int m : {4, 8}) {
                if (n >= 64) return;
                out[n].axis = a;
                out[n].N = N;
                out[n].slice_mult = m;
                n++;
            }
        }
}

int dgpu_tc_sums(dgpu_ctx *ctx, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw,
                 const float *w, const int64_t *h_type_start, int32_t ntype, const BoxSpec &box,
                 const dgpu_opts *op, DevBuf &part, int32_t *nslice_out)
{
    if (ntype < 1 || ntype > 64) return dgpu_set_error(ctx, DGPU_ERR_ARG, "ntype=%d", ntype);
    const int want_n = op->tc_tile_n;
    if (want_n && (want_n % 16 || want_n < 16 || want_n > 128))
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "tc_tile_n=%d (multiple of 16 in 16..128)", want_n);
    int64_t maxn = 0;
    for (int t = 0; t < ntype; t++) {
        const int64_t n = h_type_start[t + 1] - h_type_start[t];
        maxn = n > maxn ? n : maxn;
    }
    int lg = 0;
    while ((1LL << lg) < maxn) lg++;
    const TcKey key(box.f[0], box.f[1], box.f[2], ntype, lg, op->split * 1000 + want_n,
                    op->tc_kslice * 7 + op->tc_flush);
    TcInput in;
    in.ph0 = ph0;
    in.du = du;
    in.dv = dv;
    in.dw = dw;
    in.w = w;
    in.ts = h_type_start;
    in.ntype = ntype;
    in.box = box;
    TcChoice choice;
    auto hit = ctx->tc_tuned.find(key);
    if (hit != ctx->tc_tuned.end()) {
        choice = hit->second;
    } else {
        TcChoice cand[64];
        int nc = 0;
        tc_candidates(box, want_n, cand, nc);
        if (nc == 0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "no tensor-core tile fits the box");
        float best = 1e30f;
        for (int c = 0; c < nc; c++) {
            in.axis = cand[c].axis;
            TcPlan plan;
            if (dgpu_tc_plan(ctx, 1, &in, op, cand[c].N, cand[c].slice_mult, plan, part, ctx->tc_part)) continue;
            DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
            int rc = dgpu_tc_launch(ctx, plan);
            if (rc) return rc;
            DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[5], ctx->stream));
            rc = dgpu_tc_check(ctx);
            if (rc) return rc;
            float ms = 0.f;
            DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]));
            if (ms < best) {
                best = ms;
                choice = cand[c];
            }
        }
        ctx->tc_tuned[key] = choice;
    }
    in.axis = choice.axis;
    TcPlan plan;
    int rc = dgpu_tc_plan(ctx, 1, &in, op, choice.N, choice.slice_mult, plan, part, ctx->tc_part);
    if (rc) return rc;
    rc = dgpu_tc_launch(ctx, plan);
    if (rc) return rc;
    rc = dgpu_tc_check(ctx);
    if (rc) return rc;
    ctx->tc_last[0] = plan.probs[0].ac;
    ctx->tc_last[1] = plan.probs[0].N;
    ctx->tc_last[2] = plan.L.nbuf;
    ctx->tc_last[3] = (int32_t)plan.probs[0].slice_len;
    *nslice_out = plan.nslice[0];
    return DGPU_OK;
}
