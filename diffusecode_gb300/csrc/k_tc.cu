// Tensor-core engine: the type sums as a split-precision complex GEMM on
// tcgen05 (sm_100 family), accumulators in TMEM.
//
// For the computed box, one grid axis ac is the GEMM's N dimension
// ("columns"); the other two, ra (the longer) and rb, flattened with ra padded
// to a multiple of 8 (fra_p), form its M dimension ("rows": rg = nb*fra_p+na).
// The phase of point (row, column c) and atom j splits exactly:
//     phase = [ph0_j + na d_ra,j + nb d_rb,j] + [n_c d_ac,j]
// so  S(row,c) = sum_j U[row,j] V[j,c]  with  U = w_j exp(2 pi i A-phase),
// V = exp(2 pi i B-phase); K = the atoms of one type (a slice of them per
// work item).
//
// Operand generation.  Each CTA generates its U tile (128 rows) in shared
// memory from the 64-bit fixed-point phases, and V either the same way (V
// generated in the kernel, 32-atom stages) or not at all: with V images
// (k_tc_vgen, written once per launch) a copy warp streams them into a ring
// (64-atom stages).  A producer thread evaluates exp(2 pi i phase) at the
// start of a run of rows (or columns) (from the exact 64-bit phase) and then
// steps by the per-atom factors exp(2 pi i 8 d) and exp(2 pi i 16 d)
// (computed once per atom, rounded stochastically); a row run restarts from
// the exact phase wherever nb changes.  U is evaluated at phase + rot_j and V
// at phase - rot_j, a pseudo-random offset per atom (tc_rot): the product is
// the same, but the evaluation errors of atoms at equivalent positions no
// longer coincide (they would add up coherently).  Every FP32 value is
// split into hi (the value with its mantissa cut to the fp16 / bf16 width,
// exact in that format) and lo (the exact remainder, rounded).  V is scaled
// by 2^12 so that its lo parts stay normal fp16 numbers; all accumulators
// therefore carry 2^12, removed when they are drained.
//
// MMA form.  B holds the rows [Vr; Vi; -Vr] (3N rows), so per 16 atoms
//     D[:, 0:2N] += Ur [Vr;Vi]^T   and   D += (-Ui) [Vi;-Vr]^T
// give Re (accumulator columns 0..N-1) and Im (N..2N-1) with two MMAs of
// width 2N.  The (hi,hi) products go to the main accumulator, the (hi,lo) and
// (lo,hi) products to the correction accumulator.
//
// Accumulation.  Every MMA truncates its FP32 accumulator by about one ulp, so
// the error of one TMEM accumulator grows with the number of MMAs chained into
// it.  The main accumulator is therefore drained every `flush` stages
// (128 atoms) and added with round-to-nearest FP32 adds to a running sum
// (kept in TMEM when N <= 64, otherwise in the work item's partial in global
// memory); the small corrections accumulate over the whole work item.  With
// nbuf = 2 the main accumulator is double-buffered so that a drain overlaps the
// next chunk.  The combine kernel adds the K slices of all work items in FP64.
//
// Partials: part[(t*nslice + ks)*slab + c*nrows_p + rg], a column-major image
// of the tile space (rows with na >= fra are never written).
//
// Warp roles (448 threads): warps 0-7 produce operand stages, warp 8 owns
// TMEM and issues the MMAs (its lane 0 alone), warps 9-12 drain TMEM, warp 13
// streams the V operand images into their ring (one lane).  All
// waits are bounded (globaltimer); a wait that gives up sets an error flag,
// the CTA stops issuing, waits for its own MMAs, frees TMEM and returns.
//
// Shared-memory operands use the canonical K-major layouts: with V images, a
// row holds the 64 atoms of a stage (128 B) with the 128-byte swizzle (8-row
// groups 1024 B apart, the 16-byte chunk c of row r at chunk c ^ (r & 7));
// with V generated in the kernel, 32 atoms (64 B) with the 64-byte swizzle
// (8-row groups 512 B apart, chunk c of row r at c ^ ((r & 7) >> 1)).
#include "dgpu_internal.h"

#define TC_KA 32                               // atoms per stage, V generated in the kernel (64-byte rows)
#define TC_KB 64                               // atoms per stage, V from images (128-byte rows)
#define TC_M 128
#define TC_PROD_WARPS 8
#define TC_MMA_WARP 8
#define TC_EPI_WARP0 9
#define TC_COPY_WARP 13
#define TC_THREADS (14 * 32)
#define TC_PROD_THREADS (TC_PROD_WARPS * 32)
#define TC_A_BYTES (TC_M * TC_KA * 2)          // one A operand (e.g. Ur_hi): 8 KB
#define TC_B_BYTES (TC_M * TC_KB * 2)          // one A operand on the V-image path: 16 KB
// phase data of one 32-atom group in shared memory:
// ph0, d_ra, d_rb, d_ac (u64), w (f32), step factors along ra and ac and
// their squares (float2)
#define TC_SLOT_W (TC_KA * 32)
#define TC_SLOT_MA (TC_SLOT_W + TC_KA * 4)
#define TC_SLOT_MC (TC_SLOT_MA + TC_KA * 8)
#define TC_SLOT_MA2 (TC_SLOT_MC + TC_KA * 8)
#define TC_SLOT_MC2 (TC_SLOT_MA2 + TC_KA * 8)
#define TC_ATOM_SLOT (TC_SLOT_MC2 + TC_KA * 8)
#define TC_NSLOT 3
#define TC_VSLOTS 2                            // V ring: 64-atom images, one stage ahead
#define TC_BAR_BYTES 256
#define TC_SMEM_BUDGET (220 * 1024)
#define TC_SMEM_MAX (227 * 1024)                // the opt-in maximum of one CTA
#ifndef TC_FLUSH_STAGES
#define TC_FLUSH_STAGES 4                      // 128 atoms per drain of the main accumulator (32-atom stages)
#endif
#define TC_V_SCALE 4096.0f
#define TC_UNSCALE (1.0f / 4096.0f)

#include "dgpu_phasor.cuh"
#include "tc_ptx.cuh"

// barrier among the producer warps only; returns the OR of `stop` over them,
// so that all producers leave their loops at the same barrier (a thread that
// left alone would keep the others waiting at the next one)
__device__ __forceinline__ bool producers_sync(bool stop)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\tsetp.ne.u32 q, %1, 0;\n\tbar.red.or.pred p, 1, %2, q;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(r)
        : "r"((uint32_t)stop), "n"(TC_PROD_THREADS)
        : "memory");
    return r != 0;
}


__device__ __forceinline__ void decode_item(const TcProblem &g, int64_t item, int &t, int &ks, int &nt, int &mt)
{
    mt = (int)(item % g.m_tiles);
    int64_t r = item / g.m_tiles;
    nt = (int)(r % g.n_tiles);
    r /= g.n_tiles;
    ks = (int)(r % g.nslice);
    t = (int)(r / g.nslice);
}

// Source arrays of one problem, held in registers by the producers.
struct TcSrc {
    const uint64_t *ph0, *dra, *drb, *dac;
    const float *w;
    const float2 *ma, *mc, *ma2, *mc2;
};

// Stage the phase data of the 32-atom group starting at padded atom ab into
// an atom slot: 136 chunks of 16 bytes, one per thread of tid < 136.
__device__ __forceinline__ void stage_atoms(const TcSrc &P, uint8_t *dst, int64_t ab, int tid)
{
    if (tid < 64) {                     // ph0, d_ra, d_rb, d_ac: 16 chunks each
        const int arr = tid >> 4, ch = tid & 15;
        const uint64_t *src = arr == 0 ? P.ph0 : arr == 1 ? P.dra : arr == 2 ? P.drb : P.dac;
        cp_async16(dst + arr * (TC_KA * 8) + ch * 16, src + ab + ch * 2);
    } else if (tid < 72) {              // w: 8 chunks
        const int ch = tid - 64;
        cp_async16(dst + TC_SLOT_W + ch * 16, P.w + ab + ch * 4);
    } else if (tid < 136) {             // step factors along ra and ac and their squares: 16 chunks each
        const int arr = (tid - 72) >> 4, ch = (tid - 72) & 15;
        const int off = arr == 0 ? TC_SLOT_MA : arr == 1 ? TC_SLOT_MC : arr == 2 ? TC_SLOT_MA2 : TC_SLOT_MC2;
        const float2 *src = arr == 0 ? P.ma : arr == 1 ? P.mc : arr == 2 ? P.ma2 : P.mc2;
        cp_async16(dst + off + ch * 16, src + ab + ch * 2);
    }
    cp_async_commit();
}

// Split 4 complex values (4 atoms of one row or column) into the hi and lo
// operand words of the real and imaginary parts.
template <bool BF>
__device__ __forceinline__ void split_c4(const float2 (&x)[4], uint2 &rh, uint2 &rl, uint2 &ih, uint2 &il)
{
    split4<BF>(x[0].x, x[1].x, x[2].x, x[3].x, rh, rl);
    split4<BF>(x[0].y, x[1].y, x[2].y, x[3].y, ih, il);
}

// U row group q: Ur hi/lo and Ui hi/lo at the thread's row and atom quad
template <bool BF>
__device__ __forceinline__ void emit_rows(uint8_t *dst, int q, const float2 (&x)[4])
{
    uint2 rh, rl, ih, il;
    split_c4<BF>(x, rh, rl, ih, il);
    uint8_t *d = dst + q * TC_SBO;
    *reinterpret_cast<uint2 *>(d + 0 * TC_A_BYTES) = rh;
    *reinterpret_cast<uint2 *>(d + 1 * TC_A_BYTES) = rl;
    *reinterpret_cast<uint2 *>(d + 2 * TC_A_BYTES) = ih;
    *reinterpret_cast<uint2 *>(d + 3 * TC_A_BYTES) = il;
}

// V column group q: rows c (Vr), N+c (Vi) and 2N+c (-Vr) of the hi and lo operands
template <bool BF>
__device__ __forceinline__ void emit_cols(uint8_t *Bh, uint32_t b_bytes, uint32_t blk, uint32_t o0, int q,
                                          const float2 (&x)[4])
{
    uint2 rh, rl, ih, il;
    split_c4<BF>(x, rh, rl, ih, il);
    uint8_t *d = Bh + q * TC_SBO + o0;
    const uint2 nrh = make_uint2(rh.x ^ 0x80008000u, rh.y ^ 0x80008000u);
    const uint2 nrl = make_uint2(rl.x ^ 0x80008000u, rl.y ^ 0x80008000u);
    *reinterpret_cast<uint2 *>(d) = rh;
    *reinterpret_cast<uint2 *>(d + b_bytes) = rl;
    *reinterpret_cast<uint2 *>(d + blk) = ih;
    *reinterpret_cast<uint2 *>(d + blk + b_bytes) = il;
    *reinterpret_cast<uint2 *>(d + 2 * blk) = nrh;
    *reinterpret_cast<uint2 *>(d + 2 * blk + b_bytes) = nrl;
}

// Groups [q, qe) from the value x at group q: two interleaved chains
// (even groups and odd groups, each stepping by m^2) give the recurrence
// twice the instruction-level parallelism; the next pair is formed before the
// current pair is split and stored.
template <class Emit>
__device__ __forceinline__ void run_pairs(int q, int qe, float2 (&x0)[4], const float2 (&m)[4],
                                          const float2 (&m2)[4], Emit emit)
{
    float2 x1[4];
#pragma unroll
    for (int a = 0; a < 4; a++) x1[a] = cmulf(x0[a], m[a]);
#pragma unroll 1
    for (; q < qe; q += 2) {
        float2 y0[4], y1[4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            y0[a] = cmulf(x0[a], m2[a]);
            y1[a] = cmulf(x1[a], m2[a]);
        }
        emit(q, x0);
        if (q + 1 < qe) emit(q + 1, x1);
#pragma unroll
        for (int a = 0; a < 4; a++) {
            x0[a] = y0[a];
            x1[a] = y1[a];
        }
    }
}

// U rows of one stage for row groups [q0, q1) of the tile (8 rows each).
// The thread owns atoms k0..k0+3 and row s of every group.  Within each
// segment of constant nb it starts from the exact phase and steps by
// exp(2 pi i 8 d_ra) from group to group.  A warp's stores of one step cover
// 16 distinct 8-byte bank slots.
template <bool BF>
__device__ __forceinline__ void gen_rows(int q0, int q1, int mt, int gpn, const uint8_t *as, uint8_t *A, int s,
                                         int j, int64_t ab)
{
    const uint64_t *s_ph0 = reinterpret_cast<const uint64_t *>(as);
    const uint64_t *s_dra = s_ph0 + TC_KA, *s_drb = s_dra + TC_KA;
    const float *s_w = reinterpret_cast<const float *>(as + TC_SLOT_W);
    const float2 *s_ma = reinterpret_cast<const float2 *>(as + TC_SLOT_MA);
    const float2 *s_ma2 = reinterpret_cast<const float2 *>(as + TC_SLOT_MA2);
    const int G0 = mt * (TC_M / 8) + q0;
    int gi = G0 % gpn;
    uint32_t nb = (uint32_t)(G0 / gpn);
    const int k0 = 4 * j;
    float2 m[4], m2[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        m[a] = s_ma[k0 + a];
        m2[a] = s_ma2[k0 + a];
    }
    uint8_t *dst = A + sw_off(s, j >> 1) + (j & 1) * 8;
    auto emit = [&](int q, const float2 (&x)[4]) { emit_rows<BF>(dst, q, x); };
    for (int q = q0; q < q1;) {            // segments of constant nb (warp-uniform)
        const int qe = min(q1, q + (gpn - gi));
        const uint32_t na = (uint32_t)(gi * 8 + s);
        float2 x[4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int k = k0 + a;
            const float2 p =
                phasor_fast(tc_rot((uint64_t)(ab + k)) + s_ph0[k] + (uint64_t)na * s_dra[k] + (uint64_t)nb * s_drb[k]);
            const float wk = s_w[k];
            x[a] = make_float2(p.x * wk, p.y * wk);
        }
        run_pairs(q, qe, x, m, m2, emit);
        q = qe;
        gi = 0;
        nb++;
    }
}

// 2 complex values (2 consecutive atoms of one row) -> the hi and lo words of
// the real and imaginary parts, low half = first atom.
template <bool BF>
__device__ __forceinline__ void split_c2(const float2 (&x)[2], uint32_t &rh, uint32_t &rl, uint32_t &ih,
                                         uint32_t &il)
{
    const uint32_t mask = BF ? 0xFFFF0000u : 0xFFFFE000u;
    const float hr0 = __uint_as_float(__float_as_uint(x[0].x) & mask);
    const float hr1 = __uint_as_float(__float_as_uint(x[1].x) & mask);
    const float hi0 = __uint_as_float(__float_as_uint(x[0].y) & mask);
    const float hi1 = __uint_as_float(__float_as_uint(x[1].y) & mask);
    rh = pack2<BF>(hr0, hr1);
    rl = pack2<BF>(x[0].x - hr0, x[1].x - hr1);
    ih = pack2<BF>(hi0, hi1);
    il = pack2<BF>(x[0].y - hi0, x[1].y - hi1);
}

// Phase data of the thread's two atoms for one stage, loaded from global
// memory one stage ahead (16-byte loads: the atoms are consecutive and even).
struct AtomPair {
    ulonglong2 ph0, dra, drb;
    float2 w;
    float4 m;               // step factors exp(2 pi i 8 d_ra) of the two atoms
    float4 m2;              // and exp(2 pi i 16 d_ra)
    uint64_t rot0, rot1;    // the atoms' phase offsets (tc_rot)
};

__device__ __forceinline__ void load_pair(AtomPair &r, const TcSrc &P, int64_t k)
{
    r.ph0 = __ldg(reinterpret_cast<const ulonglong2 *>(P.ph0 + k));
    r.dra = __ldg(reinterpret_cast<const ulonglong2 *>(P.dra + k));
    r.drb = __ldg(reinterpret_cast<const ulonglong2 *>(P.drb + k));
    r.w = __ldg(reinterpret_cast<const float2 *>(P.w + k));
    r.m = __ldg(reinterpret_cast<const float4 *>(P.ma + k));
    r.m2 = __ldg(reinterpret_cast<const float4 *>(P.ma2 + k));
    r.rot0 = tc_rot((uint64_t)k);
    r.rot1 = tc_rot((uint64_t)k + 1);
}

// Where the 16 row groups of tile mt start (group G0 = 16 mt at gi0, nb0)
// and which of them begin a new nb (bit o: group G0 + o): fixed for all
// stages of a work item.
struct RowSeg {
    uint32_t gi0, nb0, bmask;
};

__device__ __forceinline__ RowSeg row_segments(int mt, int gpn)
{
    const int G0 = mt * (TC_M / 8);
    RowSeg r;
    r.gi0 = (uint32_t)(G0 % gpn);
    r.nb0 = (uint32_t)(G0 / gpn);
    r.bmask = 0;
    int gi = (int)r.gi0;
#pragma unroll
    for (int o = 0; o < TC_M / 8; o++) {
        if (o > 0 && gi == 0) r.bmask |= 1u << o;
        if (++gi == gpn) gi = 0;
    }
    return r;
}

// The thread's stmatrix address within a stage: row (lane & 7) of matrix
// (lane >> 3), i.e. of row group lane >> 3, in atom chunk warp.
__device__ __forceinline__ uint32_t stm_offset(int lane, int warp)
{
    return (uint32_t)(lane >> 3) * TC_SBO128 + sw128_off(lane & 7, warp);
}

// U rows of one 64-atom stage (128-byte rows), stored with stmatrix: warp w
// generates atom chunk w (atoms 8w..8w+7) of all 16 row groups; lane l owns
// row l >> 2 of each group and atoms 8w + 2 (l & 3) + {0, 1}, the fragment
// layout of an 8x8 b16 matrix, so that one stmatrix.x4 stores four row
// groups of one operand array.  Values step from group to group by
// exp(2 pi i 8 d_ra) on two chains (even and odd groups, by its square) and
// restart from the exact phase at every group that begins a new nb.

template <bool BF>
__device__ __forceinline__ void gen_rows_stm(const RowSeg &rs, const AtomPair &ap, uint32_t adr, int lane)
{
    const int s = lane >> 2;
    const uint64_t ph0[2] = {ap.ph0.x, ap.ph0.y}, dra[2] = {ap.dra.x, ap.dra.y}, drb[2] = {ap.drb.x, ap.drb.y};
    const float w[2] = {ap.w.x, ap.w.y};
    const uint64_t rot[2] = {ap.rot0, ap.rot1};
    float2 m[2], m2[2];
    m[0] = make_float2(ap.m.x, ap.m.y);
    m[1] = make_float2(ap.m.z, ap.m.w);
    m2[0] = make_float2(ap.m2.x, ap.m2.y);
    m2[1] = make_float2(ap.m2.z, ap.m2.w);
    // segments of constant nb: bit o of bmask marks group G0 + o as the first
    // of a segment
    const uint32_t gi0 = rs.gi0, nb0 = rs.nb0, bmask = rs.bmask;
    // exact value at group G0 + o: offset 0, or the start of a segment
    auto seed = [&](int o, float2 (&x)[2]) {
        const uint32_t na = (uint32_t)((o == 0 ? gi0 * 8 : 0) + s);
        const uint32_t nb = nb0 + (uint32_t)__popc(bmask & ((2u << o) - 1u));
#pragma unroll
        for (int a = 0; a < 2; a++) {
            const float2 p = phasor_fast(rot[a] + ph0[a] + (uint64_t)na * dra[a] + (uint64_t)nb * drb[a]);
            x[a] = make_float2(p.x * w[a], p.y * w[a]);
        }
    };
    auto starts = [&](int o) { return ((bmask >> o) & 1u) != 0u; };
    float2 e[2], o[2];                 // groups G0 + 2p (even chain) and G0 + 2p + 1 (odd chain)
    seed(0, e);
    if (starts(1)) seed(1, o);
    else {
#pragma unroll
        for (int a = 0; a < 2; a++) o[a] = cmulf(e[a], m[a]);
    }
    uint32_t R[4][4];                  // [operand array][matrix = group within four]
#pragma unroll
    for (int p = 0; p < TC_M / 16; p++) {
        const int i = (2 * p) & 3;
        split_c2<BF>(e, R[0][i], R[1][i], R[2][i], R[3][i]);
        split_c2<BF>(o, R[0][i + 1], R[1][i + 1], R[2][i + 1], R[3][i + 1]);
        if (p & 1) {
            const uint32_t base = adr + (uint32_t)(2 * (p - 1)) * TC_SBO128;
#pragma unroll
            for (int arr = 0; arr < 4; arr++)
                stmatrix_x4(base + arr * TC_B_BYTES, R[arr][0], R[arr][1], R[arr][2], R[arr][3]);
        }
        if (p < TC_M / 16 - 1) {
            const int ge = 2 * p + 2, go = ge + 1;      // offsets of the next pair
            float2 ne[2], no[2];
            if (starts(ge)) seed(ge, ne);
            else if (starts(ge - 1)) {
#pragma unroll
                for (int a = 0; a < 2; a++) ne[a] = cmulf(o[a], m[a]);
            } else {
#pragma unroll
                for (int a = 0; a < 2; a++) ne[a] = cmulf(e[a], m2[a]);
            }
            if (starts(go)) seed(go, no);
            else if (starts(ge)) {
#pragma unroll
                for (int a = 0; a < 2; a++) no[a] = cmulf(ne[a], m[a]);
            } else {
#pragma unroll
                for (int a = 0; a < 2; a++) no[a] = cmulf(o[a], m2[a]);
            }
#pragma unroll
            for (int a = 0; a < 2; a++) {
                e[a] = ne[a];
                o[a] = no[a];
            }
        }
    }
}

// V columns of one stage for column groups [q0, q1) of the tile: atoms
// k0..k0+3, column 8q+s of every group, stepping by exp(2 pi i 8 d_ac).
// B rows: Vr at c, Vi at N+c, -Vr at 2N+c, in a hi and a lo operand.
template <bool BF>
__device__ __forceinline__ void gen_cols(int q0, int q1, int nt, int N, const uint8_t *as, uint8_t *Bh,
                                         uint32_t b_bytes, int s, int j, int64_t ab)
{
    const uint64_t *s_dac = reinterpret_cast<const uint64_t *>(as) + 3 * TC_KA;
    const float2 *s_mc = reinterpret_cast<const float2 *>(as + TC_SLOT_MC);
    const float2 *s_mc2 = reinterpret_cast<const float2 *>(as + TC_SLOT_MC2);
    const int k0 = 4 * j;
    const uint32_t nc = (uint32_t)(nt * N + q0 * 8 + s);
    float2 x[4], m[4], m2[4];
#pragma unroll
    for (int a = 0; a < 4; a++) {
        const float2 p = phasor_fast((uint64_t)nc * s_dac[k0 + a] - tc_rot((uint64_t)(ab + k0 + a)));
        x[a] = make_float2(p.x * TC_V_SCALE, p.y * TC_V_SCALE);
        m[a] = s_mc[k0 + a];
        m2[a] = s_mc2[k0 + a];
    }
    const uint32_t blk = (uint32_t)(N >> 3) * TC_SBO;           // N rows further
    const uint32_t o0 = sw_off(s, j >> 1) + (j & 1) * 8;
    auto emit = [&](int q, const float2 (&v)[4]) { emit_cols<BF>(Bh, b_bytes, blk, o0, q, v); };
    run_pairs(q0, q1, x, m, m2, emit);
}

template <bool BF>
__global__ void __launch_bounds__(TC_THREADS, 1) k_tc(const TcLaunch L)
{
    extern __shared__ __align__(1024) uint8_t smem[];
    const int S = L.stages;
    const int NM = L.Nmax;
    // atoms per stage: 64 (128-byte rows) with V images, 32 (64-byte rows)
    // when V is generated in the kernel
    const int KS = L.vring ? TC_KB : TC_KA;
    const uint32_t b_bytes = (uint32_t)3 * NM * KS * 2;         // one B operand: 3N rows
    // stages hold U (and V when it is generated in-kernel); with V images,
    // V lives in a ring of TC_VSLOTS slots of 2 * b_bytes after the stages
    const uint32_t stage_bytes = 4u * TC_M * KS * 2 + (L.vring ? 0u : 2 * b_bytes);
    const uint32_t vbytes = 2 * b_bytes;
    uint8_t *vring = smem + (size_t)S * stage_bytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(vring + (L.vring ? (size_t)TC_VSLOTS * vbytes : 0));
    uint64_t *empty = full + S;
    uint64_t *mfull = empty + S;      // [2] main accumulator b ready
    uint64_t *mempty = mfull + 2;     // [2] main accumulator b drained
    uint64_t *cfull = mempty + 2;     // correction accumulator ready (end of item)
    uint64_t *cempty = cfull + 1;     // correction accumulator drained
    uint64_t *drain = cempty + 1;
    uint64_t *vfull = drain + 1;      // [TC_VSLOTS] V image of the slot landed
    uint64_t *vempty = vfull + TC_VSLOTS;   // [TC_VSLOTS] MMAs reading the slot done
    uint32_t *tbase = reinterpret_cast<uint32_t *>(vempty + TC_VSLOTS);
    uint8_t *aslot = reinterpret_cast<uint8_t *>(full) + TC_BAR_BYTES;   // TC_NSLOT x TC_ATOM_SLOT
    volatile int32_t *err = L.err;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; s++) {
            mbar_init(&full[s], TC_PROD_WARPS);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; b++) {
            mbar_init(&mfull[b], 1);
            mbar_init(&mempty[b], 4 * 32);
        }
        mbar_init(cfull, 1);
        mbar_init(cempty, 4 * 32);
        mbar_init(drain, 1);
        for (int v = 0; v < TC_VSLOTS; v++) {
            mbar_init(&vfull[v], 1);
            mbar_init(&vempty[v], 1);
        }
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

    if (warp < TC_PROD_WARPS && L.vring) {
        // ------------------------------------------------ producers (V images)
        // Every producer warp runs on its own: its lanes wait for the stage
        // buffer (a vote keeps the warp together if a wait gives up), the warp
        // writes its 8-atom chunk of U rows (gen_rows_stm) and lane 0 arrives
        // on the stage's full barrier; the phase data of its atoms is loaded
        // one stage ahead into registers.  No barrier among producers.  Stage
        // index and round are counted, not divided out of `it` (S is a
        // run-time value, and these loops are latency-bound).
        uint32_t it = 0, sb = 0, round = 0;  // it = round * S + sb
        bool ok = true;
        const int kq = 8 * warp + 2 * (lane & 3);           // the thread's first atom in a stage
        const uint32_t adr0 = smem_u32(smem) + stm_offset(lane, warp);
        for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
            const TcProblem &g = L.probs[L.item_prob[item]];
            int t, ks, nt, mt;
            decode_item(g, item - g.item0, t, ks, nt, mt);
            const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
            const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
            const int nst = a1 > a0 ? (int)((a1 - a0) / TC_KB) : 0;
            if (nst == 0) continue;
            const TcSrc src = {g.ph0, g.dra, g.drb, g.dac, g.w, g.ma, g.mc, g.ma2, g.mc2};
            const RowSeg rs = row_segments(mt, g.fra_p >> 3);
            AtomPair cur, nxt;
            load_pair(cur, src, a0 + kq);
            for (int st = 0; st < nst; st++, it++) {
                if (st + 1 < nst) load_pair(nxt, src, a0 + (int64_t)(st + 1) * TC_KB + kq);
                const bool got = round == 0 || mbar_wait(&empty[sb], (round - 1) & 1, err, 1, L.timeout_ns);
                if (!__all_sync(0xffffffffu, got)) {
                    ok = false;
                    break;
                }
                gen_rows_stm<BF>(rs, cur, adr0 + sb * stage_bytes, lane);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[sb]);   // one arrival per producer warp
                cur = nxt;
                if (++sb == (uint32_t)S) {
                    sb = 0;
                    round++;
                }
            }
        }
    } else if (warp < TC_PROD_WARPS) {
        // ------------------------------------------------------------ producers
        // Atom groups are complete (type ranges padded to 64 atoms with zero
        // weight).  Their phase data is staged in shared memory with cp.async
        // one group ahead; three slots, so that a slot is rewritten only after
        // every producer has passed the barrier that follows its last use.
        // Work split: the 16 row groups of U and the N/8 column groups of V
        // form one list, cut into four equal ranges; producer thread
        // (s = lane&7, j = atom quad, u) takes range u for its atom quad.
        const int tid = threadIdx.x;
        const int s = lane & 7, j = (lane >> 3) + 4 * (warp & 1), u = warp >> 1;
        uint32_t it = 0, sb = 0, round = 0;   // it = round * S + sb
        bool ok = true;                     // this thread saw no failed wait
        for (int64_t item = blockIdx.x; item < L.nitems; item += gridDim.x) {
            const TcProblem &g = L.probs[L.item_prob[item]];
            int t, ks, nt, mt;
            decode_item(g, item - g.item0, t, ks, nt, mt);
            const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
            const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
            const int nst = a1 > a0 ? (int)((a1 - a0) / TC_KA) : 0;
            if (nst == 0) continue;
            // previous item's slots are free; everybody stops together after a failure
            if (producers_sync(!ok)) break;
            const TcSrc src = {g.ph0, g.dra, g.drb, g.dac, g.w, g.ma, g.mc, g.ma2, g.mc2};
            const int N = g.N, gpn = g.fra_p >> 3;
            // with V images the column groups arrive by bulk copy into the ring
            const uint8_t *vimg = L.vring ? g.vimg : nullptr;
            const int ngr = TC_M / 8, ntot = ngr + (vimg ? 0 : (N >> 3)), per = (ntot + 3) >> 2;
            const int r0 = u * per, r1 = min(ntot, r0 + per);
            const int ra0 = min(r0, ngr), ra1 = min(r1, ngr);           // row groups
            const int rc0 = max(r0, ngr) - ngr, rc1 = max(r1, ngr) - ngr; // column groups
            // groups st+1 and st+2 are in flight while group st is generated;
            // the slot of group st+2 was last read for group st-1, before the
            // barrier of step st
            stage_atoms(src, aslot, a0, tid);
            if (nst > 1) stage_atoms(src, aslot + TC_ATOM_SLOT, a0 + TC_KA, tid);
            else cp_async_commit();
            for (int st = 0; st < nst; st++, it++) {
                cp_async_wait1();           // group st has landed (only the newest may be pending)
                // one thread waits for the stage buffer, the barrier tells everybody
                if (tid == 0 && ok && round > 0)
                    ok = mbar_wait(&empty[sb], (round - 1) & 1, err, 1, L.timeout_ns);
                if (producers_sync(!ok)) break;   // staged for every producer; slot of st-1 and stage sb free
                if (st + 2 < nst)
                    stage_atoms(src, aslot + ((st + 2) % TC_NSLOT) * TC_ATOM_SLOT, a0 + (int64_t)(st + 2) * TC_KA,
                                tid);
                else
                    cp_async_commit();
                const uint8_t *as = aslot + (st % TC_NSLOT) * TC_ATOM_SLOT;
                uint8_t *A = smem + (size_t)sb * stage_bytes;
                const int64_t ab = a0 + (int64_t)st * TC_KA;        // the stage's first atom
                if (ok && ra0 < ra1) gen_rows<BF>(ra0, ra1, mt, gpn, as, A, s, j, ab);
                if (ok && rc0 < rc1) gen_cols<BF>(rc0, rc1, nt, N, as, A + 4 * TC_A_BYTES, b_bytes, s, j, ab);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&full[sb]);   // one arrival per producer warp
                if (++sb == (uint32_t)S) {
                    sb = 0;
                    round++;
                }
            }
            cp_async_wait0();
        }
    } else if (warp == TC_MMA_WARP) {
        // ------------------------------------------------------------ MMA issuer
        // One thread (lane 0) waits, issues and commits; the other lanes of
        // the warp only join it at the end, so that no warp-wide step sits
        // between two stages.
        bool issued = false;
        if (lane == 0) {
            const uint32_t fmt = BF ? 1u : 0u;
            const uint32_t c_acc = tmem;                                  // correction accumulator
            uint32_t it = 0, nitem = 0, nchunk = 0, s = 0, round = 0;   // it = round * S + s
            bool ok = true;
            for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
                const TcProblem &g = L.probs[L.item_prob[item]];
                const int N = g.N;
                int t, ks, nt, mt;
                decode_item(g, item - g.item0, t, ks, nt, mt);
                const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
                const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
                const int nst = a1 > a0 ? (int)((a1 - a0) / KS) : 0;
                if (nst == 0) continue;
                // D = 128 x 2N, f32; A and B of the operand format
                const uint32_t idesc = (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)((2 * N) >> 3) << 17) |
                                       ((uint32_t)(TC_M >> 4) << 24);
                const uint32_t idesc_neg = idesc | (1u << 13);     // negate A: the -Ui products
                // B rows N.. : [Vi; -Vr]
                const uint32_t b2off = (uint32_t)(N >> 3) * (L.vring ? TC_SBO128 : TC_SBO);
                // the correction accumulator restarts with this item: previous one drained?
                if (nitem > 0 && !mbar_wait(cempty, (nitem - 1) & 1, err, 2, L.timeout_ns)) {
                    ok = false;
                    break;
                }
                for (int st0 = 0; st0 < nst && ok; st0 += L.flush, nchunk++) {
                    const int b = (int)(nchunk % L.nbuf);
                    const uint32_t use = nchunk / L.nbuf;
                    if (use > 0 && !mbar_wait(&mempty[b], (use - 1) & 1, err, 6, L.timeout_ns)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t m_acc = tmem + 2u * NM * (1u + (uint32_t)b);
                    const int st1 = min(nst, st0 + L.flush);
                    for (int st = st0; st < st1; st++, it++) {
                        if (!mbar_wait(&full[s], round & 1, err, 3, L.timeout_ns) ||
                            (L.vring &&
                             !mbar_wait(&vfull[it % TC_VSLOTS], (it / TC_VSLOTS) & 1, err, 8, L.timeout_ns))) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t A = smem_u32(smem + (size_t)s * stage_bytes);
                        const uint32_t Bh =
                            L.vring ? smem_u32(vring) + (it % TC_VSLOTS) * vbytes : A + 4 * TC_A_BYTES;
                        // descriptors: the start-address field (addr >> 4, 14 bits) is the
                        // low field, and every operand lies below 256 KB, so an offset is a
                        // plain add to the base descriptor; a K step of 16 atoms is 32 bytes
                        const uint64_t bl_off = b_bytes >> 4, b2_off = b2off >> 4;
                        auto issue = [&](uint64_t dA, uint64_t dB, uint32_t a_bytes, int nk) {
#pragma unroll 4
                            for (int kk = 0; kk < nk; kk++) {
                                const uint64_t ko = (uint64_t)kk * 2;
                                const uint64_t arh = dA + ko, arl = dA + (a_bytes >> 4) + ko;
                                const uint64_t aih = dA + (2 * a_bytes >> 4) + ko, ail = dA + (3 * a_bytes >> 4) + ko;
                                const uint64_t b1h = dB + ko, b2h = dB + b2_off + ko;
                                const uint64_t b1l = dB + bl_off + ko, b2l = dB + bl_off + b2_off + ko;
                                const uint32_t am = (st > st0 || kk > 0) ? 1u : 0u;   // main restarts per chunk
                                const uint32_t ac = (st > 0 || kk > 0) ? 1u : 0u;     // correction per item
                                // main: (hi,hi)
                                mma_f16(m_acc, arh, b1h, idesc, am);
                                mma_f16(m_acc, aih, b2h, idesc_neg, 1u);
                                // corrections: (hi,lo) and (lo,hi)
                                mma_f16(c_acc, arh, b1l, idesc, ac);
                                mma_f16(c_acc, aih, b2l, idesc_neg, 1u);
                                mma_f16(c_acc, arl, b1h, idesc, 1u);
                                mma_f16(c_acc, ail, b2h, idesc_neg, 1u);
                            }
                        };
                        if (L.vring) issue(sdesc128(A), sdesc128(Bh), TC_B_BYTES, TC_KB / 16);
                        else issue(sdesc(A), sdesc(Bh), TC_A_BYTES, TC_KA / 16);
                        mma_commit(&empty[s]);
                        if (L.vring) mma_commit(&vempty[it % TC_VSLOTS]);
                        issued = true;
                        if (++s == (uint32_t)S) {
                            s = 0;
                            round++;
                        }
                    }
                    if (!ok) break;
                    mma_commit(&mfull[b]);
                }
                if (!ok) break;
                mma_commit(cfull);
                nitem++;
            }
            // make sure no MMA of this CTA is still running before TMEM is freed
            if (issued) {
                mma_commit(drain);
                mbar_wait_quiet(drain, 0);
            }
        }
        __syncwarp();
        tc_fence_before();
    } else if (warp < TC_COPY_WARP) {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;                       // TMEM lane quadrant of this warp
        const int r = q * 32 + lane;
        const uint32_t lane_off = (uint32_t)(q * 32) << 16;
        const uint32_t t_corr = tmem + lane_off;
        const uint32_t t_sum = tmem + lane_off + 2u * NM * (1u + (uint32_t)L.nbuf);
        uint32_t nitem = 0, nchunk = 0;
        bool ok = true;
        for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
            const TcProblem &g = L.probs[L.item_prob[item]];
            const int N = g.N;
            int t, ks, nt, mt;
            decode_item(g, item - g.item0, t, ks, nt, mt);
            const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
            const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
            const int nst = a1 > a0 ? (int)((a1 - a0) / KS) : 0;
            const int64_t rg = (int64_t)mt * TC_M + r;
            const bool rv = rg < g.nrows_p && (int)(rg % g.fra_p) < g.fra;
            const int64_t nrp = g.nrows_p;
            const int ncv = min(N, g.ncols - nt * N);             // valid columns of this tile
            float2 *oc = g.part + ((int64_t)t * g.nslice + ks) * g.slab + (int64_t)nt * N * nrp + rg;
            if (nst == 0) {
                if (rv)
                    for (int c = 0; c < ncv; c++) oc[(int64_t)c * nrp] = make_float2(0.f, 0.f);
                continue;
            }
            for (int st0 = 0; st0 < nst; st0 += L.flush, nchunk++) {
                const int b = (int)(nchunk % L.nbuf);
                const bool got = lane == 0 ? mbar_wait(&mfull[b], (nchunk / L.nbuf) & 1, err, 5, L.timeout_ns) : true;
                if (!__shfl_sync(0xffffffffu, got, 0)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const bool first = st0 == 0, last = st0 + L.flush >= nst;
                if (last) {                                        // the item's corrections
                    const bool gc = lane == 0 ? mbar_wait(cfull, nitem & 1, err, 7, L.timeout_ns) : true;
                    if (!__shfl_sync(0xffffffffu, gc, 0)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                }
                const uint32_t t_main = tmem + lane_off + 2u * NM * (1u + (uint32_t)b);
                const bool keep = L.tsum && !last;                 // running sum stays in TMEM
                for (int c0 = 0; c0 < N; c0 += 16) {
                    uint32_t vr[16], vi[16];
                    float fr[16], fi[16];
                    tmem_ld16(t_main + (uint32_t)c0, vr);
                    tmem_ld16(t_main + (uint32_t)(N + c0), vi);
                    tmem_wait_ld();
#pragma unroll
                    for (int k = 0; k < 16; k++) {
                        fr[k] = __uint_as_float(vr[k]);
                        fi[k] = __uint_as_float(vi[k]);
                    }
                    if (L.tsum && !first) {
                        tmem_ld16(t_sum + (uint32_t)c0, vr);
                        tmem_ld16(t_sum + (uint32_t)(N + c0), vi);
                        tmem_wait_ld();
#pragma unroll
                        for (int k = 0; k < 16; k++) {
                            fr[k] += __uint_as_float(vr[k]);
                            fi[k] += __uint_as_float(vi[k]);
                        }
                    }
                    if (last) {
                        tmem_ld16(t_corr + (uint32_t)c0, vr);
                        tmem_ld16(t_corr + (uint32_t)(N + c0), vi);
                        tmem_wait_ld();
#pragma unroll
                        for (int k = 0; k < 16; k++) {
                            fr[k] += __uint_as_float(vr[k]);
                            fi[k] += __uint_as_float(vi[k]);
                        }
                    }
                    if (keep) {
#pragma unroll
                        for (int k = 0; k < 16; k++) {
                            vr[k] = __float_as_uint(fr[k]);
                            vi[k] = __float_as_uint(fi[k]);
                        }
                        tmem_st16(t_sum + (uint32_t)c0, vr);
                        tmem_st16(t_sum + (uint32_t)(N + c0), vi);
                    } else if (rv) {
#pragma unroll
                        for (int k = 0; k < 16; k++) {
                            if (c0 + k < ncv) {
                                float2 *o = oc + (int64_t)(c0 + k) * nrp;
                                float2 v = make_float2(fr[k] * TC_UNSCALE, fi[k] * TC_UNSCALE);
                                if (!L.tsum && !first) {
                                    const float2 old = *o;
                                    v.x += old.x;
                                    v.y += old.y;
                                }
                                *o = v;
                            }
                        }
                    }
                }
                if (keep) tmem_wait_st();
                tc_fence_before();
                mbar_arrive(&mempty[b]);
                if (last) mbar_arrive(cempty);
            }
            if (!ok) break;
            nitem++;
        }
    } else {
        // ------------------------------------------------------------ V copies
        // Lane 0 streams the V operand images of every stage into the ring, up
        // to TC_VSLOTS stages ahead of the MMAs: a slot is refilled once the
        // MMAs that read it have completed.  Off the producers' path, so that
        // their stage barrier never waits for a slot.
        if (L.vring && lane == 0) {
            uint32_t x = 0, landed = 0;       // copies issued / first copy not known to have landed
            bool ok = true;
            for (int64_t item = blockIdx.x; item < L.nitems && ok; item += gridDim.x) {
                const TcProblem &g = L.probs[L.item_prob[item]];
                int t, ks, nt, mt;
                decode_item(g, item - g.item0, t, ks, nt, mt);
                const int64_t a0 = g.ts[t] + (int64_t)ks * g.slice_len;
                const int64_t a1 = min(g.ts[t + 1], a0 + g.slice_len);
                const int nst = a1 > a0 ? (int)((a1 - a0) / TC_KB) : 0;
                const int64_t g0 = a0 / TC_KB;
                for (int y = 0; y < nst; y++, x++) {
                    const int v = (int)(x % TC_VSLOTS);
                    if (x >= TC_VSLOTS) {
                        if (!mbar_wait(&vempty[v], ((x / TC_VSLOTS) - 1) & 1, err, 9, L.timeout_ns)) {
                            ok = false;
                            break;
                        }
                        landed = x - TC_VSLOTS + 1;       // the MMAs consumed that copy: it landed
                    }
                    mbar_arrive_tx(&vfull[v], vbytes);
                    bulk_g2s(vring + (size_t)v * vbytes, g.vimg + ((g0 + y) * g.vstride + nt) * (int64_t)vbytes,
                             vbytes, &vfull[v]);
                }
            }
            // copies still in flight land before the CTA can exit (after an
            // error the MMA side may not have waited for them)
            for (uint32_t y = landed; y < x; y++) mbar_wait_quiet(&vfull[y % TC_VSLOTS], (y / TC_VSLOTS) & 1);
        }
        __syncwarp();
    }
    __syncthreads();
    if (warp == TC_MMA_WARP) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(L.tmem_cols)
                     : "memory");
    }
}

// FP64 -> FP32 with stochastic rounding, in integer arithmetic on the bits:
// the 29 significand bits that FP32 drops get a uniform 29-bit draw added
// (u >> 3) and are cut off, so the magnitude rounds up (a carry, which may
// run into the exponent) with probability equal to its distance from the
// lower neighbour in units of the spacing, and the rounding error has mean
// zero over draws.  The FP32 word is then assembled from sign, rebased
// exponent and the top 23 significand bits (no FP64 instruction: this part's
// FP64 rate is low).  For |y| in the normal FP32 range; zero stays zero.
__device__ __forceinline__ float round_stochastic(double y, uint32_t u)
{
    uint64_t b = (uint64_t)__double_as_longlong(y);
    const int e0 = (int)((b >> 52) & 0x7FF);
    if (e0 < 1023 - 125) return __uint_as_float((uint32_t)(b >> 32) & 0x80000000u);   // |y| < 2^-125: zero
    b += (uint64_t)(u >> 3);
    const uint32_t sign = (uint32_t)(b >> 32) & 0x80000000u;
    const uint32_t e = (uint32_t)((b >> 52) & 0x7FF) - 1023u + 127u;
    const uint32_t man = (uint32_t)(b >> 29) & 0x7FFFFFu;
    return __uint_as_float(sign | (e << 23) | man);
}

// exp(2 pi i t) for a 64-bit fixed-point turn t, in FP64 to about 1e-16:
// the table entry of its top 12 bits (tab[k] = exp(2 pi i k / 4096)) times
// exp(i e) of the remaining angle e < 2 pi 2^-12, by its Taylor series
// (the first omitted terms are below 1e-16).
__device__ __forceinline__ double2 phasor_f64(uint64_t t, const double2 *__restrict__ tab)
{
    const double2 a = tab[t >> 52];
    const double e = (double)(t & 0xFFFFFFFFFFFFFull) * (6.283185307179586 * 0x1p-64);
    const double e2 = e * e;
    const double c = 1.0 - e2 * (0.5 - e2 * (1.0 / 24.0));
    const double s = e * (1.0 - e2 * (1.0 / 6.0));
    return make_double2(a.x * c - a.y * s, a.x * s + a.y * c);
}

__global__ void k_tc_tab(double2 *tab)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= 4096) return;
    double s, c;
    sincospi((double)k / 2048.0, &s, &c);
    tab[k] = make_double2(c, s);
}

// the CUDA-core engines' phasor table (dgpu_phasor.cuh): exp(2 pi i j / 1024)
// rounded to FP32, entry 4j of the table above
__global__ void k_ph_tab(const double2 *__restrict__ tc_tab, float2 *__restrict__ tab)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < PH_TAB) tab[j] = make_float2((float)tc_tab[4 * j].x, (float)tc_tab[4 * j].y);
}

__device__ __forceinline__ uint64_t mix64(uint64_t z)
{
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Per-atom step factors exp(2 pi i 8 d) and exp(2 pi i 16 d) along the three
// grid axes: FP64 values (table and Taylor series; the square of the first
// for the second), rounded stochastically to FP32 (a draw per atom and
// component).  The producers step a row by these
// factors up to 16 times, so a factor's rounding error recurs in every value
// of the chain; atoms at equivalent positions have identical increments, and
// with round-to-nearest their chains would share one error and add it up
// coherently.  Stochastic rounding gives each atom its own, zero-mean error.
// mask: bit a set for each axis a whose factors are written.
__global__ void k_tc_mult(const uint64_t *__restrict__ du, const uint64_t *__restrict__ dv,
                          const uint64_t *__restrict__ dw, int64_t n, int64_t stride,
                          const double2 *__restrict__ tab, float2 *__restrict__ out, int mask)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint64_t *d[3] = {du, dv, dw};
#pragma unroll
    for (int a = 0; a < 3; a++) {
        if (!((mask >> a) & 1)) continue;
        const double2 m = phasor_f64(d[a][i] << 3, tab);
        const double2 m2 = make_double2(m.x * m.x - m.y * m.y, 2.0 * m.x * m.y);
        const uint64_t r = mix64((uint64_t)i * 4u + (uint64_t)a + 0x9E3779B97F4A7C15ull);
        const uint64_t q = mix64(r);
        out[a * stride + i] = make_float2(round_stochastic(m.x, (uint32_t)r), round_stochastic(m.y, (uint32_t)(r >> 32)));
        out[(3 + a) * stride + i] =
            make_float2(round_stochastic(m2.x, (uint32_t)q), round_stochastic(m2.y, (uint32_t)(q >> 32)));
    }
}

// V operand images: for every (64-atom group gi, column tile nt) the B rows
// [Vr; Vi; -Vr] (hi operand, then lo) of the tile's N columns, in the
// 128-byte-swizzled K-major layout the MMAs read (768 N bytes).  Each value is
// evaluated from its exact 64-bit phase; grid: one block per (gi, nt).  A
// half-warp takes the 16 atom quads of one column, i.e. one 128-byte row of
// each of the six row blocks, so every 8-byte store instruction of a warp
// fills two whole rows and goes straight to global memory (no staging in
// shared memory, no block barrier: the warps' evaluation and stores overlap).
template <bool BF>
__global__ void __launch_bounds__(256) k_tc_vgen(const uint64_t *__restrict__ dac, int N, int n_tiles,
                                                  uint8_t *__restrict__ vimg)
{
    constexpr int NQ = TC_KB / 4;      // atom quads per row
    const int64_t gi = blockIdx.x / n_tiles;
    const int nt = (int)(blockIdx.x % n_tiles);
    const uint32_t vbytes = (uint32_t)N * 768u;
    uint8_t *img = vimg + (int64_t)blockIdx.x * vbytes;
    const uint32_t half = vbytes / 2, blk = (uint32_t)(N >> 3) * TC_SBO128;
    for (int u = threadIdx.x; u < N * NQ; u += blockDim.x) {
        const int c = u / NQ, jq = u % NQ;                     // column, atom quad
        const uint32_t nc = (uint32_t)(nt * N + c);
        float2 x[4];
#pragma unroll
        for (int a = 0; a < 4; a++) {
            const int64_t j = gi * TC_KB + 4 * jq + a;
            const float2 p = phasor_acc((uint64_t)nc * dac[j] - tc_rot((uint64_t)j));
            x[a] = make_float2(p.x * TC_V_SCALE, p.y * TC_V_SCALE);
        }
        uint2 rh, rl, ih, il;
        split4<BF>(x[0].x, x[1].x, x[2].x, x[3].x, rh, rl);
        split4<BF>(x[0].y, x[1].y, x[2].y, x[3].y, ih, il);
        uint8_t *d = img + sw128_off(c, jq >> 1) + (jq & 1) * 8;
        *reinterpret_cast<uint2 *>(d) = rh;
        *reinterpret_cast<uint2 *>(d + half) = rl;
        *reinterpret_cast<uint2 *>(d + blk) = ih;
        *reinterpret_cast<uint2 *>(d + blk + half) = il;
        *reinterpret_cast<uint2 *>(d + 2 * blk) = make_uint2(rh.x ^ 0x80008000u, rh.y ^ 0x80008000u);
        *reinterpret_cast<uint2 *>(d + 2 * blk + half) = make_uint2(rl.x ^ 0x80008000u, rl.y ^ 0x80008000u);
    }
}

// ---------------------------------------------------------------------------
int dgpu_tc_init(dgpu_ctx *ctx)
{
    DGPU_CUDA(ctx, ctx->tc_tab.ensure(4096 * sizeof(double2)));
    k_tc_tab<<<16, 256, 0, ctx->stream>>>(ctx->tc_tab.as<double2>());
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, ctx->ph_tab.ensure(PH_TAB * sizeof(float2)));
    k_ph_tab<<<PH_TAB / 256, 256, 0, ctx->stream>>>(ctx->tc_tab.as<double2>(), ctx->ph_tab.as<float2>());
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}

bool dgpu_tc_available(dgpu_ctx *ctx)
{
    if (ctx->tc_avail < 0) {
        cudaDeviceProp p;
        ctx->tc_avail = (cudaGetDeviceProperties(&p, ctx->device) == cudaSuccess && p.major == 10) ? 1 : 0;
    }
    return ctx->tc_avail == 1;
}

static uint32_t pow2_cols(int n)
{
    uint32_t c = 32;
    while (c < (uint32_t)n) c <<= 1;
    return c;
}

// row axes for a column axis: ra is the longer of the other two
static void tc_row_axes(const BoxSpec &box, int ac, int &ra, int &rb)
{
    const int a = ac == 0 ? 1 : 0, b = 3 - ac - a;
    if (box.f[b] > box.f[a]) { ra = b; rb = a; }
    else { ra = a; rb = b; }
}

// padded MMA area of a column axis / tile width
static double tc_area(const BoxSpec &box, int ac, int N)
{
    const int64_t npts = (int64_t)box.f[0] * box.f[1] * box.f[2];
    const int nc = box.f[ac];
    if (nc < 2 && npts != nc) return -1.0;
    int ra, rb;
    tc_row_axes(box, ac, ra, rb);
    const int64_t rows = (int64_t)dgpu_cdiv(box.f[ra], 8) * 8 * box.f[rb];
    return (double)dgpu_cdiv(nc, N) * N * dgpu_cdiv(rows, TC_M) * TC_M;
}

// Geometry of one problem for a column axis, tile width and slicing.
// slice_atoms > 0: K slices of about that many atoms (a multi-problem launch,
// where the items of all problems share the SMs), else about slice_mult
// work items per SM for this problem alone
static void tc_problem(dgpu_ctx *ctx, const TcInput &in, const dgpu_opts *op, int axis, int N, int slice_mult,
                       int64_t slice_atoms, TcProblem &g)
{
    memset(&g, 0, sizeof(g));
    const BoxSpec &box = in.box;
    for (int k = 0; k < 3; k++) g.f[k] = box.f[k];
    g.ac = axis;
    tc_row_axes(box, axis, g.ra, g.rb);
    g.ncols = box.f[axis];
    g.fra = box.f[g.ra];
    g.fra_p = (int32_t)dgpu_cdiv(g.fra, 8) * 8;
    g.frb = box.f[g.rb];
    g.nrows_p = (int64_t)g.fra_p * g.frb;
    g.N = N;
    g.n_tiles = (int32_t)dgpu_cdiv(g.ncols, N);
    g.vstride = g.n_tiles;
    g.m_tiles = (int32_t)dgpu_cdiv(g.nrows_p, TC_M);
    g.slab = g.nrows_p * g.ncols;
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
    } else if (slice_atoms > 0) {
        nsl = dgpu_cdiv(maxn, slice_atoms);
    } else {
        nsl = dgpu_cdiv((int64_t)slice_mult * ctx->nsm, tiles);
        if (nsl > 1 && dgpu_cdiv(maxn, nsl) < 2048) nsl = dgpu_cdiv(maxn, 2048);
    }
    if (nsl < 1) nsl = 1;
    g.slice_len = dgpu_cdiv(dgpu_cdiv(maxn > 0 ? maxn : 1, nsl), TC_KB) * TC_KB;   // whole stages of either path
    g.nslice = (int32_t)dgpu_cdiv(maxn > 0 ? maxn : 1, g.slice_len);
    g.nitems = tiles * g.nslice;
    const uint64_t *dd[3] = {in.du, in.dv, in.dw};
    g.ph0 = in.ph0;
    g.dra = dd[g.ra];
    g.drb = dd[g.rb];
    g.dac = dd[axis];
    g.w = in.w;
    g.ma = in.mult + (int64_t)g.ra * in.mult_stride;
    g.mc = in.mult + (int64_t)axis * in.mult_stride;
    g.ma2 = in.mult + (int64_t)(3 + g.ra) * in.mult_stride;
    g.mc2 = in.mult + (int64_t)(3 + axis) * in.mult_stride;
}

void dgpu_tc_partref(const TcProblem &g, const float2 *p, PartRef &ref)
{
    ref.p = p;
    ref.nslice = g.nslice;
    ref.f32 = 1;
    ref.s[g.ra] = 1;
    ref.s[g.rb] = g.fra_p;
    ref.s[g.ac] = g.nrows_p;
    ref.slab = g.slab;
}

#define TC_VIMG_BUDGET ((int64_t)16 << 30)    // bytes of V images per launch

int dgpu_tc_plan(dgpu_ctx *ctx, int nprob, const TcInput *in, const dgpu_opts *op, int N, int slice_mult,
                 TcPlan &plan, DevBuf &part, DevBuf &desc, DevBuf *vimg)
{
    plan.probs.assign(nprob, TcProblem());
    plan.part_off.assign(nprob, 0);
    plan.nslice.assign(nprob, 0);
    int64_t items = 0, elems = 0;
    std::vector<int> axes(nprob);
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
        axes[p] = axis;
    }
    // several problems share the SMs: one slice length for all, from their
    // total work (tiles x atoms), so that the whole launch has about
    // slice_mult items per SM of about equal size (at least 2048 atoms)
    int64_t slice_atoms = 0;
    if (nprob > 1 && op->tc_kslice <= 0) {
        double work = 0.0;
        for (int p = 0; p < nprob; p++) {
            TcProblem g;
            tc_problem(ctx, in[p], op, axes[p], N, slice_mult, 0, g);
            work += (double)(g.nitems / g.nslice) * (double)(g.nslice * g.slice_len);
        }
        slice_atoms = (int64_t)ceil(work / ((double)slice_mult * ctx->nsm));
        if (slice_atoms < 2048) slice_atoms = 2048;
    }
    for (int p = 0; p < nprob; p++) {
        TcProblem &g = plan.probs[p];
        tc_problem(ctx, in[p], op, axes[p], N, slice_mult, slice_atoms, g);
        g.item0 = items;
        items += g.nitems;
        plan.part_off[p] = elems;
        plan.nslice[p] = g.nslice;
        elems += (int64_t)g.ntype * g.nslice * g.slab;
    }
    plan.item_prob.resize(items);
    for (int p = 0; p < nprob; p++)
        for (int64_t i = 0; i < plan.probs[p].nitems; i++) plan.item_prob[plan.probs[p].item0 + i] = p;
    DGPU_CUDA(ctx, part.ensure((size_t)(elems > 0 ? elems : 1) * sizeof(float2)));
    for (int p = 0; p < nprob; p++) plan.probs[p].part = part.as<float2>() + plan.part_off[p];
    // V images: one per (64-atom group, column tile) of every problem.  The
    // images depend only on the atoms' column steps and the column index, so
    // problems over the same atoms with the same column axis (boxes of one
    // grid at different origins) share one set, as wide as the widest.
    bool share = nprob > 1;
    int32_t wide = 0;
    for (int p = 0; p < nprob; p++) {
        const TcProblem &g = plan.probs[p];
        share = share && g.dac == plan.probs[0].dac && in[p].ts == in[0].ts && in[p].ntype == in[0].ntype;
        wide = g.n_tiles > wide ? g.n_tiles : wide;
    }
    std::vector<int64_t> voff(nprob, 0);
    int64_t vtot = 0;
    for (int p = 0; p < nprob; p++) {
        voff[p] = share ? 0 : vtot;
        if (!share || p == 0)
            vtot += in[p].ts[in[p].ntype] / TC_KB * (share ? wide : plan.probs[p].n_tiles) * (int64_t)N * 768;
    }
    // images pay when every one is re-read by several row tiles (a 3D grid);
    // thin planes with one or two row tiles generate V in the kernel
    double reads = 0.0, imgs = 0.0;
    for (int p = 0; p < nprob; p++) {
        const double ni = (double)(in[p].ts[in[p].ntype] / TC_KB) * plan.probs[p].n_tiles;
        if (!share || p == 0) imgs += share ? (double)(in[p].ts[in[p].ntype] / TC_KB) * wide : ni;
        reads += ni * plan.probs[p].m_tiles;
    }
    const bool reuse = imgs > 0 && reads >= 4.0 * imgs;
    plan.vimg = vimg && vtot > 0 && vtot <= TC_VIMG_BUDGET && op->tc_vimg >= 0 && (reuse || op->tc_vimg > 0);
    plan.vshared = share;
    if (plan.vimg) {
        DGPU_CUDA(ctx, vimg->ensure((size_t)vtot));
        for (int p = 0; p < nprob; p++) {
            plan.probs[p].vimg = vimg->as<uint8_t>() + voff[p];
            if (share) plan.probs[p].vstride = wide;
        }
    }
    const size_t pbytes = ((size_t)nprob * sizeof(TcProblem) + 255) & ~(size_t)255;
    DGPU_CUDA(ctx, desc.ensure(pbytes + (size_t)items * sizeof(int32_t) + 256));
    if (ctx->tc_defer) {
        // one copy from pinned memory that stays valid until the run's host wait
        char *h = static_cast<char *>(ctx->stage.take(pbytes + (size_t)items * sizeof(int32_t)));
        if (!h) return dgpu_set_error(ctx, DGPU_ERR_NOMEM, "pinned staging memory");
        memcpy(h, plan.probs.data(), (size_t)nprob * sizeof(TcProblem));
        memcpy(h + pbytes, plan.item_prob.data(), (size_t)items * sizeof(int32_t));
        DGPU_CUDA(ctx, cudaMemcpyAsync(desc.p, h, pbytes + (size_t)items * sizeof(int32_t), cudaMemcpyHostToDevice,
                                       ctx->stream));
    } else {
        DGPU_CUDA(ctx, cudaMemcpyAsync(desc.p, plan.probs.data(), (size_t)nprob * sizeof(TcProblem),
                                       cudaMemcpyHostToDevice, ctx->stream));
        DGPU_CUDA(ctx, cudaMemcpyAsync((char *)desc.p + pbytes, plan.item_prob.data(),
                                       (size_t)items * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
        // the host vectors must outlive the copies
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    }
    TcLaunch &L = plan.L;
    L.probs = (const TcProblem *)desc.p;
    L.item_prob = (const int32_t *)((char *)desc.p + pbytes);
    L.nitems = items;
    L.Nmax = N;
    // TMEM: correction (2N) + main x nbuf (2N each) [+ running sum (2N)]
    L.nbuf = 2 * N * 3 <= 512 ? 2 : 1;
    L.tsum = 2 * N * (2 + L.nbuf) <= 512 ? 1 : 0;
    L.bf16 = op->split == DGPU_SPLIT_BF16;
    // V images stream through a ring of 64-atom slots when it leaves room for
    // two U stages; the producers of that path hold their atoms' phase data in
    // registers, so it needs no atom slots and may use the whole shared
    // memory of the SM
    const uint32_t vbytes_img = 2u * 3u * N * TC_KB * 2;
    const int64_t room = (int64_t)TC_SMEM_MAX - TC_BAR_BYTES - (int64_t)TC_VSLOTS * vbytes_img;
    if (plan.vimg && room < 2 * 4 * TC_B_BYTES) plan.vimg = false;
    if (!plan.vimg)
        for (TcProblem &g : plan.probs) g.vimg = nullptr;
    L.vring = plan.vimg ? 1 : 0;
    const int ks_atoms = L.vring ? TC_KB : TC_KA;                 // atoms per stage
    L.flush = op->tc_flush > 0 ? (int32_t)dgpu_cdiv(op->tc_flush, ks_atoms)
                               : TC_FLUSH_STAGES * TC_KA / ks_atoms;   // 128 atoms
    const uint32_t vbytes = 2u * 3u * N * ks_atoms * 2;
    const uint32_t bar_bytes = TC_BAR_BYTES + (L.vring ? 0u : (uint32_t)(TC_NSLOT * TC_ATOM_SLOT));
    const int64_t budget = L.vring ? TC_SMEM_MAX : TC_SMEM_BUDGET;
    const uint32_t stage_bytes = 4u * TC_M * ks_atoms * 2 + (L.vring ? 0u : vbytes);
    const int stages = (int)((budget - bar_bytes - (L.vring ? (int64_t)TC_VSLOTS * vbytes : 0)) / stage_bytes);
    L.stages = stages > 4 ? 4 : stages;
    L.tmem_cols = pow2_cols(2 * N * (1 + L.nbuf + L.tsum));
    if (L.stages < 2 || L.tmem_cols > 512) return dgpu_set_error(ctx, DGPU_ERR_ARG, "tile does not fit");
    plan.smem = (size_t)L.stages * stage_bytes + (L.vring ? (size_t)TC_VSLOTS * vbytes : 0) + bar_bytes;
    if (!ctx->tc_attr) {              // once per context (and device), outside any stream capture
        DGPU_CUDA(ctx, cudaFuncSetAttribute(k_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        DGPU_CUDA(ctx, cudaFuncSetAttribute(k_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024));
        ctx->tc_attr = true;
    }
    DGPU_CUDA(ctx, ctx->flag.ensure(64));
    L.err = ctx->flag.as<int32_t>() + 8;
    L.timeout_ns = op->tc_wait_us > 0 ? (uint64_t)op->tc_wait_us * 1000ull : TC_TIMEOUT_NS;
    return DGPU_OK;
}

int dgpu_tc_launch(dgpu_ctx *ctx, const TcPlan &plan, bool timed)
{
    if (!ctx->tc_defer) DGPU_CUDA(ctx, cudaMemsetAsync(plan.L.err, 0, sizeof(int32_t), ctx->stream));
    if (plan.L.nitems < 1) return DGPU_OK;
    if (plan.vimg)
        for (const TcProblem &g : plan.probs) {
            const int64_t nimg = (g.ts[g.ntype] / TC_KB) * g.vstride;
            if (nimg < 1) continue;
            if (plan.L.bf16)
                k_tc_vgen<true><<<(unsigned)nimg, 256, 0, ctx->stream>>>(g.dac, g.N, g.vstride, g.vimg);
            else
                k_tc_vgen<false><<<(unsigned)nimg, 256, 0, ctx->stream>>>(g.dac, g.N, g.vstride, g.vimg);
            if (plan.vshared) break;                        // one set for all problems
        }
    const int grid = (int)(plan.L.nitems < ctx->nsm ? plan.L.nitems : ctx->nsm);
    if (timed) DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[6], ctx->stream));
    if (plan.L.bf16)
        k_tc<true><<<grid, TC_THREADS, plan.smem, ctx->stream>>>(plan.L);
    else
        k_tc<false><<<grid, TC_THREADS, plan.smem, ctx->stream>>>(plan.L);
    DGPU_CUDA(ctx, cudaGetLastError());
    if (timed) DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[7], ctx->stream));
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

int dgpu_tc_mult_async(dgpu_ctx *ctx, const uint64_t *du, const uint64_t *dv, const uint64_t *dw, int64_t n,
                       int64_t stride, float2 *out, int mask)
{
    if (n < 1 || !(mask & 7)) return DGPU_OK;
    k_tc_mult<<<(unsigned)dgpu_cdiv(n, 256), 256, 0, ctx->stream>>>(du, dv, dw, n, stride,
                                                                      ctx->tc_tab.as<double2>(), out, mask & 7);
    DGPU_CUDA(ctx, cudaGetLastError());
    return DGPU_OK;
}

// Candidate configurations: every column axis and tile width whose padded
// MMA area is within 25% of the smallest, at two slicings.
static void tc_candidates(const BoxSpec &box, int want_n, int kslice, TcChoice *out, int &n)
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
                if (kslice > 0 && m != 4) continue;     // the slicing is given: one candidate per tile
                out[n].axis = a;
                out[n].N = N;
                out[n].slice_mult = m;
                n++;
            }
        }
}

extern "C" double dgpu_tc_last_kernel_ms(const dgpu_ctx *ctx) { return ctx ? ctx->tc_kernel_ms : 0.0; }

int dgpu_tc_sums(dgpu_ctx *ctx, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw,
                 const float *w, const int64_t *h_type_start, int32_t ntype, const BoxSpec &box,
                 const dgpu_opts *op, DevBuf &part, PartRef *ref)
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
    const int64_t npad = h_type_start[ntype];
    DGPU_CUDA(ctx, ctx->tc_mult.ensure((size_t)TC_MULT_ARRAYS * (npad > 0 ? npad : 1) * sizeof(float2)));
    int rc;
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
    in.mult = ctx->tc_mult.as<float2>();
    in.mult_stride = npad;
    in.ts = h_type_start;
    in.ntype = ntype;
    in.box = box;
    TcChoice choice;
    auto hit = ctx->tc_tuned.find(key);
    const bool cached = hit != ctx->tc_tuned.end();
    if (cached) {
        choice = hit->second;
    } else {
        // the candidates use every axis as row or column axis: all step factors
        rc = dgpu_tc_mult_async(ctx, du, dv, dw, npad, npad, ctx->tc_mult.as<float2>(), 7);
        if (rc) return rc;
        TcChoice cand[64];
        int nc = 0;
        tc_candidates(box, want_n, op->tc_kslice, cand, nc);
        if (nc == 0) return dgpu_set_error(ctx, DGPU_ERR_ARG, "no tensor-core tile fits the box");
        float best = 1e30f;
        choice = cand[0];
        for (int c = 0; c < nc && nc > 1; c++) {
            in.axis = cand[c].axis;
            TcPlan plan;
            if (dgpu_tc_plan(ctx, 1, &in, op, cand[c].N, cand[c].slice_mult, plan, part, ctx->tc_part,
                             &ctx->tc_vimg))
                continue;
            DGPU_CUDA(ctx, cudaEventRecord(ctx->ev[4], ctx->stream));
            rc = dgpu_tc_launch(ctx, plan);
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
    rc = dgpu_tc_plan(ctx, 1, &in, op, choice.N, choice.slice_mult, plan, part, ctx->tc_part, &ctx->tc_vimg);
    if (rc) return rc;
    if (cached) {
        // the factors this plan reads: the row axis ra (the producers' steps),
        // on the in-kernel V path also the column axis
        const TcProblem &g = plan.probs[0];
        rc = dgpu_tc_mult_async(ctx, du, dv, dw, npad, npad, ctx->tc_mult.as<float2>(),
                                (1 << g.ra) | (plan.vimg ? 0 : 1 << g.ac));
        if (rc) return rc;
    }
    rc = dgpu_tc_launch(ctx, plan, !ctx->tc_defer);
    if (rc) return rc;
    if (!ctx->tc_defer) {
        rc = dgpu_tc_check(ctx);
        if (rc) return rc;
        float ms = 0.f;
        DGPU_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[6], ctx->ev[7]));
        ctx->tc_kernel_ms = ms;
    }
    ctx->tc_last[0] = plan.probs[0].ac;
    ctx->tc_last[1] = plan.probs[0].N;
    ctx->tc_last[2] = plan.L.nbuf;
    ctx->tc_last[3] = (int32_t)plan.probs[0].slice_len;
    dgpu_tc_partref(plan.probs[0], part.as<float2>(), *ref);
    return DGPU_OK;
}
