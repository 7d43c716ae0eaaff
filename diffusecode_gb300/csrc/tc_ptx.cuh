// tcgen05 / TMA / mbarrier building blocks shared by the tensor-core kernels
// (sm_100 family): shared-memory descriptors of the 64-byte-swizzled K-major
// operand layout, MMA issue and commit, TMEM loads and stores, bounded
// mbarrier waits, bulk copies, and the fp16/bf16 hi/lo operand split.
#pragma once
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

// K-major operand rows of 64 bytes (32 16-bit values); 8-row groups of 512 B
#define TC_SBO 512
#define TC_TIMEOUT_NS 2000000000ull            // 2 s per wait

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

// try_wait that may suspend the thread until the phase completes, at most
// TC_SUSPEND_NS: a waiting warp takes no issue slots from the producers
#define TC_SUSPEND_NS 20000
__device__ __forceinline__ bool mbar_try_suspend(uint64_t *bar, uint32_t parity)
{
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "n"(TC_SUSPEND_NS)
        : "memory");
    return ok != 0;
}

// bounded wait for another warp's progress: false if the error flag is up or
// the wait ran longer than limit_ns (recorded as `code` in the flag)
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int32_t *err, int code,
                                          uint64_t limit_ns = TC_TIMEOUT_NS)
{
    if (mbar_try(bar, parity)) return true;
    const uint64_t t0 = gtimer();
    for (;;) {
        if (mbar_try_suspend(bar, parity)) return true;
        if (*err) return false;
        if (gtimer() - t0 > limit_ns) {
            atomicCAS((int32_t *)err, 0, code);
            return false;
        }
    }
}

// arrive on a barrier and announce tx bytes that an async copy will complete
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *bar, uint32_t bytes)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(
                     smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// one bulk global -> shared copy (16-byte aligned, size a multiple of 16)
// completing `bytes` of transaction on bar
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar)
{
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// wait that ignores the error flag (time-bounded, always the full
// TC_TIMEOUT_NS): used to let the CTA's own MMAs and bulk copies complete
// before it frees TMEM and exits after an error
__device__ __forceinline__ void mbar_wait_quiet(uint64_t *bar, uint32_t parity)
{
    const uint64_t t0 = gtimer();
    while (!mbar_try_suspend(bar, parity))
        if (gtimer() - t0 > TC_TIMEOUT_NS) return;
}

__device__ __forceinline__ void cp_async16(void *dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait1() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait0() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// K-major operand with the 64-byte swizzle: row r of an 8-row group at
// (r&7)*64 B, its 16-byte chunk c stored at chunk c ^ ((r&7)>>1); 8-row groups
// SBO = 512 B apart (each group 512-byte aligned).
// four 8x8 b16 matrices from registers to shared memory: lane l gives the
// address of row (l & 7) of matrix (l >> 3); register i of lane l holds
// row l >> 2, columns 2 (l & 3) and 2 (l & 3) + 1 of matrix i (low half first)
__device__ __forceinline__ void stmatrix_x4(uint32_t addr, uint32_t r0, uint32_t r1, uint32_t r2, uint32_t r3)
{
    asm volatile("stmatrix.sync.aligned.m8n8.x4.shared.b16 [%0], {%1, %2, %3, %4};" ::"r"(addr), "r"(r0), "r"(r1),
                 "r"(r2), "r"(r3)
                 : "memory");
}

__device__ __forceinline__ uint32_t sw_off(int r, int chunk)
{
    return (uint32_t)((r >> 3) * TC_SBO + (r & 7) * 64 + ((chunk ^ ((r & 7) >> 1)) << 4));
}

// K-major operand with the 128-byte swizzle: rows of 128 bytes (64 16-bit
// values), 8-row groups of 1024 B, the 16-byte chunk c of row r stored at
// chunk c ^ (r & 7).  The buffer must start on a 1024-byte boundary.
#define TC_SBO128 1024
__device__ __forceinline__ uint32_t sw128_off(int r, int chunk)
{
    return (uint32_t)((r >> 3) * TC_SBO128 + (r & 7) * 128 + ((chunk ^ (r & 7)) << 4));
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                      // leading byte offset: unused for swizzled K-major
    d |= (uint64_t)((TC_SBO >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;                      // descriptor version of the sm_100 family
    d |= (uint64_t)4 << 61;                      // 64-byte swizzle
    return d;
}

// descriptor of the 128-byte-swizzled K-major layout (layout type 2)
__device__ __forceinline__ uint64_t sdesc128(uint32_t saddr)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;                      // leading byte offset: unused for swizzled K-major
    d |= (uint64_t)((TC_SBO128 >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;                      // descriptor version of the sm_100 family
    d |= (uint64_t)2 << 61;                      // 128-byte swizzle
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

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16])
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], "
        "{%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(taddr),
        "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]), "r"(r[8]),
        "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// ---------------------------------------------------------------------------
// operand generation

// exp(2 pi i phase) from the top 32 bits of a 64-bit fixed-point turn (MUFU)
__device__ __forceinline__ float2 phasor_fast(uint64_t ph)
{
    float s, c;
    __sincosf((float)(int32_t)(ph >> 32) * 1.4629180792671596e-09f, &s, &c);   // 2 pi / 2^32
    return make_float2(c, s);
}

// A per-atom phase offset (a Weyl sequence over the atom's slot index, in
// 2^-64 turns).  The tensor-core engine evaluates U at phase + rot and V at
// phase - rot, so that their product is unchanged while the rounding and
// approximation errors of the evaluated values differ from atom to atom:
// atoms at equivalent positions (a perfect lattice, one layer) would
// otherwise carry identical errors, which add up coherently in their sum.
__device__ __forceinline__ uint64_t tc_rot(uint64_t j) { return j * 0x9E3779B97F4A7C15ull; }

// exp(2 pi i phase) of a 64-bit fixed-point turn to about one FP32 ulp: the
// signed phase as x = 2 turns in [-1, 1) splits into its top 23 bits (exact
// in FP32, evaluated by sincospif) and a remainder below 2^-22 (its next 23
// bits) applied as a first-order rotation; both integers become floats by the
// exponent-bias construction (an integer add and one FP32 subtract), not by a
// conversion instruction.  Used where a value is evaluated once per launch
// (the V operand images); the kernels' seeds use the hardware approximation
// above, whose error (a few 1e-7, a smooth function of the phase) tc_rot makes
// random from atom to atom.
__device__ __forceinline__ float2 phasor_acc(uint64_t ph)
{
    const int32_t hi = (int32_t)((int64_t)ph >> 41);                  // in [-2^22, 2^22)
    const uint32_t lo = (uint32_t)(ph >> 18) & 0x7FFFFFu;               // in [0, 2^23)
    const float xf = (__int_as_float(0x4B400000 + hi) - 12582912.0f) * 0x1p-22f;
    const float dth = (__uint_as_float(0x4B000000u | lo) - 8388608.0f) * (3.14159265358979f * 0x1p-45f);
    float s, c;
    sincospif(xf, &s, &c);
    return make_float2(fmaf(-s, dth, c), fmaf(c, dth, s));
}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

template <bool BF>
__device__ __forceinline__ uint32_t pack2(float a, float b)
{
    if (BF) {
        __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
        return *reinterpret_cast<uint32_t *>(&v);
    }
    __half2 v = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t *>(&v);
}

// 4 values (4 consecutive atoms of one row) -> hi and lo, 4 x 16 bit each.
// hi keeps the leading 11 (fp16) or 8 (bf16) significant bits of the FP32
// value, so it is exact in the operand format (fp16 subnormals aside, which
// only occur below 2^-14 where the absolute error stays below 2^-25); lo is
// the exact FP32 remainder, rounded to the operand format.
template <bool BF>
__device__ __forceinline__ void split4(float x0, float x1, float x2, float x3, uint2 &hi, uint2 &lo)
{
    const uint32_t mask = BF ? 0xFFFF0000u : 0xFFFFE000u;
    const float h0 = __uint_as_float(__float_as_uint(x0) & mask);
    const float h1 = __uint_as_float(__float_as_uint(x1) & mask);
    const float h2 = __uint_as_float(__float_as_uint(x2) & mask);
    const float h3 = __uint_as_float(__float_as_uint(x3) & mask);
    hi.x = pack2<BF>(h0, h1);
    hi.y = pack2<BF>(h2, h3);
    lo.x = pack2<BF>(x0 - h0, x1 - h1);
    lo.y = pack2<BF>(x2 - h2, x3 - h3);
}

