// Plain FP32 direct sum on CUDA cores.
//
// Replaces the hot loop of four_strucf_omp (discus/prog/four_strucf_OMP_mod.f90:155-182):
// for every grid point of the computed box and every atom of a type,
// phase = ph0 + n0*d0 + n1*d1 + n2*d2 (64-bit fixed point, exact mod 1),
// then w exp(2 pi i phase) in FP32 by table-driven angle addition
// (dgpu_phasor.cuh, the table in shared memory) accumulated in FP32 over one
// shared-memory chunk of atoms and in FP64 across chunks.  Each thread owns
// Q consecutive points along one grid axis, so consecutive points differ by
// one 64-bit add.  In REF22 mode the phase keeps only its top 16 bits, the
// reference's (iarg >> 6) & 0xFFFF table index.
//
// Work split: blockIdx.x = point tile, blockIdx.y = atom slice, blockIdx.z =
// atom type.  Each (type, slice) writes its own partial sum part[t][s][p];
// the combine kernel adds the slices in a fixed order (deterministic).
#include "dgpu_internal.h"
#include "dgpu_phasor.cuh"

#define DIR_NT 128
#define DIR_Q 8

struct DirectGeom {
    int32_t f[3];          // box
    int32_t a0, a1, a2;    // axis permutation, a0 = per-thread run axis
    int32_t nq;            // ceil(f[a0]/Q)
    int64_t nslots;        // nq * f[a1] * f[a2]
    int64_t pbox;          // f0*f1*f2
    int32_t nslice;
    int64_t slice_len;
    int64_t ts[65];        // type_start (0-based types)
};

template <bool REF>
__global__ void __launch_bounds__(DIR_NT)
k_direct(const uint64_t *__restrict__ ph0, const uint64_t *__restrict__ du,
         const uint64_t *__restrict__ dv, const uint64_t *__restrict__ dw,
         const float *__restrict__ w, const float2 *__restrict__ gtab, const DirectGeom g,
         double2 *__restrict__ part)
{
    __shared__ uint64_t s_b[DIR_NT], s_d0[DIR_NT], s_d1[DIR_NT], s_d2[DIR_NT];
    __shared__ float s_w[DIR_NT];
    __shared__ float2 tab[PH_TAB];
    for (int j = threadIdx.x; j < PH_TAB; j += DIR_NT) tab[j] = gtab[j];

    const int t = blockIdx.z, s = blockIdx.y;
    const int64_t a_lo = g.ts[t] + (int64_t)s * g.slice_len;
    const int64_t a_hi = min(g.ts[t + 1], a_lo + g.slice_len);

    const int64_t slot = (int64_t)blockIdx.x * DIR_NT + threadIdx.x;
    const bool valid = slot < g.nslots;
    int32_t n[3] = {0, 0, 0};
    {
        int64_t sl = valid ? slot : 0;
        int32_t iq = (int32_t)(sl % g.nq);
        int64_t rest = sl / g.nq;
        n[g.a0] = iq * DIR_Q;
        n[g.a1] = (int32_t)(rest % g.f[g.a1]);
        n[g.a2] = (int32_t)(rest / g.f[g.a1]);
    }
    const uint32_t m0 = (uint32_t)n[g.a0], m1 = (uint32_t)n[g.a1], m2 = (uint32_t)n[g.a2];

    double accd[DIR_Q][2];
#pragma unroll
    for (int k = 0; k < DIR_Q; k++) accd[k][0] = accd[k][1] = 0.0;

    for (int64_t base = a_lo; base < a_hi; base += DIR_NT) {
        const int cnt = (int)min((int64_t)DIR_NT, a_hi - base);
        __syncthreads();
        if (threadIdx.x < cnt) {
            int64_t a = base + threadIdx.x;
            uint64_t d[3] = {du[a], dv[a], dw[a]};
            s_b[threadIdx.x] = REF ? ph0[a] : ph0[a] + PH_ROUND;
            s_d0[threadIdx.x] = d[g.a0];
            s_d1[threadIdx.x] = d[g.a1];
            s_d2[threadIdx.x] = d[g.a2];
            s_w[threadIdx.x] = w[a];
        }
        __syncthreads();
        // FP32 sums over the chunk with Fast2Sum compensation: a coherent sum
        // of nearly equal terms would otherwise round with a bias that grows
        // with the chunk length (~ n 2^-24 of the sum)
        float accf[DIR_Q][2], cmpf[DIR_Q][2];
#pragma unroll
        for (int k = 0; k < DIR_Q; k++) accf[k][0] = accf[k][1] = cmpf[k][0] = cmpf[k][1] = 0.f;
        for (int j = 0; j < cnt; j++) {
            const uint64_t d0 = s_d0[j];
            uint64_t ph = s_b[j] + m0 * d0 + m1 * s_d1[j] + m2 * s_d2[j];
            const PhWeight wj = ph_weight(s_w[j]);
#pragma unroll
            for (int k = 0; k < DIR_Q; k++) {
                // REF22: the top 16 bits, the reference's table index, then rounded as any phase
                const uint64_t q = REF ? (ph & 0xFFFF000000000000ull) + PH_ROUND : ph;
                const float2 e = ph_phasor(q, tab, wj);
                const float y0 = e.x, y1 = e.y;
                const float t0 = accf[k][0] + y0, t1 = accf[k][1] + y1;
                cmpf[k][0] += y0 - (t0 - accf[k][0]);
                cmpf[k][1] += y1 - (t1 - accf[k][1]);
                accf[k][0] = t0;
                accf[k][1] = t1;
                ph += d0;
            }
        }
#pragma unroll
        for (int k = 0; k < DIR_Q; k++) {
            accd[k][0] += (double)accf[k][0] + (double)cmpf[k][0];
            accd[k][1] += (double)accf[k][1] + (double)cmpf[k][1];
        }
    }
    if (!valid) return;
    double2 *out = part + ((int64_t)t * g.nslice + s) * g.pbox;
#pragma unroll
    for (int k = 0; k < DIR_Q; k++) {
        int32_t nn[3] = {n[0], n[1], n[2]};
        nn[g.a0] += k;
        if (nn[g.a0] >= g.f[g.a0]) break;
        int64_t p = nn[0] + (int64_t)g.f[0] * (nn[1] + (int64_t)g.f[1] * nn[2]);
        out[p] = make_double2(accd[k][0], accd[k][1]);
    }
}

int dgpu_direct_sums(dgpu_ctx *ctx, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv,
                     const uint64_t *dw, const float *w, const int64_t *h_type_start, int32_t ntype,
                     int32_t ref_mask, const BoxSpec &box, DevBuf &part, int32_t *nslice_out)
{
    if (ntype < 1 || ntype > 64) return dgpu_set_error(ctx, DGPU_ERR_ARG, "ntype=%d", ntype);
    DirectGeom g;
    memset(&g, 0, sizeof(g));
    for (int k = 0; k < 3; k++) g.f[k] = box.f[k];
    // run axis: the longest axis of the box
    int a0 = 0;
    for (int k = 1; k < 3; k++)
        if (box.f[k] > box.f[a0]) a0 = k;
    g.a0 = a0;
    g.a1 = (a0 + 1) % 3;
    g.a2 = (a0 + 2) % 3;
    g.nq = (int32_t)dgpu_cdiv(box.f[a0], DIR_Q);
    g.nslots = (int64_t)g.nq * box.f[g.a1] * box.f[g.a2];
    g.pbox = (int64_t)box.f[0] * box.f[1] * box.f[2];
    int64_t maxn = 0;
    for (int t = 0; t < ntype; t++) {
        g.ts[t] = h_type_start[t];
        maxn = maxn > (h_type_start[t + 1] - h_type_start[t]) ? maxn : (h_type_start[t + 1] - h_type_start[t]);
    }
    g.ts[ntype] = h_type_start[ntype];
    int64_t tiles = dgpu_cdiv(g.nslots, DIR_NT);
    int64_t want = dgpu_cdiv(8LL * ctx->nsm, tiles * ntype);
    int64_t maxs = maxn / 256 > 1 ? maxn / 256 : 1;
    int32_t nslice = (int32_t)(want < 1 ? 1 : (want > maxs ? maxs : want));
    if (nslice > 65535) nslice = 65535;
    g.nslice = nslice;
    g.slice_len = dgpu_cdiv(maxn > 0 ? maxn : 1, nslice);
    DGPU_CUDA(ctx, part.ensure((size_t)ntype * nslice * g.pbox * sizeof(double2)));
    if (tiles > 0x7fffffff) return dgpu_set_error(ctx, DGPU_ERR_ARG, "grid too large");
    dim3 grid((unsigned)tiles, (unsigned)nslice, (unsigned)ntype);
    if (ref_mask)
        k_direct<true><<<grid, DIR_NT, 0, ctx->stream>>>(ph0, du, dv, dw, w, ctx->ph_tab.as<float2>(), g,
                                                         part.as<double2>());
    else
        k_direct<false><<<grid, DIR_NT, 0, ctx->stream>>>(ph0, du, dv, dw, w, ctx->ph_tab.as<float2>(), g,
                                                          part.as<double2>());
    DGPU_CUDA(ctx, cudaGetLastError());
    *nslice_out = nslice;
    return DGPU_OK;
}
