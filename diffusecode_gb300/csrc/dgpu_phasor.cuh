// Phasors of exact 64-bit phases on CUDA cores by table-driven angle
// addition (Tang's table-driven method for elementary functions): a phase
// ph (2^64 = one turn) plus PH_ROUND splits into
//   * its top 10 bits, the nearest of PH_TAB table angles 2 pi j / 1024,
//     whose exp(i angle) the table holds (FP64 sincospi rounded to FP32);
//   * the next 23 bits less 2^22, the remainder d in units of PH_KAPPA
//     (|d| <= pi / 1024 rad, resolution 2 pi 2^-33, rounded to nearest),
// and exp(i d) = 1 - d^2/2 + i d (1 - d^2/6) to within 4e-12.
#pragma once
#include <stdint.h>

#define PH_TAB 1024                                      // table angles 2 pi j / PH_TAB
#define PH_ROUND ((1ull << 53) + (1ull << 30))           // table index and remainder rounded to nearest
#define PH_KAPPA (3.14159265358979f * 0x1p-32f)          // radians per unit of the remainder, 2 pi / 2^33
#define PH_S6 (-(PH_KAPPA * PH_KAPPA) / 6.0f)

// The weights of one atom: w, w PH_KAPPA and -w PH_KAPPA^2 / 2
struct PhWeight {
    float w, wk, wc;
};

__device__ __forceinline__ PhWeight ph_weight(float w)
{
    return {w, w * PH_KAPPA, w * (-0.5f * PH_KAPPA * PH_KAPPA)};
}

// w exp(2 pi i ph / 2^64) for a phase that already carries PH_ROUND; tab is
// the PH_TAB-entry table (shared memory).  w T is formed exactly inside the
// last FMA, so the weighted phasor is rounded once (plus the table's own
// rounding).
__device__ __forceinline__ float2 ph_phasor(uint64_t ph, const float2 *__restrict__ tab, PhWeight a)
{
    const float2 T = tab[(uint32_t)(ph >> 54)];
    const float d = __uint_as_float(((uint32_t)(ph >> 31) & 0x7FFFFFu) | 0x4B000000u) - 12582912.0f;
    const float d2 = d * d;
    const float v = (a.wk * d) * fmaf(d2, PH_S6, 1.0f);      // w sin(d)
    const float u = d2 * a.wc;                                // w (cos(d) - 1)
    return make_float2(fmaf(T.x, a.w, fmaf(T.x, u, -T.y * v)), fmaf(T.y, a.w, fmaf(T.y, u, T.x * v)));
}
