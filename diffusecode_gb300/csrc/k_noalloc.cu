// Allocation-free per-type structure-factor sum.
//
// Some callers of the per-type sum cannot allocate device memory: a reverse
// Monte Carlo loop that re-evaluates the contribution of a few atoms after
// every move (thousands of calls per second, where cudaMalloc/cudaFree would
// synchronise the device each time), code that runs inside a memory budget
// owned by another allocator, or code that enqueues work on a stream it does
// not own.  dgpu_four_strucf_noalloc serves them: the caller passes device
// inputs and outputs and a stream, and the library's working memory is one
// file-scope __device__ array of fixed size that every GPU loading the
// library holds until the process exits.
//
// Limits: at most NOALLOC_MAX_ATOMS atoms and NOALLOC_MAX_POINTS computed
// points (fnum(1)*fnum(2)*fnum(3)) per call; larger requests return
// DGPU_ERR_SCRATCH_SIZE.  All calls share the array, so calls whose work
// overlaps on the GPU (two streams, or two host threads) race; calls queued
// on one stream are ordered and safe.  Every call rewrites the parts of the
// array it reads, so nothing carries over from one call to the next.
//
// Set-up: the device address of the array is looked up once per device
// (cudaGetSymbolAddress, with that device current) on the first call made on
// that device; make that first call before any stream capture begins.  The
// address is kept with the CUDA context it belongs to and looked up again
// when a later call finds a different context current on that device (for
// instance a new primary context after cudaDeviceReset).  The stream must
// belong to the device that is current at the call.
#include <cuda.h>

#include <mutex>

#include "dgpu_internal.h"

#define NOALLOC_MAX_ATOMS 131072
#define NOALLOC_MAX_POINTS 262144
#define NOALLOC_NT 128
#define NOALLOC_Q 8
// per-atom phase data (4 x uint64 + weight) and one complex double per point
#define NOALLOC_ATOM_BYTES ((size_t)NOALLOC_MAX_ATOMS * (4 * 8 + 4))
#define NOALLOC_BYTES (NOALLOC_ATOM_BYTES + (size_t)NOALLOC_MAX_POINTS * 16)

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

namespace {

std::mutex g_mu;
struct Cached {
    CUcontext ctx;
    void *addr;
};
Cached g_addr[256];

// cuCtxGetCurrent of the CUDA driver API, looked up through the runtime
// (the library does not link libcuda itself)
typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
CtxGetCurrentFn ctx_get_current()
{
    static CtxGetCurrentFn fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<CtxGetCurrentFn>(p);
    }
    return fn;
}

// device address of the scratch array for the current device and context
int scratch_address(void **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return DGPU_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_mu);
    const CtxGetCurrentFn get = ctx_get_current();
    if (!get) return DGPU_ERR_CUDA;
    CUcontext cur = nullptr;              // null before the runtime's first use on this thread
    if (get(&cur) != CUDA_SUCCESS) return DGPU_ERR_CUDA;
    if (!cur || !g_addr[dev].addr || g_addr[dev].ctx != cur) {
        void *p = nullptr;
        // the look-up also makes the device's primary context current
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return DGPU_ERR_CUDA;
        if (get(&cur) != CUDA_SUCCESS || !cur) return DGPU_ERR_CUDA;
        g_addr[dev].addr = p;
        g_addr[dev].ctx = cur;
    }
    *out = g_addr[dev].addr;
    return DGPU_OK;
}

struct Geo {
    double u[3], v[3], w[3], off[9];
    int32_t lmn[6];
    int32_t num[3], fnum[3];
};

__device__ __forceinline__ double na_dot(const double *a, double x0, double x1, double x2)
{
    return __dadd_rn(__dadd_rn(__dmul_rn(a[0], x0), __dmul_rn(a[1], x1)), __dmul_rn(a[2], x2));
}

// NINT(2^22 * (x - INT(x))), four_strucf_OMP_mod.f90:143-148
__device__ __forceinline__ int64_t na_inc22(double x)
{
    return (int64_t)llround(__dmul_rn(4194304.0, __dadd_rn(__dsub_rn(x, trunc(x)), 0.0)));
}

// per-atom REF22 phase data in units of 2^-64 turn
__global__ void k_na_phase(const double *__restrict__ xat, int64_t n, Geo g, uint64_t *ph0, uint64_t *du,
                           uint64_t *dv, uint64_t *dw)
{
    int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const double x0 = xat[k], x1 = xat[n + k], x2 = xat[2 * n + k];
    const int64_t iu = na_inc22(na_dot(g.u, x0, x1, x2)), iv = na_inc22(na_dot(g.v, x0, x1, x2));
    const int64_t iw = na_inc22(na_dot(g.w, x0, x1, x2));
    const int64_t ju = na_inc22(na_dot(g.off + 0, x0, x1, x2)), jv = na_inc22(na_dot(g.off + 3, x0, x1, x2));
    const int64_t jw = na_inc22(na_dot(g.off + 6, x0, x1, x2));
    const int64_t base = (int64_t)g.lmn[0] * iu + (int64_t)g.lmn[1] * iv + (int64_t)g.lmn[2] * iw +
                         (int64_t)g.lmn[3] * ju + (int64_t)g.lmn[4] * jv + (int64_t)g.lmn[5] * jw;
    ph0[k] = (uint64_t)base << 42;
    du[k] = (uint64_t)iu << 42;
    dv[k] = (uint64_t)iv << 42;
    dw[k] = (uint64_t)iw << 42;
}

// sum over all atoms for Q consecutive points along the first axis of fnum;
// phases keep their top 16 bits (the reference's 2^16-entry table index).
// FP32 sums over a shared-memory chunk with Fast2Sum compensation (a coherent
// sum of nearly equal terms, as on a Bragg row, would otherwise round with a
// bias that grows with the chunk length), FP64 across chunks.
__global__ void __launch_bounds__(NOALLOC_NT) k_na_sum(const uint64_t *__restrict__ ph0,
                                                       const uint64_t *__restrict__ du,
                                                       const uint64_t *__restrict__ dv,
                                                       const uint64_t *__restrict__ dw, int64_t n, Geo g,
                                                       double2 *__restrict__ part)
{
    __shared__ uint64_t s_b[NOALLOC_NT], s_u[NOALLOC_NT], s_v[NOALLOC_NT], s_w[NOALLOC_NT];
    const int32_t nq = (g.fnum[0] + NOALLOC_Q - 1) / NOALLOC_Q;
    const int64_t nslots = (int64_t)nq * g.fnum[1] * g.fnum[2];
    const int64_t slot = (int64_t)blockIdx.x * NOALLOC_NT + threadIdx.x;
    const bool valid = slot < nslots;
    const int64_t sl = valid ? slot : 0;
    const uint32_t i0 = (uint32_t)(sl % nq) * NOALLOC_Q;
    const uint32_t j = (uint32_t)((sl / nq) % g.fnum[1]);
    const uint32_t l = (uint32_t)(sl / ((int64_t)nq * g.fnum[1]));
    double accd[NOALLOC_Q][2];
#pragma unroll
    for (int k = 0; k < NOALLOC_Q; k++) accd[k][0] = accd[k][1] = 0.0;
    for (int64_t a0 = 0; a0 < n; a0 += NOALLOC_NT) {
        const int cnt = (int)min((int64_t)NOALLOC_NT, n - a0);
        __syncthreads();
        if (threadIdx.x < cnt) {
            s_b[threadIdx.x] = ph0[a0 + threadIdx.x];
            s_u[threadIdx.x] = du[a0 + threadIdx.x];
            s_v[threadIdx.x] = dv[a0 + threadIdx.x];
            s_w[threadIdx.x] = dw[a0 + threadIdx.x];
        }
        __syncthreads();
        float accf[NOALLOC_Q][2], cmpf[NOALLOC_Q][2];
#pragma unroll
        for (int k = 0; k < NOALLOC_Q; k++) accf[k][0] = accf[k][1] = cmpf[k][0] = cmpf[k][1] = 0.f;
        for (int a = 0; a < cnt; a++) {
            const uint64_t d = s_u[a];
            uint64_t ph = s_b[a] + i0 * d + j * s_v[a] + l * s_w[a];
#pragma unroll
            for (int k = 0; k < NOALLOC_Q; k++) {
                const float x = (float)(int32_t)((ph & 0xFFFF000000000000ull) >> 32) * 4.656612873077393e-10f;
                float sn, cs;
                sincospif(x, &sn, &cs);
                const float t0 = accf[k][0] + cs, t1 = accf[k][1] + sn;
                cmpf[k][0] += cs - (t0 - accf[k][0]);
                cmpf[k][1] += sn - (t1 - accf[k][1]);
                accf[k][0] = t0;
                accf[k][1] = t1;
                ph += d;
            }
        }
#pragma unroll
        for (int k = 0; k < NOALLOC_Q; k++) {
            accd[k][0] += (double)accf[k][0] + (double)cmpf[k][0];
            accd[k][1] += (double)accf[k][1] + (double)cmpf[k][1];
        }
    }
    if (!valid) return;
#pragma unroll
    for (int k = 0; k < NOALLOC_Q; k++) {
        const uint32_t i = i0 + k;
        if (i < (uint32_t)g.fnum[0])
            part[i + (int64_t)g.fnum[0] * (j + (int64_t)g.fnum[1] * l)] = make_double2(accd[k][0], accd[k][1]);
    }
}

// tcsf(num) = cfact(istl) * sum on fnum, zero elsewhere (fourier_form.f90:147-177)
__global__ void k_na_form(const double2 *__restrict__ part, Geo g, const double2 *__restrict__ cfact,
                          const int32_t *__restrict__ istl, double2 *__restrict__ tcsf)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t np = (int64_t)g.num[0] * g.num[1] * g.num[2];
    if (p >= np) return;
    const int64_t i = p % g.num[0], j = (p / g.num[0]) % g.num[1], l = p / ((int64_t)g.num[0] * g.num[1]);
    double2 out = make_double2(0.0, 0.0);
    if (i < g.fnum[0] && j < g.fnum[1] && l < g.fnum[2]) {
        const double2 s = part[i + (int64_t)g.fnum[0] * (j + (int64_t)g.fnum[1] * l)];
        if (cfact) {
            const int32_t q = istl[p];
            if (q < 0 || q > DGPU_CFPKT) {      // not a table index: flag the point, read nothing
                out = make_double2(__longlong_as_double(0x7ff8000000000000ll), 0.0);
            } else {
                const double2 c = cfact[q];
                out = make_double2(s.x * c.x - s.y * c.y, s.x * c.y + s.y * c.x);
            }
        } else {
            out = s;
        }
    }
    tcsf[p] = out;
}

}  // namespace

extern "C" int dgpu_four_strucf_noalloc(void *stream, const double *d_xat, int64_t nxat, const double uin[3],
                                        const double vin[3], const double win[3], const double off_shift[9],
                                        const int32_t lmn[6], const int32_t num[3], const int32_t fnum[3],
                                        const double *d_cfact, const int32_t *d_istl, double *d_tcsf)
{
    if (!uin || !vin || !win || !off_shift || !lmn || !num || !fnum || !d_tcsf) return DGPU_ERR_ARG;
    if (nxat < 0 || (nxat > 0 && !d_xat) || (d_cfact && !d_istl)) return DGPU_ERR_ARG;
    for (int k = 0; k < 3; k++)
        if (num[k] < 1 || fnum[k] < 1 || fnum[k] > num[k]) return DGPU_ERR_ARG;
    const int64_t npts = (int64_t)fnum[0] * fnum[1] * fnum[2];
    if (nxat > NOALLOC_MAX_ATOMS || npts > NOALLOC_MAX_POINTS) return DGPU_ERR_SCRATCH_SIZE;
    void *base = nullptr;
    int rc = scratch_address(&base);
    if (rc) return rc;
    cudaStream_t st = (cudaStream_t)stream;
    if (st) {
        // the scratch address and the launches belong to the current device
        int sdev = -1, dev = -2;
        if (cudaStreamGetDevice(st, &sdev) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess) return DGPU_ERR_ARG;
        if (sdev != dev) return DGPU_ERR_ARG;
    }
    Geo g;
    for (int k = 0; k < 3; k++) {
        g.u[k] = uin[k];
        g.v[k] = vin[k];
        g.w[k] = win[k];
        g.num[k] = num[k];
        g.fnum[k] = fnum[k];
    }
    for (int k = 0; k < 9; k++) g.off[k] = off_shift[k];
    for (int k = 0; k < 6; k++) g.lmn[k] = lmn[k];
    uint64_t *ph0 = reinterpret_cast<uint64_t *>(base);
    uint64_t *du = ph0 + NOALLOC_MAX_ATOMS, *dv = du + NOALLOC_MAX_ATOMS, *dw = dv + NOALLOC_MAX_ATOMS;
    double2 *part = reinterpret_cast<double2 *>(static_cast<unsigned char *>(base) + NOALLOC_ATOM_BYTES);
    if (nxat > 0) k_na_phase<<<(unsigned)((nxat + 255) / 256), 256, 0, st>>>(d_xat, nxat, g, ph0, du, dv, dw);
    const int64_t nslots = (int64_t)((fnum[0] + NOALLOC_Q - 1) / NOALLOC_Q) * fnum[1] * fnum[2];
    k_na_sum<<<(unsigned)((nslots + NOALLOC_NT - 1) / NOALLOC_NT), NOALLOC_NT, 0, st>>>(ph0, du, dv, dw, nxat, g,
                                                                                        part);
    const int64_t np = (int64_t)num[0] * num[1] * num[2];
    k_na_form<<<(unsigned)((np + 255) / 256), 256, 0, st>>>(part, g, reinterpret_cast<const double2 *>(d_cfact),
                                                             d_istl, reinterpret_cast<double2 *>(d_tcsf));
    return cudaGetLastError() == cudaSuccess ? DGPU_OK : DGPU_ERR_CUDA;
}
