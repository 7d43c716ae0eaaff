// The Lanczos filter of four_run's epilogue (do_four_filter,
// discus/prog/fourier_sup.f90:1646-1803; 'set filter,lanczos' with
// width/damp/scale, fourier.f90:1156-1186, defaults fourier_reset.f90:101-105).
//
// The reference convolves dsi with a windowed sinc kernel through FFTW
// (do_lanczos_{1,2,3}d_fft, lib_f90/lib_lanczos.f90:224-426; lib_f90/lib_conv.f90):
// kernel table and field are moved to the FFT origin by maptofftfd, both are
// transformed forward, multiplied and transformed FORWARD again, and
// mapfftfdtoline moves the result back.  Two forward transforms give the
// circular convolution at negated indices, which the back map undoes up to
// the shifts its index formulas carry (one sample for even extents; the 1D
// back map drops the even-extent term the 2D/3D ones have).  The result is
// finally scaled so that its sum is the input's (times four_rscale).
//
// Here the same linear operator is applied directly: the kernel is a
// product of per-axis factors (wsinc and lqgm are products over the axes and
// the window test |q-g| < m holds on all axes or not at all), nonzero on at
// most 2m-1 offsets per axis, so the nD convolution is one circular pass per
// axis with that axis's taps, and output point o of an axis reads input
// point (s(o) - j) mod n for tap j.  The host derives s(o) and the taps from
// the reference's own index formulas, so the shifts come out as the FFT
// route has them.  One thread per output point and pass, FP64 throughout;
// the sums of the normalisation are FP64 block reductions.
#include <math.h>

#include <vector>

#include "dgpu_internal.h"

namespace {

const double PI_F = 3.1415926535897932384626433832795028841971693993751;

double sinc_ref(double x)                     // lib_functions.f90:10-30
{
    return fabs(x) < 1.0e-7 ? 1.0 : sin(x) / x;
}

// one axis of the filter: taps (j, w) and the source offset s(o) of every
// output point o
struct AxisPass {
    int n = 0;
    std::vector<int32_t> s;
    std::vector<int32_t> tj;
    std::vector<double> tw;
};

// The axis factor of the kernel table at offset d = q - g (1D: wsinc_1d is
// sinc squared), and the table's loops (do_lanczos_*d_fft: i1 = (n+1)/2,
// t = i1 - m - 1 .. i1 + m + 1, nscale = 1).  Returns false where the
// reference's table indices leave 1..n.
bool axis_pass(int n, int m, double rcut, bool one_d, AxisPass &a)
{
    const int c1 = (n + 1) / 2;                    // the table's centre (1-based)
    const int lo = (int)lrint(-(double)m - 1.0) + c1, hi = (int)lrint((double)m + 1.0) + c1;
    if (lo < 1 || hi > n) return false;
    a.n = n;
    const int l = (n - 1) % 2;
    for (int t = lo; t <= hi; t++) {
        const double d = (double)c1 - (double)t;
        double f = sinc_ref(PI_F * d * rcut);
        if (one_d) f *= sinc_ref(PI_F * d * rcut);
        f *= fabs(d) < (double)m ? sinc_ref(PI_F * d / (double)m) : 0.0;
        if (f == 0.0) continue;
        // table entry t (1-based) lands at FFT index mod(t + n/2 - l, n)
        a.tj.push_back((int32_t)((t + n / 2 - l) % n));
        a.tw.push_back(f);
    }
    // FFT index k of the twice-forward-transformed product holds the
    // circular convolution at -k; mapfftfdtoline writes it to field index
    // o = n - 1 - mod(k + n/2 - l', n) (l' = l for 2D/3D, 0 for 1D)
    // conv[-k] = sum_j b[j] a_fft[(-k - j) mod n] with a_fft[p] = field[(p + c0) mod n],
    // c0 the field index maptofftfd sends to 0: (c0 + 1 + n/2 - l) mod n = 0
    a.s.assign((size_t)n, -1);
    const int lb = one_d ? 0 : l;
    const int c0 = ((n - (n / 2 - l + 1)) % n + n) % n;
    for (int k = 0; k < n; k++) {
        const int o = n - 1 - (k + n / 2 - lb) % n;
        a.s[(size_t)o] = ((c0 - k) % n + n) % n;
    }
    return true;
}

// out = sum_t w[t] in[.., (s[o] - j[t]) mod n along the axis, ..]
__global__ void k_filter_axis(const double *__restrict__ in, double *__restrict__ out, int n0, int n1, int n2,
                              int axis, const int32_t *__restrict__ s, const int32_t *__restrict__ tj,
                              const double *__restrict__ tw, int ntap)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t np = (int64_t)n0 * n1 * n2;
    if (p >= np) return;
    int c[3] = {(int)(p % n0), (int)((p / n0) % n1), (int)(p / ((int64_t)n0 * n1))};
    const int n = axis == 0 ? n0 : axis == 1 ? n1 : n2;
    const int64_t stride = axis == 0 ? 1 : axis == 1 ? (int64_t)n0 : (int64_t)n0 * n1;
    const int so = s[c[axis]];
    const int64_t base = p - (int64_t)c[axis] * stride;
    double acc = 0.0;
    for (int t = 0; t < ntap; t++) {
        int i = so - tj[t];
        i = i < 0 ? i + n : i;
        acc += tw[t] * in[base + (int64_t)i * stride];
    }
    out[p] = acc;
}

__global__ void k_filter_sum(const double *__restrict__ a, int64_t np, double *__restrict__ part)
{
    __shared__ double sh[256];
    double v = 0.0;
    for (int64_t p = (int64_t)blockIdx.x * 256 + threadIdx.x; p < np; p += (int64_t)gridDim.x * 256) v += a[p];
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// dst = src * (sum_in / sum_out) * scale, the sums from the two partial sets
__global__ void k_filter_scale(const double *__restrict__ src, double *__restrict__ dst, int64_t np,
                               const double *__restrict__ pin, const double *__restrict__ pout, int nb,
                               double scale)
{
    __shared__ double f;
    if (threadIdx.x == 0) {
        double si = 0.0, so = 0.0;
        for (int k = 0; k < nb; k++) {
            si += pin[k];
            so += pout[k];
        }
        f = si / so * scale;
    }
    __syncthreads();
    for (int64_t p = (int64_t)blockIdx.x * 256 + threadIdx.x; p < np; p += (int64_t)gridDim.x * 256)
        dst[p] = src[p] * f;
}

// Filters one contiguous field of extents e[3] (the axes listed in ax are
// filtered; the others have extent 1) in place.
int filter_field(dgpu_ctx *ctx, double *d_f, const int e[3], const std::vector<int> &ax, int m, double rcut,
                 double scale)
{
    const int64_t np = (int64_t)e[0] * e[1] * e[2];
    const bool one_d = ax.size() == 1;
    std::vector<AxisPass> passes(ax.size());
    size_t ints = 0, dbls = 0;
    for (size_t k = 0; k < ax.size(); k++) {
        if (!axis_pass(e[ax[k]], m, rcut, one_d, passes[k]))
            return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED,
                                  "Lanczos filter: extent %d on axis %d is below 2 width + 3 (%s), where the "
                                  "reference's kernel table leaves its bounds",
                                  e[ax[k]], ax[k] + 1, e[ax[k]] % 2 ? "odd" : "even: 2 width + 4");
        ints += passes[k].s.size() + passes[k].tj.size();
        dbls += passes[k].tw.size();
    }
    const int nb = 152;
    // device scratch: two fields, the partial sums, the pass tables
    const size_t fb = (size_t)np * sizeof(double);
    DGPU_CUDA(ctx, ctx->filt.ensure(2 * fb + 2 * nb * sizeof(double) + dbls * sizeof(double) + ints * 4 + 256));
    double *tmp = ctx->filt.as<double>(), *tmp2 = tmp + np, *pin = tmp2 + np, *pout = pin + nb;
    double *tw = pout + nb;
    int32_t *ti = (int32_t *)(tw + dbls);
    std::vector<double> hw;
    std::vector<int32_t> hi;
    for (auto &a : passes) {
        hw.insert(hw.end(), a.tw.begin(), a.tw.end());
        hi.insert(hi.end(), a.s.begin(), a.s.end());
        hi.insert(hi.end(), a.tj.begin(), a.tj.end());
    }
    DGPU_CUDA(ctx, cudaMemcpyAsync(tw, hw.data(), hw.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(ti, hi.data(), hi.size() * sizeof(int32_t), cudaMemcpyHostToDevice, ctx->stream));
    k_filter_sum<<<nb, 256, 0, ctx->stream>>>(d_f, np, pin);
    DGPU_CUDA(ctx, cudaGetLastError());
    const unsigned nblk = (unsigned)dgpu_cdiv(np, 256);
    const double *src = d_f;
    double *bufs[2] = {tmp, tmp2};
    size_t oi = 0, ow = 0;
    for (size_t k = 0; k < passes.size(); k++) {
        const AxisPass &a = passes[k];
        double *dst = bufs[k % 2];
        k_filter_axis<<<nblk, 256, 0, ctx->stream>>>(src, dst, e[0], e[1], e[2], ax[k], ti + oi, ti + oi + a.n,
                                                      tw + ow, (int)a.tw.size());
        DGPU_CUDA(ctx, cudaGetLastError());
        oi += a.s.size() + a.tj.size();
        ow += a.tw.size();
        src = dst;
    }
    k_filter_sum<<<nb, 256, 0, ctx->stream>>>(src, np, pout);
    DGPU_CUDA(ctx, cudaGetLastError());
    k_filter_scale<<<nb, 256, 0, ctx->stream>>>(src, d_f, np, pin, pout, nb, scale);
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));      // the host tables are temporaries
    return DGPU_OK;
}

}  // namespace

// do_four_filter on the device array dsi(num) (Fortran order)
int dgpu_four_filter_dev(dgpu_ctx *ctx, const int32_t num[3], const dgpu_opts *op, double *d_dsi)
{
    if (op->filter != DGPU_FILTER_LANCZOS) return DGPU_OK;
    if (op->filter_scale != 1.0)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED,
                              "Lanczos filter: four_rscale other than 1 (the reference's strided copy of the "
                              "field does not fit the equal-sized output)");
    if (op->filter_width < 1) return dgpu_set_error(ctx, DGPU_ERR_ARG, "Lanczos filter: width < 1");
    const int m = op->filter_width, w2 = 2 * m + 1;
    const double rcut = op->filter_damp;
    int dim = 0;
    for (int k = 0; k < 3; k++) dim += num[k] > 1;
    const int64_t s1 = num[0], s2 = (int64_t)num[0] * num[1];
    if (dim == 3) {
        if (num[0] > w2 && num[1] > w2 && num[2] > w2) {
            const int e[3] = {num[0], num[1], num[2]};
            return filter_field(ctx, d_dsi, e, {0, 1, 2}, m, rcut, op->filter_scale);
        }
        if (num[2] <= w2) {                               // (i, j) slices, contiguous
            for (int k = 0; k < num[2]; k++) {
                const int e[3] = {num[0], num[1], 1};
                int rc = filter_field(ctx, d_dsi + k * s2, e, {0, 1}, m, rcut, op->filter_scale);
                if (rc) return rc;
            }
            return DGPU_OK;
        }
        // (i, l) or (j, l) slices: gathered into a contiguous field and back
        const int fixed = num[1] <= w2 ? 1 : num[0] <= w2 ? 0 : -1;
        if (fixed < 0) return DGPU_OK;
        const int a0 = fixed == 1 ? 0 : 1;
        const int e[3] = {num[a0], num[2], 1};
        const int64_t nf = (int64_t)e[0] * e[1];
        std::vector<double> all((size_t)(s2 * num[2])), sl((size_t)nf);
        DGPU_CUDA(ctx, cudaMemcpyAsync(all.data(), d_dsi, all.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                       ctx->stream));
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        DGPU_CUDA(ctx, ctx->filt_slice.ensure((size_t)nf * sizeof(double)));
        double *d_sl = ctx->filt_slice.as<double>();
        for (int f = 0; f < num[fixed]; f++) {
            for (int l = 0; l < num[2]; l++)
                for (int q = 0; q < num[a0]; q++) {
                    const int64_t i = fixed == 1 ? q : f, j = fixed == 1 ? f : q;
                    sl[(size_t)(q + (int64_t)num[a0] * l)] = all[(size_t)(i + s1 * j + s2 * l)];
                }
            DGPU_CUDA(ctx, cudaMemcpyAsync(d_sl, sl.data(), nf * sizeof(double), cudaMemcpyHostToDevice,
                                           ctx->stream));
            int rc = filter_field(ctx, d_sl, e, {0, 1}, m, rcut, op->filter_scale);
            if (rc) return rc;
            DGPU_CUDA(ctx, cudaMemcpyAsync(sl.data(), d_sl, nf * sizeof(double), cudaMemcpyDeviceToHost,
                                           ctx->stream));
            DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
            for (int l = 0; l < num[2]; l++)
                for (int q = 0; q < num[a0]; q++) {
                    const int64_t i = fixed == 1 ? q : f, j = fixed == 1 ? f : q;
                    all[(size_t)(i + s1 * j + s2 * l)] = sl[(size_t)(q + (int64_t)num[a0] * l)];
                }
        }
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_dsi, all.data(), all.size() * sizeof(double), cudaMemcpyHostToDevice,
                                       ctx->stream));
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        return DGPU_OK;
    }
    if (dim == 2) {
        // the reference filters dsi(:, :, 1) over num(1:2)
        if (num[0] < 2 || num[1] < 2)
            return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED,
                                  "Lanczos filter: a plane needs its two axes first (the reference filters "
                                  "dsi(:,:,1) and its kernel table leaves its bounds otherwise)");
        const int e[3] = {num[0], num[1], 1};
        return filter_field(ctx, d_dsi, e, {0, 1}, m, rcut, op->filter_scale);
    }
    if (dim == 1) {
        if (num[0] < 2)
            return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED,
                                  "Lanczos filter: a line needs the first axis (the reference filters "
                                  "dsi(:,1,1))");
        const int e[3] = {num[0], 1, 1};
        return filter_field(ctx, d_dsi, e, {0}, m, rcut, op->filter_scale);
    }
    return DGPU_OK;
}

extern "C" int dgpu_four_filter(dgpu_ctx *ctx, const int32_t num[3], const dgpu_opts *opts, double *dsi)
{
    if (!ctx || !num || !opts || !dsi) return DGPU_ERR_ARG;
    for (int k = 0; k < 3; k++)
        if (num[k] < 1) return dgpu_set_error(ctx, DGPU_ERR_ARG, "num");
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t np = (int64_t)num[0] * num[1] * num[2];
    DGPU_CUDA(ctx, ctx->dsi.ensure((size_t)np * sizeof(double)));
    double *d = ctx->dsi.as<double>();
    DGPU_CUDA(ctx, cudaMemcpyAsync(d, dsi, (size_t)np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    int rc = dgpu_four_filter_dev(ctx, num, opts, d);
    if (rc) return rc;
    DGPU_CUDA(ctx, cudaMemcpyAsync(dsi, d, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return DGPU_OK;
}
