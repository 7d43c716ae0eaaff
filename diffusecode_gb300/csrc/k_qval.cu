// qval (discus/prog/qval.f90:65-290): the value the output menu writes at a
// grid point, from csf, acsf and dsi of the last four_run and the form-factor
// tables.  One thread per grid point; the per-type sums run over the types.
//
// Reproduced as the reference indexes: the form-factor sums read
// istl(i, j, 1) (k ignored) and S(Q)'s Q^2 istl(i, 1, 1); the sign of a
// type's <f> is that of Re cfact_pure(1, type) (sin(theta)/lambda = 0.001);
// Q^2 is rounded to default REAL; the random phase tests h = eck + i vi_1 +
// j vi_2 for integers within 1e-6.  The <f> value (11, 19) keeps the sign
// variable at its initial 1.0: the reference leaves the saved sign of an
// earlier call there.
#include <math.h>

#include <vector>

#include "dgpu_internal.h"

#define QV_MAXT 64

struct QvalSpec {
    int32_t value, laver, nscat, n0, n1, n2;
    double amount[QV_MAXT];      // cr_amount(l), l = 1..nscat
    double signum[QV_MAXT];      // sign of Re cfact_pure(1, l)
    double n_real, u2aver;
    double eck[3], vi[9];
};

__device__ __forceinline__ double qv_abs(double2 c) { return sqrt(c.x * c.x + c.y * c.y); }

__global__ void k_qval(const QvalSpec *__restrict__ q, const double2 *__restrict__ csf,
                       const double2 *__restrict__ acsf, const double *__restrict__ dsi,
                       const int32_t *__restrict__ istl, const double2 *__restrict__ cfact,
                       const double2 *__restrict__ cfpure, const double *__restrict__ rnd, double *__restrict__ out)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t np = (int64_t)q->n0 * q->n1 * q->n2;
    if (p >= np) return;
    const int64_t i = p % q->n0, j = (p / q->n0) % q->n1;
    const double rad = 3.1415926535897932384626433832795028841971693993751 / 180.0;
    const double2 f = q->laver ? acsf[p] : csf[p];
    const double f2 = f.x * f.x + f.y * f.y;
    const int v = q->value;
    double r = 0.0;
    if (v == DGPU_VAL_INTEN) {
        r = q->laver ? f2 : dsi[p];
    } else if (v == DGPU_VAL_AMPLI) {
        r = sqrt(f2);
    } else if (v == DGPU_VAL_PHASE) {
        r = (f.x == 0.0 && f.y == 0.0) ? 0.0 : atan2(f.y, f.x) / rad;
    } else if (v == DGPU_VAL_REAL) {
        r = f.x;
    } else if (v == DGPU_VAL_IMAG) {
        r = f.y;
    } else if (v == DGPU_VAL_RANPH) {
        bool bragg = true;
        for (int l = 0; l < 3; l++) {
            const double h = q->eck[l] + q->vi[l] * (double)(float)i + q->vi[3 + l] * (double)(float)j;
            bragg = bragg && fabs(h - round(h)) < 0.000001;
        }
        if (bragg) r = (f.x == 0.0 && f.y == 0.0) ? 0.0 : atan2(f.y, f.x) / rad;
        else r = (rnd[p] - 0.5) * 360.0;
    } else if (v == DGPU_VAL_IQ) {
        r = (q->laver ? f2 : dsi[p]) / q->n_real;
    } else {
        const int32_t s = istl[i + (int64_t)q->n0 * j];            // istl(i, j, 1)
        const bool pure = v == DGPU_VAL_SQ || v == DGPU_VAL_F2AVER || v == DGPU_VAL_FAVER2 || v == DGPU_VAL_FAVER;
        const double2 *tab = pure ? cfpure : cfact;
        double sum = 0.0;
        for (int l = 1; l <= q->nscat; l++) {
            const double2 c = tab[(int64_t)(l - 1) * DGPU_NTAB + s];
            const double a = q->amount[l];
            if (v == DGPU_VAL_F2AVER || v == DGPU_VAL_F2AVERB) sum += (c.x * c.x + c.y * c.y) * a;
            else if (v == DGPU_VAL_FAVER || v == DGPU_VAL_FAVERB) sum += qv_abs(c) * a;     // sign kept at 1.0
            else sum += qv_abs(c) * a * q->signum[l];
        }
        if (v == DGPU_VAL_SQ) {
            const double I = q->laver ? f2 : dsi[p];
            const double zpi = 2.0 * 3.1415926535897932384626433832795028841971693993751;
            const double st = 2.0 * (double)istl[i] * DGPU_CFINC;   // istl(i, 1, 1)
            const double q2 = (double)(float)(zpi * zpi * (st * st));
            r = I / (sum * sum) / q->n_real + 1.0 - exp(-q2 * q->u2aver);
        } else if (v == DGPU_VAL_FAVER2 || v == DGPU_VAL_FAVER2B) {
            const double t = sum / q->n_real;
            r = t * t;
        } else {
            r = sum / q->n_real;
        }
    }
    out[p] = r;
}

extern "C" int dgpu_qval(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *opts,
                         int32_t value, int32_t laver, const double *csf, const double *acsf, const double *dsi,
                         const double *rand, double *out)
{
    if (!ctx || !cr || !grid || !opts || !out) return DGPU_ERR_ARG;
    const bool known = (value >= 1 && value <= 7) || (value >= 9 && value <= 11) || value == 13 ||
                       (value >= 17 && value <= 19);
    if (value == 14 || value == 15 || value == 16)
        return dgpu_set_error(ctx, DGPU_ERR_UNSUPPORTED, "PDF output values (%d) are not on this path", value);
    if (!known) return dgpu_set_error(ctx, DGPU_ERR_ARG, "output value %d", value);
    if (laver ? !acsf : !csf) return dgpu_set_error(ctx, DGPU_ERR_ARG, "csf/acsf missing");
    const bool needs_dsi = !laver && (value == DGPU_VAL_INTEN || value == DGPU_VAL_SQ || value == DGPU_VAL_IQ);
    if (needs_dsi && !dsi) return dgpu_set_error(ctx, DGPU_ERR_ARG, "dsi missing");
    if (value == DGPU_VAL_RANPH && !rand) return dgpu_set_error(ctx, DGPU_ERR_ARG, "random phases need rand");
    const bool tables = value == DGPU_VAL_SQ || value >= DGPU_VAL_F2AVER;
    if (tables && (cr->nscat < 1 || cr->nscat >= QV_MAXT || !cr->iscat || !cr->scat || !cr->occ || !cr->dw))
        return dgpu_set_error(ctx, DGPU_ERR_ARG, "crystal tables missing");
    for (int k = 0; k < 3; k++)
        if (grid->inc[k] < 1) return dgpu_set_error(ctx, DGPU_ERR_ARG, "inc(%d)=%d", k + 1, grid->inc[k]);
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t np = (int64_t)grid->inc[0] * grid->inc[1] * grid->inc[2];

    QvalSpec q;
    memset(&q, 0, sizeof(q));
    q.value = value;
    q.laver = laver ? 1 : 0;
    q.nscat = cr->nscat;
    q.n0 = grid->inc[0];
    q.n1 = grid->inc[1];
    q.n2 = grid->inc[2];
    for (int k = 0; k < 3; k++) q.eck[k] = grid->eck[k];
    memcpy(q.vi, grid->vi, sizeof(q.vi));
    // cr_amount, cr_n_real_atoms, cr_u2aver (chem_aver, chem_aver_mod.f90:495-537)
    if (cr->iscat && cr->nscat >= 1 && cr->nscat < QV_MAXT) {
        std::vector<int64_t> amount((size_t)cr->nscat + 1, 0);
        for (int64_t a = 0; a < cr->natoms; a++)
            if (cr->iscat[a] >= 0 && cr->iscat[a] <= cr->nscat) amount[cr->iscat[a]]++;
        double u2 = 0.0, nreal = 0.0;
        for (int l = 0; l <= cr->nscat; l++) {
            q.amount[l] = (double)amount[l];
            if (cr->dw) u2 += cr->dw[l] * (double)amount[l];
            if (l > 0) nreal += (double)amount[l];
        }
        const double pi = 3.1415926535897932384626433832795028841971693993751;
        q.n_real = nreal;
        q.u2aver = u2 / nreal / 8.0 / (double)(float)(pi * pi);
    }
    // tables: istl, cfact and cfact_pure (four_formtab without Debye-Waller and occupancy)
    double2 *d_cf = nullptr, *d_cfp = nullptr;
    int32_t *d_istl = nullptr;
    if (tables) {
        DGPU_CUDA(ctx, ctx->istl.ensure((size_t)np * sizeof(int32_t)));
        int rc = dgpu_stltab_dev(ctx, grid->eck, grid->vi, grid->inc, cr->rten, ctx->istl.as<int32_t>());
        if (rc) return rc;
        d_istl = ctx->istl.as<int32_t>();
        DGPU_CUDA(ctx, ctx->cfact.ensure((size_t)2 * cr->nscat * DGPU_NTAB * sizeof(double2)));
        d_cf = ctx->cfact.as<double2>();
        d_cfp = d_cf + (size_t)cr->nscat * DGPU_NTAB;
        rc = dgpu_formtab_dev(ctx, cr, opts, d_cf);
        if (rc) return rc;
        std::vector<double> ones((size_t)cr->nscat + 1, 1.0);
        dgpu_crystal pc = *cr;
        pc.occ = ones.data();
        dgpu_opts po = *opts;
        po.ldbw = 0;
        rc = dgpu_formtab_dev(ctx, &pc, &po, d_cfp);      // synchronises: ones may go
        if (rc) return rc;
        std::vector<double2> first((size_t)cr->nscat);
        for (int l = 1; l <= cr->nscat; l++)
            DGPU_CUDA(ctx, cudaMemcpyAsync(&first[l - 1], d_cfp + (size_t)(l - 1) * DGPU_NTAB + 1, sizeof(double2),
                                           cudaMemcpyDeviceToHost, ctx->stream));
        DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int l = 1; l <= cr->nscat; l++) q.signum[l] = first[l - 1].x < 0.0 ? -1.0 : 1.0;
    }
    // inputs and output in one staging buffer: spec | csf-or-acsf | dsi | rand | out
    const size_t spec_b = (sizeof(QvalSpec) + 255) & ~(size_t)255;
    DGPU_CUDA(ctx, ctx->wbuf.ensure(spec_b + (size_t)np * 5 * sizeof(double)));
    uint8_t *base = ctx->wbuf.as<uint8_t>();
    QvalSpec *d_q = reinterpret_cast<QvalSpec *>(base);
    double2 *d_f = reinterpret_cast<double2 *>(base + spec_b);
    double *d_dsi = reinterpret_cast<double *>(d_f + np);
    double *d_rnd = d_dsi + np;
    double *d_out = d_rnd + np;
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_q, &q, sizeof(q), cudaMemcpyHostToDevice, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_f, laver ? acsf : csf, (size_t)np * sizeof(double2), cudaMemcpyHostToDevice,
                                   ctx->stream));
    if (needs_dsi)
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_dsi, dsi, (size_t)np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    if (value == DGPU_VAL_RANPH)
        DGPU_CUDA(ctx, cudaMemcpyAsync(d_rnd, rand, (size_t)np * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    k_qval<<<(unsigned)dgpu_cdiv(np, 256), 256, 0, ctx->stream>>>(d_q, laver ? nullptr : d_f, laver ? d_f : nullptr,
                                                                   d_dsi, d_istl, d_cf, d_cfp, d_rnd, d_out);
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaMemcpyAsync(out, d_out, (size_t)np * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));      // q and the host arrays are read by now
    return DGPU_OK;
}

// ---------------------------------------------------------------------------
// calc_hkl (discus/prog/fourier_sup.f90:3230-3549): F at listed reflections

struct HklSpec {
    int32_t lo[3], n[3];
    double ncells, scale, exti, rlambda;
    double rten[9];
};

__global__ void k_calc_hkl(HklSpec s, const int32_t *__restrict__ hkl, int64_t nrefl, const double2 *__restrict__ csf,
                           double *__restrict__ out)
{
    const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= nrefl) return;
    const int32_t h = hkl[3 * r], k = hkl[3 * r + 1], l = hkl[3 * r + 2];
    double ic = 0.0, sg = 0.0, ph = 0.0;
    if (h != 0 || k != 0 || l != 0) {
        const int64_t idx = (h - s.lo[0]) + (int64_t)s.n[0] * ((k - s.lo[1]) + (int64_t)s.n[1] * (l - s.lo[2]));
        const double2 f = csf[idx];
        const double qq = sqrt(f.x * f.x + f.y * f.y) / s.ncells;
        // d* = do_blen(.false., hkl, 0): sqrt(h^T G* h)
        const double hv[3] = {(double)h, (double)k, (double)l};
        double d2 = 0.0;
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) d2 += hv[a] * s.rten[3 * b + a] * hv[b];
        const double rad = 3.1415926535897932384626433832795028841971693993751 / 180.0;
        const double tth = 2.0 * (asin(0.5 * s.rlambda * sqrt(d2)) / rad);       // 2 asind(...) in degrees
        const double ext = pow(1.0 / (1.0 + 0.001 * s.exti * qq * qq * s.rlambda * s.rlambda * s.rlambda /
                                                sin(tth * rad)),
                               0.25);
        ph = atan2(f.y, f.x) / rad;
        const double e = qq * ext;
        ic = e * e * s.scale;
        sg = sqrt(fabs(ic));
    }
    out[r] = ic;
    out[nrefl + r] = sg;
    out[2 * nrefl + r] = ph;
}

extern "C" int dgpu_calc_hkl(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *opts, const int32_t *hkl,
                             int64_t nrefl, double scale, double exti, double rlambda, double *icalc, double *sigi,
                             double *phase)
{
    if (!ctx || !cr || !opts || !hkl || nrefl < 0 || !icalc || !sigi) return DGPU_ERR_ARG;
    if (nrefl == 0) return DGPU_OK;
    int32_t lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};          // the reference's extrema start at 0
    for (int64_t r = 0; r < nrefl; r++)
        for (int a = 0; a < 3; a++) {
            lo[a] = hkl[3 * r + a] < lo[a] ? hkl[3 * r + a] : lo[a];
            hi[a] = hkl[3 * r + a] > hi[a] ? hkl[3 * r + a] : hi[a];
        }
    dgpu_grid g;
    memset(&g, 0, sizeof(g));
    for (int a = 0; a < 3; a++) {
        g.inc[a] = hi[a] - lo[a] + 1;
        g.vi[4 * a] = 1.0;                                  // vi = identity
        for (int c = 0; c < 4; c++) g.eck[3 * c + a] = lo[a];
        g.eck[3 * (a + 1) + a] = hi[a];                     // corners lr, ul, tl along h, k, l
    }
    const int64_t np = (int64_t)g.inc[0] * g.inc[1] * g.inc[2];
    DGPU_CUDA(ctx, cudaSetDevice(ctx->device));
    dgpu_crystal dc;
    int rc = dgpu_stage_crystal(ctx, cr, dc);
    if (rc) return rc;
    DGPU_CUDA(ctx, ctx->csf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->acsf.ensure(np * sizeof(double2)));
    DGPU_CUDA(ctx, ctx->dsi.ensure(np * sizeof(double)));
    rc = dgpu_four_run_dev(ctx, &dc, &g, opts, ctx->csf.as<double2>(), ctx->acsf.as<double2>(),
                           ctx->dsi.as<double>(), nullptr);
    if (rc < 0) return rc;
    HklSpec s;
    memset(&s, 0, sizeof(s));
    for (int a = 0; a < 3; a++) {
        s.lo[a] = lo[a];
        s.n[a] = g.inc[a];
    }
    s.ncells = (double)cr->icc[0] * cr->icc[1] * cr->icc[2];
    s.scale = scale;
    s.exti = exti;
    s.rlambda = rlambda;
    memcpy(s.rten, cr->rten, sizeof(s.rten));
    DGPU_CUDA(ctx, ctx->wbuf.ensure((size_t)nrefl * (3 * sizeof(double) + 3 * sizeof(int32_t)) + 256));
    double *d_out = ctx->wbuf.as<double>();
    int32_t *d_hkl = reinterpret_cast<int32_t *>(d_out + 3 * nrefl);
    DGPU_CUDA(ctx, cudaMemcpyAsync(d_hkl, hkl, (size_t)nrefl * 3 * sizeof(int32_t), cudaMemcpyHostToDevice,
                                   ctx->stream));
    k_calc_hkl<<<(unsigned)dgpu_cdiv(nrefl, 256), 256, 0, ctx->stream>>>(s, d_hkl, nrefl, ctx->csf.as<double2>(),
                                                                          d_out);
    DGPU_CUDA(ctx, cudaGetLastError());
    DGPU_CUDA(ctx, cudaMemcpyAsync(icalc, d_out, (size_t)nrefl * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaMemcpyAsync(sigi, d_out + nrefl, (size_t)nrefl * sizeof(double), cudaMemcpyDeviceToHost,
                                   ctx->stream));
    if (phase)
        DGPU_CUDA(ctx, cudaMemcpyAsync(phase, d_out + 2 * nrefl, (size_t)nrefl * sizeof(double),
                                       cudaMemcpyDeviceToHost, ctx->stream));
    DGPU_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return rc;
}
