// Anisotropic-ADP groups and lots (k_lots.cu) and the lot epilogue
// (k_epilogue.cu).
#pragma once
#include <vector>

#include "dgpu_internal.h"

// Numbers the (type, ADP type) pairs present among the atoms (cr: device
// iscat and ianis), fills the group part of fs (gtype, gU, ar, ngroup,
// adbw = ldbw, ldbw = 0) and leaves every atom's group in ctx->geff.
int dgpu_anis_groups(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, FormSpec &fs, int32_t *ngroup);

// four_csize (fourier_sup.f90:2533-2555)
void dgpu_csize(const dgpu_crystal *cr, const dgpu_opts *op, int32_t cs[3]);
bool dgpu_lots_on(const dgpu_opts *op);
// cell (ii,jj,kk) of the ls_xyz box belongs to the lot (ellipsoid test of
// fourier_sup.f90:1908-1937, summed x1 + x2 + x3 as there)
bool dgpu_lot_member(const dgpu_opts *op, int32_t ii, int32_t jj, int32_t kk);

struct LotGeom {
    int32_t icc[3], ls[3];
    int32_t ncatoms, ngroup, ncs;      // ncs: cells of the lot shape
    int64_t natoms, cr_end, nextra, per_lot;
    double dim0[3];
    int64_t dlo[3];                    // NINT(cr_dim(:,1))
};

struct LotPlan {
    LotGeom geo;
    int64_t nlots = 0;
    int32_t ngroup = 0, per_chunk = 0, ncell = 0;
    const int32_t *d_orig = nullptr, *d_shape = nullptr, *d_member = nullptr;
    std::vector<int32_t> shape;        // host copy of the shape's cells (3 per cell)
};
int dgpu_lot_plan(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op, int32_t ngroup, LotPlan &lp);
// Atoms of lots [lot0, lot0+nlot) into ctx->lpos / ltype / locc from slot
// slot0 on (the caller sizes the buffers), types L*ngroup + group (0 = empty
// slot); *nslots = nlot * per_lot.
int dgpu_lot_gather(dgpu_ctx *ctx, const LotPlan &lp, int64_t lot0, int32_t nlot, const double *pos,
                    const int32_t *geff, const float *aocc, int64_t slot0, int64_t *nslots,
                    int32_t *lorig = nullptr);   // lorig: the source atom of each slot (-1: empty)

// What the chi^2 gradient needs of the last four_run with lots: its plan,
// groups, phase geometry, engine and the lot normalisation.
struct LotKeep {
    LotPlan lp;
    int32_t ngroup = 0;
    int32_t engine = 0;
    const int32_t *eiscat = nullptr;   // device: types, or the (type, ADP) groups
    PhaseGeom geo;
    double dnorm = 1.0;
};

// epilogue of the lots
int dgpu_group_factors(dgpu_ctx *ctx, const FormSpec &fs, const BoxSpec &box, const int32_t *istl,
                       const double2 *cfact, double2 *fac);
int dgpu_lot_combine(dgpu_ctx *ctx, int32_t ngroup, int32_t nlot, const BoxSpec &box, const PartRef *part,
                     const double2 *fac, const double2 *acsf, double2 *csf, double *dsi, int32_t last);
int dgpu_lot_scale(dgpu_ctx *ctx, const BoxSpec &box, double2 *csf, double *dsi, double dscale, double cscale);
