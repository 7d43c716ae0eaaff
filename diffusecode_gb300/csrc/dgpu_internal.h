// Internal declarations of the GB300 Fourier structure-factor library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <tuple>
#include <vector>
#include <stdio.h>
#include <string.h>

#include "../../include/discus_gpu.h"

#define DGPU_NTAB (DGPU_CFPKT + 1)
#define DGPU_DISC_MAXSYM 192   // DISCAMB symmetry operation numbers 0..192 (discus_discamb.f90:82)

// ---------------------------------------------------------------------------
// device buffer that only grows
struct DevBuf {
    void *p = nullptr;
    size_t cap = 0;
    cudaError_t ensure(size_t bytes) {
        if (bytes <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        size_t want = bytes < 256 ? 256 : bytes;
        cudaError_t e = cudaMalloc(&p, want);
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
    template <class T> T *as() const { return reinterpret_cast<T *>(p); }
};

// Pinned host memory handed out in order and taken back all at once after a
// host wait: the source of asynchronous uploads whose host copy must outlive
// the call that enqueues them.
struct HostArena {
    char *p = nullptr;
    size_t cap = 0, used = 0;
    std::vector<char *> old;              // outgrown blocks, freed at the next reset
    void *take(size_t bytes) {
        bytes = (bytes + 255) & ~(size_t)255;
        if (used + bytes > cap) {
            size_t want = cap * 2 > bytes ? cap * 2 : bytes;
            if (want < ((size_t)1 << 20)) want = (size_t)1 << 20;
            char *q = nullptr;
            if (cudaMallocHost(reinterpret_cast<void **>(&q), want) != cudaSuccess) return nullptr;
            if (p) old.push_back(p);
            p = q;
            cap = want;
            used = 0;
        }
        void *r = p + used;
        used += bytes;
        return r;
    }
    void reset() {                        // only after the uploads from it have completed
        for (char *q : old) cudaFreeHost(q);
        old.clear();
        used = 0;
    }
    void release() {
        reset();
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

// Per-atom phase data, grouped by type (SoA).  Phases are 64-bit fixed point
// in units of 2^-64 turn: phase(n) = ph0 + n0*d0 + n1*d1 + n2*d2 (mod 2^64).
struct AtomSet {
    uint64_t *ph0, *du, *dv, *dw;
    float *w;
    int64_t *type_start;   // [nscat+2] (host copy kept in HostAtomSet)
    int64_t n;             // total atoms stored
};

struct Tables {
    int32_t *istl;         // [np] full grid
    double2 *cfact;        // [nscat][NTAB]
};

// one tensor-core launch configuration (chosen by the autotuner)
struct TcChoice {
    int32_t axis = -1, N = 0, slice_mult = 4;
};
typedef std::tuple<int32_t, int32_t, int32_t, int32_t, int32_t, int32_t, int32_t> TcKey;

struct BatchState;   // k_batch.cu
struct LotKeep;      // dgpu_lots.h
struct FormSpec;

#define DGPU_NEV 10
struct dgpu_ctx {
    int device = 0;
    int nsm = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[DGPU_NEV] = {};   // 0-1 four_run, 2-3 sums, 4-7 tensor core, 8-9 powder
    char err[512] = {0};
    // cached buffers
    DevBuf pos, iscat, aocc, sel;
    DevBuf counts;                      // per-block type counts, their scan, type starts
    DevBuf ph0, du, dv, dw, w;          // main atom set
    DevBuf aph0, adu, adv, adw, aw;     // folded atoms for <F>
    DevBuf aaidx;                       // original atom index of each folded slot
    DevBuf istl, cfact, part, apart, lat, csf, acsf, dsi, stats, flag;
    DevBuf tc_part, tc_work, aidx;          // aidx: original atom index of each prepared slot
    DevBuf tc_mult;                         // per-atom step factors of the tensor-core engine
    DevBuf tc_tab;                          // exp(2 pi i k / 4096), FP64, for the step factors
    DevBuf ph_tab;                          // exp(2 pi i j / 1024), FP32, the CUDA-core phasor table
    DevBuf filt, filt_slice;                // Lanczos filter: work fields, sums, pass tables; one slice
    DevBuf tc_vimg;                         // V operand images of the tensor-core engine
    DevBuf adj_qimg, adj_items;             // tensor-core adjoint: Q images, work items
    int64_t ts_main[2 * 64 + 4] = {};      // type ranges of the last main atom preparation
    DevBuf ianis, geff, ghist;              // ADP types, group of every atom, (type, ADP) histogram
    DevBuf isymb, dtab;                     // DISCAMB: symmetry of every atom, the form-factor tables
    DevBuf lpos, ltype, locc, lplan, lfac;  // lot crystals, lot plan, group factors
    FormSpec *fs_main = nullptr;            // host copy of the last main combine's FormSpec
    FormSpec *fs_type = nullptr;            // host copy of the last per-type FormSpec (<F> combine)
    LotKeep *lot_keep = nullptr;            // the last four_run's lots, for the gradient (null: no lots)
    DevBuf lorig;                           // lots: source atom of each gathered slot
    // <F> of the last four_run when it was a box lattice in closed form:
    // A(h) = norm L(h) sum_t c_t(h) S_t(h) over the folded atoms (aph0.., ts)
    struct AverKeep {
        int32_t on = 0;
        int32_t nscat = 0;
        int32_t lat_n[3] = {0, 0, 0};
        double lat_d[3] = {0, 0, 0};
        double norm = 0.0;
        int64_t ts[2 * 64 + 4] = {};
    } aver;
    DevBuf wbuf, acc_csf, acc_dsi;          // four_weight staging; four_accumulate sums
    DevBuf rlist, rsum;                     // refinement of <F>-cancelling points: list, exact sums
    DevBuf slab_ph0;                        // powder: per-slab origin phases of the atoms
    int64_t acc_np = 0;                     // points of the accumulated sums (0: none)
    std::vector<int32_t> symm_inv;          // inverses of the point-group operations (four_symm), 9 each
    // what ctx->istl and ctx->cfact hold (the reference recomputes its tables
    // only when the grid or the form factors change, four_layer,
    // fourier_sup.f90:2578-2582): buffer, capacity and the inputs
    struct TabKey {
        const void *p = nullptr;
        size_t cap = 0;
        std::vector<double> k;
    } stl_key, cf_key;
    DevBuf gq, gpart, grad, batch_desc, batch_aux;
    double batch_ms = 0.0;
    bool batch_by_member = false;           // the last dgpu_batch_run ran member by member (no graph)
    double tc_kernel_ms = 0.0;              // duration of the last single-problem tensor-core launch
    std::map<TcKey, TcChoice> tc_tuned;   // autotuner results per problem shape
    BatchState *batch[2] = {nullptr, nullptr};   // captured population graphs (most recent first)
    int32_t tc_last[4] = {-1, -1, -1, -1};
    // Deferred tensor-core launches (a run of launches with one host wait at
    // its end): plans are uploaded from the pinned arena, the error flag is
    // cleared once before the run and read after it.
    int tc_defer = 0;
    HostArena stage;
    // per-device facts set on first use by this context (a process may hold
    // contexts on several GPUs): tensor cores present, shared-memory opt-ins
    int tc_avail = -1;
    bool tc_attr = false, adj_attr = false;
    std::vector<cudaEvent_t> run_ev;        // event pairs around the launches of such a run
};

// error helpers ---------------------------------------------------------
int dgpu_set_error(dgpu_ctx *ctx, int code, const char *fmt, ...);
#define DGPU_CUDA(ctx, call)                                                          \
    do {                                                                              \
        cudaError_t _e = (call);                                                      \
        if (_e != cudaSuccess)                                                        \
            return dgpu_set_error((ctx), _e == cudaErrorMemoryAllocation ? DGPU_ERR_NOMEM \
                                                                         : DGPU_ERR_CUDA, \
                                  "%s: %s (%s:%d)", #call, cudaGetErrorString(_e),   \
                                  __FILE__, __LINE__);                                \
    } while (0)

// ---------------------------------------------------------------------------
// Phase geometry passed to kernels
struct PhaseGeom {
    int32_t mode;          // DGPU_PHASE_*
    int32_t lmn[6];
    double eck[3];         // eck(:,1)
    double vi[9];          // vi(:,1..3) column-major
    double off[9];         // off_shift column-major
};

// host side: fourier_lmn
int dgpu_lmn_host(const double eck[12], const double vi[9], const int32_t inc[3],
                  int32_t lmn[6], double off[9]);

// prepare.cu ------------------------------------------------------------
// Stable gather of atoms by type into phase data.  If fold != 0, atoms are
// folded into their unit cell (four_aver) and only selected cells are kept.
// h_type_start receives 2*nscat+1 values: the start of each type's range
// (multiples of 64; the gaps are zero-weight padding), the padded total, and
// the real atom count of each type.
struct FoldSpec {
    int32_t fold;
    int32_t ncatoms;
    int32_t icc[3];
    double dim0[3];
    const uint8_t *sel;    // device, may be null (all cells)
};
int dgpu_prepare_atoms(dgpu_ctx *ctx, const double *d_pos, const int32_t *d_iscat,
                       const float *d_aocc, int64_t natoms, int32_t nscat,
                       const PhaseGeom &g, const FoldSpec &fs, DevBuf &ph0, DevBuf &du,
                       DevBuf &dv, DevBuf &dw, DevBuf &w, int64_t *h_type_start, DevBuf *idx = nullptr);
// The same in two phases, for callers that learn the type starts of several
// atom sets with one host wait: the count phase (per-block type counts,
// their scan and the type starts d_ts, device only) into a region of
// dgpu_prepare_region_bytes, then the scatter with the padded total.
struct PrepRegion {
    int32_t *counts;
    int64_t *offs;
    int64_t *d_ts;         // 2*nscat+1 values as h_type_start
    int64_t nblk;
};
size_t dgpu_prepare_region_bytes(int64_t natoms, int32_t nscat);
PrepRegion dgpu_prepare_region(void *base, int64_t natoms, int32_t nscat);
int dgpu_prepare_count(dgpu_ctx *ctx, const int32_t *d_iscat, int64_t natoms, int32_t nscat, const FoldSpec &fs,
                       const PrepRegion &r);
int dgpu_prepare_scatter(dgpu_ctx *ctx, const double *d_pos, const int32_t *d_iscat, const float *d_aocc,
                         int64_t natoms, int32_t nscat, const PhaseGeom &g, const FoldSpec &fs, const PrepRegion &r,
                         int64_t total, DevBuf &ph0, DevBuf &du, DevBuf &dv, DevBuf &dw, DevBuf &w,
                         DevBuf *idx = nullptr);
// idx: where the original atom index of every slot goes (ctx->aidx when null)
// Lattice points of all cells (four_getav LOT_OFF) as one atom set.
int dgpu_prepare_lattice(dgpu_ctx *ctx, const int32_t icc[3], const double dim0[3],
                         const PhaseGeom &g, DevBuf &ph0, DevBuf &du, DevBuf &dv,
                         DevBuf &dw, DevBuf &w);

// tables.cu -------------------------------------------------------------
int dgpu_stltab_dev(dgpu_ctx *ctx, const double eck[3], const double vi[9],
                    const int32_t num[3], const double rten[9], int32_t *d_istl);
int dgpu_formtab_dev(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op,
                     double2 *d_cfact);
int dgpu_increments_dev(dgpu_ctx *ctx, const double *d_xat, int64_t nxat,
                        const double uin[3], const double vin[3], const double win[3],
                        const double off[9], int64_t *d_out);

// direct.cu -------------------------------------------------------------
// Sum over the atoms of each type: part[t][s][p] (complex double) on the
// box fnum; ntype types with atom ranges from type_start.
struct BoxSpec {
    int32_t f[3];          // computed box
    int32_t num[3];        // full grid
};
int dgpu_direct_sums(dgpu_ctx *ctx, const uint64_t *ph0, const uint64_t *du,
                     const uint64_t *dv, const uint64_t *dw, const float *w,
                     const int64_t *h_type_start, int32_t ntype, int32_t ref_mask,
                     const BoxSpec &box, DevBuf &part, int32_t *nslice_out);

// tc.cu -----------------------------------------------------------------
// One problem (one crystal's type sums): geometry, atom arrays and the output
// partials.  Lives in global memory; a launch may cover many problems.
struct TcProblem {
    int32_t f[3];
    int32_t ra, rb, ac;       // row axes (ra the longer) and column axis
    int32_t fra, fra_p, frb;  // row extents; ra padded to a multiple of 8
    int32_t ncols;
    int32_t N;               // columns per tile (multiple of 16, <= TcLaunch::Nmax)
    int32_t m_tiles, n_tiles, nslice, ntype;
    int32_t vstride;         // column tiles per atom group in the V images (n_tiles, or more when shared)
    int64_t nrows_p;         // fra_p * frb: rows of the tile space (rg = nb * fra_p + na)
    int64_t slice_len, nitems, item0, slab;
    int64_t ts[65];
    const uint64_t *ph0, *dra, *drb, *dac;   // phase data along the row axes and the column axis
    const float *w;
    const float2 *ma, *mc;   // per-atom exp(2 pi i 8 d) along ra and ac
    const float2 *ma2, *mc2; // per-atom exp(2 pi i 16 d) along ra and ac
    uint8_t *vimg;           // B rows of every (atom group, column tile), or null: generated in-kernel;
                             // problems with the same atoms and column steps share one set
    float2 *part;            // part[(t*nslice+ks)*slab + c*nrows_p + rg]
};

// Launch-wide constants: shared-memory and TMEM layout follow Nmax.
struct TcLaunch {
    const TcProblem *probs;
    const int32_t *item_prob;   // problem index of every work item
    int64_t nitems;
    int32_t Nmax, stages, flush, nbuf, bf16;
    int32_t tsum;               // running sum of the main accumulator kept in TMEM
    int32_t vring;              // V operand streamed from images through a shared-memory ring
    uint32_t tmem_cols;
    int32_t *err;
    uint64_t timeout_ns;        // limit of one wait for another warp's progress
};

#include <vector>
// Step factors per atom: exp(2 pi i 8 d) along the three grid axes, then
// exp(2 pi i 16 d) along them (dgpu_tc_mult_async).
#define TC_MULT_ARRAYS 6
// One problem's inputs for a tensor-core launch.
struct TcInput {
    const uint64_t *ph0, *du, *dv, *dw;
    const float *w;
    const float2 *mult;       // step factors: mult[k * mult_stride + atom], k < TC_MULT_ARRAYS
    int64_t mult_stride;
    const int64_t *ts;        // host: padded type ranges (ntype + 1 values)
    int32_t ntype;
    BoxSpec box;
    int32_t axis;             // column axis, -1 = least padding
};
// A planned launch: descriptors uploaded, partial buffer allocated.
struct TcPlan {
    std::vector<TcProblem> probs;
    std::vector<int32_t> item_prob;
    TcLaunch L;
    size_t smem = 0;
    std::vector<int64_t> part_off;     // float2 offset of each problem's partials
    std::vector<int32_t> nslice;
    bool vimg = false;                 // V images generated before the main kernel
    bool vshared = false;              // one image set serves every problem
};
// vimg: buffer for the V images of the launch (null, or too large for the
// image budget: V is generated inside the kernel instead)
int dgpu_tc_plan(dgpu_ctx *ctx, int nprob, const TcInput *in, const dgpu_opts *op, int N, int slice_mult,
                 TcPlan &plan, DevBuf &part, DevBuf &desc, DevBuf *vimg);
// Enqueues the V images and the kernel only; timed: events ev[6], ev[7]
// around the main kernel.
int dgpu_tc_launch(dgpu_ctx *ctx, const TcPlan &plan, bool timed = false);
int dgpu_tc_check(dgpu_ctx *ctx);                               // waits, reads the error flag
struct PartRef;
// Per-atom step factors exp(2 pi i 8 d) of du, dv, dw (n atoms) into
// out[axis * stride + atom]; enqueue only.
// The step factors' FP64 table, once per context (at creation).
int dgpu_tc_init(dgpu_ctx *ctx);
// mask: the axes (bit a for axis a) whose factors are written
int dgpu_tc_mult_async(dgpu_ctx *ctx, const uint64_t *du, const uint64_t *dv, const uint64_t *dw, int64_t n,
                       int64_t stride, float2 *out, int mask = 7);
// Layout of a problem's partials for the combine kernels.
void dgpu_tc_partref(const TcProblem &g, const float2 *p, PartRef &ref);
// Single problem with autotuned tile; partial sums are float2 (FP32, one per
// work item, RN-accumulated drains); ref receives their layout.  With
// ctx->tc_defer set (and the tile already tuned) it enqueues without a host
// wait, and the caller reads the error flag with dgpu_tc_check after the run.
int dgpu_tc_sums(dgpu_ctx *ctx, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv,
                 const uint64_t *dw, const float *w, const int64_t *h_type_start,
                 int32_t ntype, const BoxSpec &box, const dgpu_opts *op, DevBuf &part,
                 PartRef *ref);
bool dgpu_tc_available(dgpu_ctx *ctx);

// epilogue.cu -----------------------------------------------------------
// Form factors of the combine and adjoint kernels.  The partial sums come
// per group g = 1..ngroup: a scattering type (isotropic crystal, gtype[g] = g)
// or a (type, ADP type) pair of an anisotropic crystal, whose factor is
// cfact(gtype[g]) times, when adbw, exp(-2 pi^2 h^T (a*_i a*_j U_ij) h) with
// the group's U (four_dbwtab, fourier_sup.f90:2809-2831).  ldbw here is the
// isotropic term inside cfact: off for an anisotropic crystal (:2729).
struct FormSpec {
    int32_t mode;          // DGPU_FORM_*
    int32_t nscat;
    int32_t lxray, power, ano, ldbw;
    int32_t ngroup, adbw;
    int32_t gtype[64];     // group -> scattering type
    double scat[64 * 11];  // per type coefficients (types 1..nscat, <=63)
    double occ[64], dw[64], delfr[64], delfi[64];
    double rten[9];
    double eck[3], vi[9];
    double gU[64 * 6];     // U11, U22, U33, U23, U13, U12 of each group (A^2)
    double ar[3];          // reciprocal cell lengths (1/A)
    // DISCAMB: group g takes table gtab[g] (< dntab) of dtab (device) at nint(h)
    int32_t disc, dntab;
    int32_t dmax[3];
    int32_t gtab[64];
    const double2 *dtab;
};
// Partial sums part[t][s][p] of either engine: double2 (direct) or float2 (TC).
// Element (point i,j,l of the box, type t, slice k) at
// (t*nslice + k)*slab + i*s[0] + j*s[1] + l*s[2]; s[0] == 0 means the dense
// box order (s = 1, f0, f0*f1; slab = f0*f1*f2).
struct PartRef {
    const void *p;
    int32_t nslice;
    int32_t f32;
    int64_t s[3];
    int64_t slab;
};
int dgpu_combine(dgpu_ctx *ctx, const FormSpec &fs, const BoxSpec &box, const PartRef &part,
                 const int32_t *istl, const double2 *cfact,
                 const double2 *acsf_box_in, double2 *csf, double *dsi, double diff_scale);
int dgpu_aver_combine(dgpu_ctx *ctx, const FormSpec &fs, const BoxSpec &box,
                      const PartRef &apart, const int32_t *istl,
                      const double2 *cfact, const double2 *lat, int32_t lat_nslice,
                      int32_t lat_closed, const int32_t icc[3], const double dim0[3],
                      double norm, double2 *acsf);

// Points whose |<F>|^2 exceeds REFINE_TAU * N <|f|^2> are recomputed exactly
// after a tensor-core run with <F> subtracted (k_refine.cu).
#define REFINE_TAU 64.0
struct RefineSpec {
    BoxSpec box;
    const FormSpec *fsm, *fst;             // host: groups of the main sums, plain types of <F>
    const int32_t *istl;
    const double2 *cfact;
    const uint64_t *ph0, *du, *dv, *dw;    // main atom set, by group
    const float *w;
    const int64_t *ts_main;                // host type ranges (2 ngroup + 1 values)
    int32_t ngroup;
    const uint64_t *aph0, *adu, *adv, *adw;   // atoms folded into one cell, by type
    const float *aw;
    const int64_t *ts_fold;
    int32_t nscat;
    int32_t lat_n[3];                      // closed-form lattice of <F>
    double lat_d[3], norm, diff_scale;
};
int dgpu_refine_aver(dgpu_ctx *ctx, const RefineSpec &r, double2 *csf, double2 *acsf, double *dsi, int64_t *nref);
int dgpu_friedel_mirror(dgpu_ctx *ctx, const BoxSpec &box, int32_t idim, double2 *csf,
                        double2 *acsf, double *dsi);
int dgpu_qinfo(dgpu_ctx *ctx, const double eck[3], const double vi[9], const int32_t num[3],
               const double *dsi, double res[7]);

// enqueue-only helpers for captured sequences (batch)
void dgpu_type_ranges(const int32_t *iscat, int64_t n, int32_t nscat, int64_t *ts);
int64_t dgpu_prepare_blocks(int64_t natoms);
int dgpu_prepare_async(dgpu_ctx *ctx, const double *d_pos, const int32_t *d_iscat, const float *d_aocc,
                       int64_t natoms, int32_t nscat, const PhaseGeom &g, int32_t *counts, int64_t *offs,
                       int64_t *ts_dev, uint64_t *ph0, uint64_t *du, uint64_t *dv, uint64_t *dw, float *w,
                       int32_t *idx);
int dgpu_stltab_async(dgpu_ctx *ctx, const double eck[3], const double vi[9], const int32_t num[3],
                      const double rten[9], int32_t *d_istl, int32_t *d_flag);
size_t dgpu_formcoef_bytes();
void dgpu_formcoef_fill(const dgpu_crystal *cr, void *host);
int dgpu_formtab_async(dgpu_ctx *ctx, const void *d_coef, int32_t nscat, const dgpu_opts *op, double2 *d_cfact);
int dgpu_combine_async(dgpu_ctx *ctx, const FormSpec *d_fs, const BoxSpec &box, const PartRef &part,
                       const int32_t *istl, const double2 *cfact, double2 *csf, double *dsi, double diff_scale);

// ---- member-indexed launches of a batch (one launch for all members) -----
// Member blockIdx.y of a launch runs the blocks its own size needs; the rest
// of the launch's blocks return at once.  The arrays of member descriptors
// live in device memory (filled once per batch shape).
struct PrepMember {
    const double *pos;
    const int32_t *iscat;
    const float *aocc;
    int64_t n, nblk;       // atoms, prepare blocks
    int32_t nscat, num[3]; // nscat: partial-sum groups
    int32_t ncf, ldbw_cf;  // scattering types and isotropic Debye-Waller term of cfact
    PhaseGeom g;
    int32_t *counts;
    int64_t *offs, *ts;
    uint64_t *ph0, *du, *dv, *dw;
    float *w;
    int32_t *idx;
    double rten[9];
    int32_t *istl;
    const void *coef;      // FormCoef of the member's types
    double2 *cfact;
};
// type counts, scan and scatter of every member's atoms
int dgpu_prepare_members(dgpu_ctx *ctx, const PrepMember *d_m, int32_t nc, int64_t max_nblk);
// istl and cfact of every member (constants of a batch shape); flag: set
// when an istl exceeds the form-factor table
int dgpu_tables_members(dgpu_ctx *ctx, const PrepMember *d_m, int32_t nc, int64_t max_np, int32_t max_nscat,
                        const dgpu_opts *op, int32_t *flag);

struct PartLayout {
    int64_t s0, s1, s2, slab;
    int64_t m1, m2, nthr;      // strides of axes a1, a2; slots walked
    int32_t a0, a1, a2;        // box axes from innermost to outermost
};
PartLayout dgpu_part_layout(const PartRef &r, const BoxSpec &box);
struct EpiMember {
    const FormSpec *fs;    // device
    BoxSpec box;
    const float2 *part;
    int32_t nslice, idim;
    PartLayout lay;
    const int32_t *istl;
    const double2 *cfact;
    double2 *csf;
    double *dsi;
    double ds, sqds;
    int64_t np;
};
// combine and Friedel mirror of every member (tensor-core FP32 partials)
int dgpu_epilogue_members(dgpu_ctx *ctx, const EpiMember *d_m, int32_t nc, int64_t max_thr, int64_t max_np);
struct AdjMember {
    const FormSpec *fs;    // device
    BoxSpec box;
    int32_t idim, nscat;
    const double2 *csf;
    const double *dsi;
    const int32_t *istl;
    const double2 *cfact;
    const double *it, *wt;
    double *g, *chi;       // chi: 512 block parts, then chi^2 at chi[512]
    double *chi_out;       // chi^2 again, contiguous over the members
    double sqds;
    int64_t np, nb;
    float2 *Q;
};
// g, chi^2 and Q of every member (the per-atom sums follow on the tensor cores)
int dgpu_adjoint_members(dgpu_ctx *ctx, const AdjMember *d_m, int32_t nc, int64_t max_nb);

// ---- adjoint of the lots (k_adjoint.cu, dgpu_api.cu) --------------------
int dgpu_lot_adj_q(dgpu_ctx *ctx, int32_t ngroup, int32_t nlot, const BoxSpec &box, int32_t halved,
                   const PartRef &part, const double2 *fac, const double2 *acsf, const double *g, double scale,
                   float2 *Q, double2 *fsum);
// idx[i] = src[idx[i]] (slot -> source atom), -1 kept
int dgpu_compose_index(dgpu_ctx *ctx, int32_t *idx, const int32_t *src, int64_t n);
// CUDA-core per-atom sums of ntype types with weights Q ([t][box point])
int dgpu_adj_atom_sums(dgpu_ctx *ctx, const BoxSpec &box, const dgpu_grid *grid, int32_t ntype, const int64_t *ts,
                       const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw,
                       const float *w, const int32_t *aidx, const float2 *Q, double *gpos, double *gocc, bool atomic);
int dgpu_lots_adjoint(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *op,
                      const BoxSpec &box, int32_t idim, const double *d_g, double *gpos, double *gocc, double2 *fsum);
int dgpu_adjoint_async(dgpu_ctx *ctx, const FormSpec *d_fs, const BoxSpec &box, int32_t friedel_dim,
                       const dgpu_grid *grid, double diff_scale, int32_t nscat, const int64_t *ts,
                       const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw,
                       const float *w, const int32_t *aidx, const double2 *csf, const double *dsi,
                       const int32_t *istl, const double2 *cfact, const double *it, const double *wt, double *g,
                       double *chi, float2 *Q, double *gpos, double *gocc, bool cuda_core_sums = true);
int dgpu_friedel_test(const dgpu_grid *g, const dgpu_opts *op, int32_t fnum[3]);
// One work item: an atom tile of one type, a column chunk and a row range.
struct AdjItem {
    int64_t a0;          // first padded atom of the tile
    int64_t a_end;       // end of the type's atom range
    int32_t t;           // type (0-based)
    int32_t kc;          // column chunk
    int32_t rt0, rt1;    // row tiles
    int32_t prob = 0;    // problem of the launch (batch member)
    int32_t pad_ = 0;
};

// Geometry of one tensor-core adjoint launch.
struct AdjTcGeom {
    int32_t f[3];
    int32_t ra, rb, ac, fra, frb, ncols;
    int32_t rtiles, nstage;        // row tiles, 32-column stages over all columns
    int64_t rows, pbox;
    int32_t ec;                    // n_c V' scaled by 2^ec
    int64_t sra, srb, sac;         // box-order strides of the row and column axes
    double eck[3], vi[9];
};

// A planned tensor-core adjoint: geometry, work items, number of Q images.
struct AdjTcPlan {
    AdjTcGeom g;
    std::vector<AdjItem> items;
    int64_t nimg = 0;
    int32_t nscat = 0;
};
void dgpu_adjtc_plan(dgpu_ctx *ctx, const BoxSpec &box, const dgpu_grid *grid, int32_t nscat, const int64_t *ts,
                     AdjTcPlan &plan);
// One problem of a tensor-core adjoint launch: geometry, prepared atoms (row
// axes and column axis), Q and its images and scale, gradient outputs.
struct AdjTcProb {
    AdjTcGeom g;
    const uint64_t *ph0, *dra, *drb, *dac;
    const float *w;
    const int32_t *aidx;
    const float2 *Q;
    uint8_t *qimg;
    uint32_t *qmax;
    double *gpos, *gocc;
    int64_t nimg;
    int32_t nscat;
};
void dgpu_adjtc_prob(const AdjTcPlan &plan, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv,
                     const uint64_t *dw, const float *w, const int32_t *aidx, const float2 *Q, uint8_t *img,
                     uint32_t *qmax, double *gpos, double *gocc, AdjTcProb &P);
// Q scales (zeroed by the caller), Q images and the per-atom sums of every
// member in three launches; d_items carry each item's member in prob.
int dgpu_adjtc_members(dgpu_ctx *ctx, const AdjTcProb *d_probs, int32_t nc, int64_t max_nimg, const AdjItem *d_items,
                       int64_t nitems, int32_t *err);
size_t dgpu_adjtc_img_bytes(const AdjTcPlan &plan);
// Enqueue only: Q scale, Q images, main kernel (d_items: the plan's items on
// the device; err: zeroed by the caller, read after the stream).
int dgpu_adjtc_enqueue(dgpu_ctx *ctx, const AdjTcPlan &plan, const AdjItem *d_items, uint8_t *d_img,
                       uint32_t *d_qmax, const uint64_t *ph0, const uint64_t *du, const uint64_t *dv,
                       const uint64_t *dw, const float *w, const int32_t *aidx, const float2 *Q, double *gpos,
                       double *gocc, int32_t *err);
// Tensor-core adjoint sums (k_adjtc.cu): adds the gradient of every prepared
// atom of the ntype type ranges ts (host) to gpos / gocc (device, indexed by
// aidx); Q: nscat * box points, FP32 complex, dense box order.
int dgpu_adjtc_sums(dgpu_ctx *ctx, const BoxSpec &box, const dgpu_grid *grid, int32_t nscat, const int64_t *ts,
                    const uint64_t *ph0, const uint64_t *du, const uint64_t *dv, const uint64_t *dw, const float *w,
                    const int32_t *aidx, const float2 *Q, double *gpos, double *gocc);
void dgpu_batch_free(dgpu_ctx *ctx);

// the whole four_run with device-resident crystal arrays and outputs
int dgpu_stage_crystal(dgpu_ctx *ctx, const dgpu_crystal *cr, dgpu_crystal &dc);
// do_four_filter on the device array dsi(num) when opts->filter is set (k_filter.cu)
int dgpu_four_filter_dev(dgpu_ctx *ctx, const int32_t num[3], const dgpu_opts *op, double *d_dsi);
int dgpu_four_run_dev(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *g, const dgpu_opts *op,
                      double2 *d_csf, double2 *d_acsf, double *d_dsi, dgpu_info *info);

// adjoint.cu / batch.cu ---------------------------------------------------
int dgpu_chi2_grad_impl(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                        const dgpu_opts *op, const double *i_target, const double *weight,
                        double *chi2, double *grad_pos, double *grad_occ, dgpu_info *info, bool device = false);
int dgpu_fill_formspec(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *op,
                       const dgpu_grid *g, FormSpec &fs);

// small helpers -------------------------------------------------------------
static inline int64_t dgpu_cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
