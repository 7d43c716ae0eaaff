/*
 * discus_gpu.h -- C-ABI of the GB300 Fourier structure-factor library.
 *
 * This is the drop-in boundary for DISCUS's `fourier` -> `run` path
 * (discus/prog/fourier.f90:639-747 -> four_run, discus/prog/fourier_sup.f90:11-323).
 * Every entry point takes plain pointers, sizes and POD structs; nothing
 * here depends on PyTorch.  Arrays follow the Fortran layout DISCUS uses:
 * column-major, first index fastest, so a Fortran caller passes its module
 * arrays (csf, dsi, acsf, cr_pos, cr_iscat, ...) straight through
 * ISO_C_BINDING without copies.
 *
 * Complex arrays are interleaved (re, im) doubles, i.e. Fortran
 * COMPLEX(KIND=8) / C99 double _Complex.
 *
 * Return values: 0 = success, >0 = warning (result valid), <0 = error.
 * Errors map onto DISCUS's ier_num/ier_typ (lib_f90/errlist_mod.f90:48);
 * the mapping is given beside each code.  dgpu_last_error() returns the
 * message that would go into ier_msg.
 */
#ifndef DISCUS_GPU_H
#define DISCUS_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define DGPU_OK                 0
#define DGPU_WARN_NO_CELL       1   /* four_aver: ncell == 0 (ier_num=+1, ER_FOUR)            */
#define DGPU_ERR_ARG          (-1)  /* invalid argument / shape                                */
#define DGPU_ERR_CUDA         (-2)  /* CUDA runtime failure                                     */
#define DGPU_ERR_NOMEM        (-3)  /* device allocation failed                                 */
#define DGPU_ERR_STL_RANGE    (-4)  /* sin(theta)/lambda beyond table (ier_num=-3, ER_FOUR)    */
#define DGPU_ERR_ZERO_INC     (-5)  /* inc>1 with zero increment vector (ier_num=-132, ER_APPL) */
#define DGPU_ERR_UNSUPPORTED  (-6)  /* option not available on this path                       */
#define DGPU_ERR_TIMEOUT      (-7)  /* a bounded device wait gave up                            */
#define DGPU_ERR_CANCELLED   (-14)  /* cancel flag seen (ier_num=-14, ER_COMM, like ier_ctrlc)  */
#define DGPU_ERR_NO_ATOMS   (-198)  /* cr_natoms < 1 (ier_num=-198, ER_APPL)                   */
#define DGPU_ERR_SCRATCH_SIZE (-20) /* request exceeds a fixed scratch capacity                */
#define DGPU_ERR_NO_ACCUM   (-175)  /* accumulation finished without sums (ier_num=-175, ER_APPL) */
#define DGPU_ERR_IO          (-21)  /* a file could not be opened, read or written (ier_num=-2, ER_IO) */

/* ---- tables (discus/prog/discus_config_mod.f90:27-28, diffuse_mod.f90:20-21) */
#define DGPU_CFPKT   9999          /* last index of the sin(theta)/lambda table              */
#define DGPU_CFINC   0.001         /* its step in 1/Angstrom                                 */
#define DGPU_I2PI    65536         /* entries of the phase table cex(0:MASK)                 */

/* ---- phase arithmetic --------------------------------------------------- */
/* REF22: the reference's integer phase.  Per-atom increments are
 * NINT(2^22 * frac(x.v)) and the phase index is (iarg>>6)&0xFFFF, i.e. the
 * phase is truncated to 2^-16 turn (four_strucf_OMP_mod.f90:136-148,163-170).
 * EXACT64: 64-bit fixed-point h.r mod 1 (2^-64 turn resolution).           */
#define DGPU_PHASE_REF22    0
#define DGPU_PHASE_EXACT64  1

/* Form factor: TABLE = cfact(istl) lookup on the 0.001 1/A grid
 * (four_formtab/four_stltab, fourier_sup.f90:2637-2743); ANALYTIC = the
 * same formula evaluated at the exact sin(theta)/lambda of each point.     */
#define DGPU_FORM_TABLE     0
#define DGPU_FORM_ANALYTIC  1

/* Engine for the atom x point sum. */
#define DGPU_ENGINE_AUTO    0   /* TC when the phase mode allows it, else DIRECT */
#define DGPU_ENGINE_DIRECT  1   /* FP32 direct sum on CUDA cores                 */
#define DGPU_ENGINE_TC      2   /* tcgen05 split-precision complex GEMM          */

/* Lots (diffuse_mod.f90:10-12): sub-volumes whose intensities are averaged. */
#define DGPU_LOT_OFF        1   /* whole crystal (0 is read as OFF as well)      */
#define DGPU_LOT_BOX        2   /* ls_xyz box of unit cells                      */
#define DGPU_LOT_ELI        3   /* ellipsoid inscribed in that box               */

/* Operand split of the tensor-core engine. */
#define DGPU_SPLIT_F16      0   /* fp16 hi + fp16 lo, 3 products  (default)      */
#define DGPU_SPLIT_BF16     1   /* bf16 hi + bf16 lo, 3 products                 */

typedef struct dgpu_ctx dgpu_ctx;   /* opaque: device, stream, cached buffers */

/* The crystal: crystal_mod (discus/prog/crystal_mod.f90:25-138). */
typedef struct dgpu_crystal {
    int64_t        natoms;     /* cr_natoms                                              */
    const double  *pos;        /* cr_pos(3,natoms): pos[3*i+k], lattice units            */
    const int32_t *iscat;      /* cr_iscat(1,:): type 1..nscat, 0 = VOID (skipped)       */
    const float   *atom_occ;   /* per-atom occupancy weight, NULL = 1 (not in DISCUS)    */
    int32_t        nscat;      /* cr_nscat                                               */
    int32_t        ncatoms;    /* cr_ncatoms, sites per unit cell                        */
    int32_t        icc[3];     /* cr_icc, unit cells per axis                            */
    double         dim0[3];    /* cr_dim0(:,1), lower corner of the crystal              */
    double         rten[9];    /* cr_rten(3,3), reciprocal metric tensor, column-major   */
    const double  *scat;       /* cr_scat(11,0:nscat): scat[11*t+0]=c, [11*t+2i-1]=a_i,
                                  [11*t+2i]=b_i (i=1..5)                                  */
    const double  *occ;        /* cr_occ(0:nscat)                                        */
    const double  *dw;         /* cr_dw(0:nscat), isotropic B in A^2                     */
    const double  *delfr;      /* cr_delfr(0:nscat), f', used only when ano != 0         */
    const double  *delfi;      /* cr_delfi(0:nscat), f'', used only when ano != 0        */
    /* Anisotropic ADPs (crystal_mod.f90:47,94,103,118).  is_anis == 0: the
       crystal is isotropic (cr_dw in cfact) and ianis/anis_full are ignored.
       is_anis != 0: cfact carries no Debye-Waller term and each (type, ADP)
       group is multiplied by exp(-2 pi^2 h^T (a*_i a*_j U_ij) h) at every
       point (four_dbwtab, fourier_sup.f90:2747-2855) when ldbw is set.      */
    int32_t        is_anis;    /* cr_is_anis                                             */
    int32_t        nanis;      /* cr_nanis                                               */
    const int32_t *ianis;      /* cr_iscat(3,:), ADP type 1..nanis of each atom          */
    const double  *anis_full;  /* cr_anis_full(6,nanis): U11,U22,U33,U23,U13,U12 in A^2  */
    double         ar[3];      /* cr_ar, reciprocal cell lengths in 1/A                  */
    double         dim_lo[3];  /* cr_dim(:,1), lower corner of the atom positions; lots
                                  use it to place atoms stored after the
                                  ncatoms*icc(1)*icc(2)*icc(3) block (fourier_sup.f90:1886-1899) */
    const int32_t *isym;       /* cr_iscat(2,:), the symmetry operation that generated
                                  each atom; read only with DISCAMB form factors     */
} dgpu_crystal;

/* DISCAMB aspherical form factors (discus_discamb.f90:15-26): the tables
 * discamb_read (:136-400) reads and discamb_set_form_tsc (:447-546) expands
 * per symmetry operation, supplied by the caller as `cr_scat` is.  Type t
 * (1..nscat) has nsymm[t-1] tables, one per symmetry operation number listed
 * in isymm (disc_list(t)%isymm(1:), types one after another); table m holds
 * complex values over integer h in [-maxhkl, maxhkl] per axis, element
 * (h,k,l) at form_tsc[2*(m*T + (h+mh0) + (2mh0+1)((k+mh1) + (2mh1+1)(l+mh2)))]
 * (real, imaginary), T = (2mh0+1)(2mh1+1)(2mh2+1).  four_run then sums the
 * atoms per (type, symmetry, ADP type) group (fourier_sup.f90:166-193,
 * four_getatm_discamb :2259-2436) and multiplies each group's sum at grid
 * point h by table(nint(h)) and, with ldbw, by the group's four_dbw term
 * (tcsf_form_discamb, fourier_form.f90:63-102).                             */
typedef struct dgpu_discamb {
    int32_t        maxhkl[3];
    const int32_t *nsymm;      /* nscat values                                        */
    const int32_t *isymm;      /* sum(nsymm) symmetry operation numbers, 0..192       */
    const double  *form_tsc;   /* sum(nsymm) tables, host memory                      */
} dgpu_discamb;

/* The reciprocal-space grid: diffuse_mod eck/vi/inc (diffuse_mod.f90:100,113-119). */
typedef struct dgpu_grid {
    double  eck[12];   /* eck(3,4): corners ll, lr, ul, tl, column-major         */
    double  vi[9];     /* vi(3,3): abscissa, ordinate, top increment vectors    */
    int32_t inc[3];    /* points per axis (num)                                 */
} dgpu_grid;

/* Fourier menu state that four_run reads (fourier_reset.f90:42-101 defaults). */
typedef struct dgpu_opts {
    int32_t lxray;          /* 1: X-ray Gaussian form factors; 0: neutron, c only    */
    int32_t power;          /* diff_power: number of Gaussians, 4 or 5              */
    int32_t ano;            /* anomalous scattering                                 */
    int32_t ldbw;           /* 'temp use': isotropic Debye-Waller in cfact          */
    int32_t friedel;        /* four_friedel: halve the grid when allowed            */
    double  fave;           /* 'set aver': 0 off, 1 all cells; 0<fave<1 needs cells  */
    const uint8_t *aver_cells; /* cell selection for 0<fave<1, cells(csize1,csize2,csize3)
                                  (csize = icc for a periodic crystal), drawn by the
                                  caller's ran1 stream (fourier_sup.f90:1235-1241)   */
    double  diff_scale;     /* intensity scale (fourier_sup.f90:281-282), default 1  */
    int32_t phase;          /* DGPU_PHASE_*                                         */
    int32_t form;           /* DGPU_FORM_*                                          */
    int32_t engine;         /* DGPU_ENGINE_*                                        */
    int32_t split;          /* DGPU_SPLIT_* (tensor-core engine)                    */
    int32_t tc_tile_n;      /* tensor-core N tile in points (0 = autotuned)         */
    int32_t tc_kslice;      /* atoms per tensor-core work item (0 = autotuned)      */
    int32_t tc_flush;       /* atoms per drain of the main TMEM accumulator (0 = 128) */
    volatile int32_t *cancel; /* optional host flag polled between atom types      */
    /* Lots (fourier.f90:467-531, diffuse_mod.f90:75-82, defaults fourier_reset.f90:44-51). */
    int32_t ilots;          /* DGPU_LOT_*                                           */
    int32_t nlots;          /* number of lots (ignored with lot_all)                */
    int32_t ls_xyz[3];      /* lot size in unit cells, 1..icc (default 5)           */
    int32_t lot_all;        /* every origin of csize once, in DISCUS order          */
    int32_t lperiod;        /* periodic crystal: csize = icc, else max(1,icc-ls+1)  */
    const int32_t *lot_origins; /* lbeg(3,nlots), 1-based origin cells 1..csize, drawn
                                  by the caller's ran1 stream as four_ranloc does
                                  (fourier_sup.f90:2513-2530); unused with lot_all  */
    int32_t tc_vimg;        /* tensor-core V operand: 0 auto (images when each is
                               re-read by 4+ row tiles), 1 images, -1 in-kernel  */
    int32_t tc_wait_us;     /* tensor-core type sums: limit of one wait of a warp
                               for another's progress, microseconds (0: 2 s).  A
                               wait that runs out stops the kernel, which waits
                               for its own MMAs and copies, frees its tensor
                               memory and returns DGPU_ERR_TIMEOUT; the context
                               stays usable.  For tests of that path.            */
    const dgpu_discamb *discamb; /* DISCAMB form factors instead of the independent
                               atom model (diff_table RAD_DISC, fourier_sup.f90:
                               107-118); NULL = off.  Not with <F> subtraction:
                               the reference multiplies its lattice sum by the
                               table of type 0, which does not exist.            */
    /* Lanczos filter of dsi at the end of four_run (do_four_filter,
       fourier_sup.f90:284-290,1646-1803; 'set filter,lanczos', fourier.f90:
       1156-1186; defaults fourier_reset.f90:101-105).                          */
    int32_t filter;         /* DGPU_FILTER_OFF / DGPU_FILTER_LANCZOS               */
    int32_t filter_width;   /* four_width m: window |q-g| < m (default 4)           */
    double  filter_damp;    /* four_damp: sinc(pi (q-g) damp) (default 0.5)          */
    double  filter_scale;   /* four_rscale (default 1; other values UNSUPPORTED)     */
} dgpu_opts;

#define DGPU_FILTER_OFF      0
#define DGPU_FILTER_LANCZOS  1

/* What four_run reports besides the arrays. */
typedef struct dgpu_info {
    int32_t fnum[3];           /* points computed (Friedel-reduced)                   */
    int32_t friedel_dim;       /* 0 none, else the halved axis (diff_idim)            */
    int32_t lmn[6];            /* fourier_lmn output                                  */
    double  off_shift[9];      /* fourier_lmn output                                  */
    int32_t ncell;             /* cells used for <F>                                  */
    int32_t engine_used;       /* DGPU_ENGINE_DIRECT or DGPU_ENGINE_TC                */
    int64_t pairs;             /* atom x full-grid-point pairs of the type sums       */
    int64_t pairs_aver;        /* atom/cell x point pairs of <F>                      */
    double  res[7];            /* four_qinfo: res[0]=6, diffumin, diffumax, diffuave,
                                  diffusig, braggmin, braggmax (fourier_sup.f90:2930-2936) */
    double  kernel_ms;         /* device time of the atom x point sums               */
    double  total_ms;          /* device time of the whole call                      */
    int32_t tc_config[4];      /* tensor-core engine: column axis, N tile, main
                                  accumulator buffers, atoms per K slice (-1 if unused) */
    int64_t refined;           /* points recomputed exactly on CUDA cores after a
                                  tensor-core run with <F> subtracted: those where
                                  |<F>|^2 > 64 N<|f|^2>, whose F - <F> cancels
                                  more digits than the FP32 type sums carry      */
} dgpu_info;

/* ---- context ------------------------------------------------------------ */
int  dgpu_ctx_create(int device, dgpu_ctx **out);
int  dgpu_ctx_destroy(dgpu_ctx *ctx);
const char *dgpu_last_error(const dgpu_ctx *ctx);
void dgpu_default_opts(dgpu_opts *opts);   /* fourier_reset.f90 defaults + engine AUTO */

/* ---- the whole path ----------------------------------------------------- */
/* Replaces four_run (discus/prog/fourier_sup.f90:11-323) for the independent
 * atom model: tables, Friedel reduction, <F> (four_aver), the loop over lots,
 * the per-type (isotropic) or per-(type, ADP) (anisotropic) structure-factor
 * sums, csf -= acsf, dsi += |csf|^2, lot normalisation, mirror, scale and
 * four_qinfo statistics.  Host buffers: csf/acsf are complex num(1)*num(2)*num(3),
 * dsi is real.  acsf may be NULL.  With lots, csf is that of the last lot.  */
int dgpu_four_run(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                  const dgpu_opts *opts, double *csf, double *acsf, double *dsi,
                  dgpu_info *info);

/* Same as dgpu_four_run, but cr->pos, cr->iscat, cr->atom_occ and the three
 * output arrays are DEVICE pointers (resident in HBM); the small per-type
 * arrays (scat, occ, dw, delfr, delfi) stay on the host.                   */
int dgpu_four_run_device(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                         const dgpu_opts *opts, double *d_csf, double *d_acsf,
                         double *d_dsi, dgpu_info *info);

/* ---- per-type drop-in ----------------------------------------------------- */
/* Replaces four_strucf (discus/prog/four_strucf_OMP_mod.f90:19-68) as the
 * RMC/stack/powder callers use it: the reference's REF22 phase of nxat atoms
 * xat(nxat,3) on the grid num with increments uin/vin/win, corner lmn and
 * off_shift, then (if cfact != NULL) tcsf *= cfact(istl) on fnum
 * (fourier_form.f90:147-177).  tcsf is complex num(1)*num(2)*num(3); points
 * outside fnum are zero.  cfact is complex(0:CFPKT) for this type, istl is
 * int32 num(1)*num(2)*num(3).  Host buffers.                                */
int dgpu_four_strucf(dgpu_ctx *ctx, const double *xat, int64_t nxat,
                     const double uin[3], const double vin[3], const double win[3],
                     const double off_shift[9], const int32_t lmn[6],
                     const int32_t num[3], const int32_t fnum[3],
                     const double *cfact, const int32_t *istl, double *tcsf);

/* Allocation-free variant of dgpu_four_strucf for callers that cannot
 * allocate device memory: reverse Monte Carlo loops re-evaluating a few atoms
 * per move (where a cudaMalloc/cudaFree per call would synchronise the
 * device), code living inside another allocator's memory budget, or code
 * enqueuing on a stream it does not own.  It has no counterpart in the
 * reference.  All pointers named d_* are device memory, arrays as in
 * dgpu_four_strucf (cfact = complex(0:CFPKT) or NULL, istl int32 num points,
 * tcsf complex num points); stream is a cudaStream_t (NULL = default stream)
 * of the device that is current at the call (another device's stream:
 * DGPU_ERR_ARG).  The call only enqueues work: the result is ready when the
 * stream reaches it.  An istl value outside 0..CFPKT gives a NaN at that
 * point (no table read).
 * Working memory is one fixed __device__ array per GPU (8.5 MiB, held until
 * process exit): at most 131072 atoms and 262144 computed points
 * (fnum(1)*fnum(2)*fnum(3)) per call, else DGPU_ERR_SCRATCH_SIZE.  Calls that
 * overlap on the GPU share that array and race; calls on one stream are safe.
 * The first call on a device looks the array up (cudaGetSymbolAddress) and
 * should come before any stream capture; it is looked up again when a later
 * call finds another CUDA context current on that device (after
 * cudaDeviceReset, say).                                                     */
int dgpu_four_strucf_noalloc(void *stream, const double *d_xat, int64_t nxat,
                             const double uin[3], const double vin[3], const double win[3],
                             const double off_shift[9], const int32_t lmn[6],
                             const int32_t num[3], const int32_t fnum[3],
                             const double *d_cfact, const int32_t *d_istl, double *d_tcsf);

/* ---- tables (each replaces one reference routine; host buffers) ---------- */
/* fourier_lmn (discus/prog/fourier_lmn_mod.f90:4-280), host quad precision. */
int dgpu_fourier_lmn(const double eck[12], const double vi[9], const int32_t inc[3],
                     int32_t lmn[6], double off_shift[9]);
/* four_stltab (fourier_sup.f90:2637-2687), computed on the device.         */
int dgpu_four_stltab(dgpu_ctx *ctx, const dgpu_grid *grid, const double rten[9],
                     int32_t *istl);
/* four_formtab (fourier_sup.f90:2691-2743): cfact(0:CFPKT, 1:nscat), complex. */
int dgpu_four_formtab(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *opts,
                      double *cfact);
/* Per-atom REF22 increments iincu,iincv,iincw,jincu,jincv,jincw
 * (four_strucf_OMP_mod.f90:136-148) as int64 [6][nxat], computed on the device. */
int dgpu_four_increments(dgpu_ctx *ctx, const double *xat, int64_t nxat,
                         const double uin[3], const double vin[3], const double win[3],
                         const double off_shift[9], int64_t *inc_out);

/* ---- epilogue steps of four_run after the sums --------------------------- */
/* four_weight (fourier_sup.f90:1428-1643): dsi3d = dsi, except that with
 * fave == 0 the Bragg points (h, k, l all within 1e-4 of integers) are
 * divided by scalef = ncells * voxel / V*, the number of unit cells (or lot
 * cells) along the grid's dimensions times the reciprocal volume of one grid
 * step over that of the cell, when |scalef - 1| > 1e-5.  cr supplies icc and
 * rten; opts supplies fave and the lot size.  Host arrays of num points.   */
int dgpu_four_weight(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                     const dgpu_opts *opts, const double *dsi, double *dsi3d);
/* Same with device arrays; enqueued on the context's stream. */
int dgpu_four_weight_device(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                            const dgpu_opts *opts, const double *d_dsi, double *d_dsi3d);

/* four_accumulate (fourier_sup.f90:3784-3840): sums of csf and dsi over
 * several runs, kept in the context's device memory.  mode (diffuse_mod.f90:
 * 154-157): INIT clears the sums, ACCUM adds csf/dsi (host arrays of the
 * grid), FINISHED writes the sums into csf/dsi and clears them (with
 * fave < 0 the Bragg points first take the mean of their grid neighbours,
 * four_fill_csf/four_fill_dsi :3844-4044), SINGLE does nothing unless
 * symm != 0.  symm != 0 (four_symm): SINGLE and FINISHED first average
 * csf/dsi over the point-group operations set by dgpu_set_symmetry
 * (four_symm_csf/four_symm_dsi, :4048-4290), then fill the Bragg points.    */
#define DGPU_ACCUM_INIT      (-1)
#define DGPU_ACCUM_SINGLE      0
#define DGPU_ACCUM_ACCUM       1
#define DGPU_ACCUM_FINISHED    2
/* The point-group operations of four_symm: spc_mat(1:3,1:3,i), i = 1..nops
 * with nops = spc_n / n_center (n_center from the first letter of
 * cr_spcgr: P 1, A/B/C/I 2, F 4, R with cr_syst 6 3; fourier_sup.f90:
 * 4102-4118), column-major 3x3 each, operation 1 the identity.  Integer
 * matrices of determinant +-1 (DGPU_ERR_ARG otherwise).  Kept in the
 * context; nops = 0 clears them.  Replaces the reference's read of the
 * global spc_mat / spc_n (wyckoff_mod).                                      */
int dgpu_set_symmetry(dgpu_ctx *ctx, int32_t nops, const double *mats);

int dgpu_four_accumulate(dgpu_ctx *ctx, int32_t mode, int32_t symm, const dgpu_grid *grid, double fave,
                         double *csf, double *dsi);

/* do_four_filter (fourier_sup.f90:1646-1803) on a host array dsi(num)
 * (Fortran order), in place: with filter = LANCZOS the field is convolved
 * with the windowed sinc kernel the reference builds (do_lanczos_{1,2,3}d_fft,
 * lib_f90/lib_lanczos.f90), circularly, with the index shifts of its FFT
 * maps (lib_f90/map_1dtofield.f90), and scaled to the input's sum.  3D grids
 * with an extent <= 2 width + 1 are filtered in 2D slices as the reference
 * does; planes must span axes 1-2 and lines axis 1 (where the reference
 * reads outside its kernel table otherwise: DGPU_ERR_UNSUPPORTED, as for a
 * filtered extent below 2 width + 3, or 2 width + 4 when even).
 * dgpu_four_run applies it to dsi before the statistics; this entry is for
 * the caller's dsi3d copy (fourier_sup.f90:287-290, fave == 0).            */
int dgpu_four_filter(dgpu_ctx *ctx, const int32_t num[3], const dgpu_opts *opts, double *dsi);

/* ---- output values ------------------------------------------------------- */
/* qval (discus/prog/qval.f90:65-290): the value the output menu writes at a
 * grid point, from the arrays of the last four_run.  value (qval.f90:3-21):  */
#define DGPU_VAL_INTEN     1   /* dsi, or |acsf|^2 with laver                    */
#define DGPU_VAL_AMPLI     2   /* |F|                                            */
#define DGPU_VAL_PHASE     3   /* atan2(Im F, Re F) in degrees, 0 for F = 0      */
#define DGPU_VAL_REAL      4
#define DGPU_VAL_IMAG      5
#define DGPU_VAL_RANPH     6   /* phase at integer hkl, else (r - 0.5)*360       */
#define DGPU_VAL_SQ        7   /* S(Q) = I/<f>^2/N + 1 - exp(-Q^2 <u^2>)         */
#define DGPU_VAL_F2AVER    9   /* <f^2>, from cfact without Debye-Waller/occ     */
#define DGPU_VAL_FAVER2   10   /* <f>^2                                          */
#define DGPU_VAL_FAVER    11   /* <f>                                            */
#define DGPU_VAL_IQ       13   /* I/N                                            */
#define DGPU_VAL_F2AVERB  17   /* the same three from cfact (Debye-Waller, occ)  */
#define DGPU_VAL_FAVER2B  18
#define DGPU_VAL_FAVERB   19
/* out receives num(1)*num(2)*num(3) values; F = csf, or acsf with laver != 0.
 * csf/acsf/dsi are host arrays as dgpu_four_run returns them (acsf may be NULL
 * without laver); rand (RANPH only) holds one value in [0,1) per point, drawn
 * by the caller's ran1 stream.  The per-type sums use cr (types, scattering
 * tables, dw), opts (lxray, power, ano, ldbw) and istl(i, j, 1) / istl(i, 1, 1)
 * exactly as qval indexes them.  PDF values (14-16) are DGPU_ERR_UNSUPPORTED. */
int dgpu_qval(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid, const dgpu_opts *opts,
              int32_t value, int32_t laver, const double *csf, const double *acsf, const double *dsi,
              const double *rand, double *out);

/* calc_hkl (discus/prog/fourier_sup.f90:3230-3549), the numeric core: F at
 * a list of integer reflections hkl(3,nrefl).  four_run runs on the integer
 * box from min(0, h_min) to max(0, h_max) (same for k, l) with vi = identity
 * and the caller's crystal and options; for every reflection
 *   |F| = |csf(h,k,l)| / (icc1 icc2 icc3),
 *   ext = (1 / (1 + 0.001 exti |F|^2 rlambda^3 / sin(2 asin(0.5 rlambda dstar))))^(1/4)
 *   with dstar the length of (h,k,l) in the reciprocal metric,
 *   icalc = (|F| ext)^2 scale,  sigi = sqrt(|icalc|),  phase = atan2d(Im, Re) of csf;
 * the reflection 0 0 0 gives zeros.  Host arrays of nrefl values; phase may be
 * NULL.  Reading and writing the HKLF4/CIF files stays with the caller.      */
int dgpu_calc_hkl(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *opts, const int32_t *hkl,
                  int64_t nrefl, double scale, double exti, double rlambda, double *icalc, double *sigi,
                  double *phase);

/* ---- output files --------------------------------------------------------- */
/* calc_hkl with its files (fourier_sup.f90:3230-3549): reads the reflections
 * of infile -- HKLF4 records (3I4,2F8.2), a line starting with '#', '!' or
 * 'd' is DGPU_ERR_ARG; or a CIF whose _refln_ loop starts with index_h,
 * index_k, index_l and carries at most three values before its last column
 * -- runs dgpu_calc_hkl on them and writes calcfile (HKLF4: h k l icalc sigi,
 * (3I4,2F8.2); CIF: h k l and the row's values with _refln_F_squared_calc
 * replaced by icalc, (3I4,3F12.2)) and the list file, calcfile with its
 * trailing "hkl" replaced by "fcf" or ".fcf" appended (3I4,2F10.2,F7.2:
 * h k l, sqrt|Iobs| (HKLF4) or h (CIF), sqrt|icalc|, phase).  The reflection
 * 0 0 0 is written as zeros to calcfile only.                                */
#define DGPU_HKL_CIF    1
#define DGPU_HKL_HKLF4  4
int dgpu_calc_hkl_files(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_opts *opts, const char *infile,
                        const char *calcfile, int32_t style, double scale, double exti, double rlambda);

/* The writers of the output menu, host-side (format = the reference's ityp):
 *   STANDARD  do_output ityp 0 (graphic.f90:1704-1847): 1D "x y" records
 *             (2(1X,E12.5)); 2D a NIPL file (header lines, npkt1 npkt2,
 *             x/y ranges, rows of 5(1X,E12.5), output_save_file_2d,
 *             discus_s_out_file.f90:124-260); 3D one such file per layer,
 *             named path.PART_nnnn;
 *   GNUPLOT   ityp 3: 2D rows "h_abs h_ord value h_third" (4(1X,E12.5)), a
 *             blank record after each row; nothing for 1D data;
 *   HKLF4, LIST5, LIST9  ityp 6-8: reflections with INT(h) /= 0 0 0, the
 *             amplitude per unit cell, extinction and scale (valmax) as
 *             graphic.f90:1598-1702,1893-1991 and the 1D rows :2012-2109;
 *   NIPL3D    ityp 9: list-directed inc and ranges, then the rows of the
 *             first layer (the reference closes the file after it);
 *   VTK       vtk_write (vtk_mod.f90:4-35): STRUCTURED_POINTS header and the
 *             values (the caller's dsi, nvalues of them) as E13.6E2;
 *   MRC       mrc_write (lib_f90/mrc_data.f90:19-139): 1024-byte header,
 *             3072-byte extended header, REAL(4) map, i fastest;
 *   XPLOR     xplor_write (discus_xplor.f90:16-139), path gets ".xplor"
 *             unless it ends in it; the output range (lrange ...) applies.
 * values: qval's array for `value` over inc (Fortran order, nvalues =
 * inc1 inc2 inc3; VTK: dsi).  ampl/phase: qval's arrays for values 2 and 3
 * (SHELX formats; HKLF4 needs no phase on 2D/3D grids).  PGM, PPM and
 * postscript are disabled in the reference (error -6), NeXus needs a
 * library this build does not link: DGPU_ERR_UNSUPPORTED.
 *   HDF5      gen_hdf5_write (lib_f90/hdf_write.f90:12-326), the "Yell 1.0"
 *             file of the 'hdf5' format (graphic.f90:604-635): data =
 *             values x scale with dimensions (inc1, inc2, inc3), the third
 *             fastest, the largest scaled to valmax when valmax > 0;
 *             format, is_direct (value 14 or 15), lower_limits, step_sizes,
 *             step_sizes_abs/_ord/_top, unit_cell (a0, win), PROGRAM.
 *             Written without an HDF5 library, from the file format
 *             specification.                                               */
#define DGPU_OUT_STANDARD  0
#define DGPU_OUT_GNUPLOT   3
#define DGPU_OUT_HKLF4     6
#define DGPU_OUT_LIST5     7
#define DGPU_OUT_LIST9     8
#define DGPU_OUT_NIPL3D    9
#define DGPU_OUT_VTK      11
#define DGPU_OUT_MRC      12
#define DGPU_OUT_HDF5     13
#define DGPU_OUT_XPLOR    14

typedef struct dgpu_nipl {            /* write_discus_nipl_header (discus_nipl_header.f90:5-172)  */
    int64_t natoms;                   /* cr_natoms                                              */
    int32_t nscat, ncatoms;           /* cr_nscat, cr_ncatoms                                   */
    const char *at_lis;               /* cr_at_lis(0:nscat): 4 characters each, blank padded    */
    const int64_t *amount;            /* cr_amount(0:nscat)                                     */
    const double *dw;                 /* cr_dw(0:nscat)                                         */
    int32_t four_last;                /* |four_last| < 3: FOURIER section; < 0: with lots       */
    int32_t radiation;                /* diff_radiation: 1 xray, 2 neutron, 3 electron          */
    double rlambda;
    const char *lambda;               /* wave-length symbol, "" when given as a number          */
    int32_t ldbw, ano;
    int32_t inc[3];                   /* the Fourier's inc, eck(3,4), vi(3,3) (column-major)    */
    double eck[12];
    double vi[9];
} dgpu_nipl;

typedef struct dgpu_output {
    int32_t format;                   /* DGPU_OUT_*                                             */
    int32_t value;                    /* qval code of values (XPLOR title, 1D SHELX rows)       */
    int32_t inc[3];                   /* out_inc                                                */
    int32_t extr_abs, extr_ord, extr_top;   /* 1..3                                             */
    double eck[12];                   /* out_eck(3,4), column-major                             */
    double vi[9];                     /* out_vi(3,3), column-major                              */
    double rten[9];                   /* cr_rten: |h| for the extinction and the header angles  */
    double ar[3], wrez[3];            /* cr_ar, cr_wrez (MRC, XPLOR)                            */
    int32_t icc[3];                   /* cr_icc: the amplitude per unit cell                    */
    int32_t lrange, lcenter, lpixel;  /* XPLOR range: out_lrange, out_lcenter, out_lpixel       */
    int32_t center[3], pixel[3];      /* out_center, out_pixel                                  */
    char quad[4];                     /* out_quad ('l', 'r' or blank per axis)                  */
    double valmax;                    /* SHELX scale: NINT -1 by F(000), -2 by the largest
                                         reflection, > 0 this factor, else 1;
                                         HDF5: > 0 the largest value written                    */
    double f000;                      /* qval(1,1,1,2) of the run at 0 0 0 (valmax -1)          */
    double exti, rlambda;             /* diff_exti, rlambda                                     */
    const char *name;                 /* cr_name (XPLOR title)                                  */
    const dgpu_nipl *nipl;            /* header of STANDARD 2D/3D files; NULL: no header lines  */
    double out_fac;                   /* out: the SHELX scale applied                           */
    double a0[3], win[3];             /* cr_a0, cr_win (HDF5 unit_cell)                         */
    double scale;                     /* out_scale (HDF5: values x scale; 0 reads as 1)         */
} dgpu_output;

int dgpu_output_write(const char *path, dgpu_output *out, const double *values, const double *ampl,
                      const double *phase, int64_t nvalues);

/* ---- powder pattern, "complete" mode -------------------------------------- */
/* powder_complete (discus/prog/powder.f90:1829-2593) with pow_four_mode =
 * fourier: the structure factor four_run_powder (powder.f90:3143-3206) along
 * every (h, k) rod inside the d* <= ds_max sphere, binned onto the Q scale by
 * powder_split (powder.f90:2975-3008).
 *
 *   h:  ih = h_start..h_end, h_start = ano ? -int(a0(1) ds_max / dH) : 0,
 *       hh = ih dH + shift(1);
 *   k:  the range of the circle d* = ds_max in the plane hh as do_proj
 *       (metric.f90:337-548) returns it for "hh,0,0, 1,0,0, rdrr" and
 *       "0,1,0, 1,0,0, ddrr" (its parallel part is v / (u.v) / |v|^2, which
 *       is what the reference enumerates), k = 0.. in the plane h = 0 without ano;
 *   l:  int(l_lo / dL) .. int(l_hi / dL), l_lo/l_hi the roots of
 *       d*(hh, kk, l) = ds_max, from l = 0 on the rod h = k = 0 without ano;
 *   every point with pow_l_all, or with h, k or l more than 0.51 steps from
 *       an integer, and qmin <= Q = 2 pi d* <= qmax + deltaq adds
 *       |F|^2 x calc_preferred (powder.f90:3332-3376) to pow_qsp(itth1) and
 *       pow_qsp(itth1 + 1), split linearly, itth1 = int((Q - qmin) / deltaq);
 *   without ano the pattern is doubled at the end.
 * F is four_run's sum over all atoms and types: no <F> subtraction, no lots,
 * no diff_scale; cfact from (lxray, power, ano, ldbw) of opts, and, as
 * four_run_powder passes is_anis = .false. while four_formtab drops the
 * isotropic term of an anisotropic crystal, no Debye-Waller factor at all for
 * an anisotropic crystal.  The device evaluates F on h-slabs of the (h, k, l)
 * box that holds the rods (EXACT64 phases, either engine) and bins only the
 * rod points.  Not covered: stacking-fault crystals (scale_diffuse,
 * set_scale_mode) and the structure transformation trans_to_short: dL must
 * be the smallest of the three steps (else DGPU_ERR_UNSUPPORTED).  The
 * form-factor averages pow_f2aver/pow_faver2 are computed afterwards, in
 * phases_set_mod, and stay with the caller.                                 */
#define DGPU_PREF_NONE      0
#define DGPU_PREF_RIETVELD  1   /* g2 + (1 - g2) exp(g1 alpha^2), alpha in degrees */
#define DGPU_PREF_MARCH     2   /* g2 + (1 - g2) ((g1 cos alpha)^2 + sin^2 alpha / g1)^(-3/2) */
typedef struct dgpu_powder {
    double  hkl_del[3];    /* pow_hkl_del: dH, dK, dL                                */
    double  hkl_shift[3];  /* pow_hkl_shift                                          */
    double  a0[3];         /* cr_a0, A (pow_hkl_max = a0 ds_max)                      */
    double  gten[9];       /* cr_gten, direct metric tensor, column-major            */
    double  ds_max;        /* pow_ds_max, 1/A                                         */
    double  qmin;          /* pow_qmin, 1/A                                           */
    double  qmax;          /* pow_qmax                                               */
    double  deltaq;        /* pow_deltaq                                             */
    int32_t l_all;         /* pow_l_all: integer (Bragg) points are binned as well   */
    int32_t pref_type;     /* DGPU_PREF_*                                            */
    double  pref_hkl[3];   /* pow_pref_hkl                                           */
    double  pref_g1;       /* pow_pref_g1                                            */
    double  pref_g2;       /* pow_pref_g2                                            */
    int32_t slabs;         /* h-slabs the device evaluates, 0 = automatic; no
                              counterpart in the reference                        */
} dgpu_powder;

typedef struct dgpu_powder_info {
    int32_t n_pkt;         /* pow_npkt: pow_qsp has n_pkt + 1 values, itth 0..n_pkt  */
    int32_t nslab;         /* device grids evaluated                                 */
    int64_t rods;          /* (h, k) rods of powder_complete                         */
    int64_t rod_points;    /* points on those rods (four_run_powder's points)        */
    int64_t grid_points;   /* points evaluated on the device                         */
    int64_t binned;        /* points added to pow_qsp                                */
    int64_t pairs;         /* atom x evaluated-point pairs                           */
    double  kernel_ms;     /* device time of the atom x point sums                   */
    double  total_ms;      /* device time of the whole call                          */
} dgpu_powder_info;

/* n_pkt = NINT((qmax + deltaq - qmin) / deltaq) + 2 (powder.f90:1957), or <0. */
int32_t dgpu_powder_npkt(const dgpu_powder *pw);
/* pow_qsp: host array of n_pkt + 1 doubles (overwritten).  info may be NULL. */
int dgpu_powder_complete(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_powder *pw,
                         const dgpu_opts *opts, double *pow_qsp, dgpu_powder_info *info);

/* ---- adjoint: chi^2 and its gradient ------------------------------------- */
/* chi2 = sum_h w(h) (I(h) - I_target(h))^2 over the full grid, I = diff_scale*|csf|^2
 * as dgpu_four_run computes it (EXACT64 phase, ANALYTIC or TABLE form).
 * grad_pos is d chi2 / d cr_pos (3*natoms, lattice units), grad_occ is
 * d chi2 / d atom_occ (natoms).  VOID atoms get zero.  Host buffers; the
 * gradient arrays may be NULL.  Used by RMC/REFINE in place of finite
 * differences (refine/prog/refine_run.f90:491-759).                         */
int dgpu_chi2_grad(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                   const dgpu_opts *opts, const double *i_target, const double *weight,
                   double *chi2, double *grad_pos, double *grad_occ, dgpu_info *info);

/* Same as dgpu_chi2_grad with everything per atom and per point resident in
 * HBM: cr->pos, cr->iscat, cr->atom_occ (and cr->ianis), d_i_target,
 * d_weight, d_grad_pos and d_grad_occ are DEVICE pointers; chi2 is a host
 * double.  For optimisation loops that keep the crystal on the GPU (the
 * torch.autograd wrapper): no per-atom or per-point host copy per call.     */
int dgpu_chi2_grad_device(dgpu_ctx *ctx, const dgpu_crystal *cr, const dgpu_grid *grid,
                          const dgpu_opts *opts, const double *d_i_target, const double *d_weight,
                          double *chi2, double *d_grad_pos, double *d_grad_occ, dgpu_info *info);

/* ---- batched population --------------------------------------------------- */
/* Many independent crystals (a DIFFEV population, diffev/prog/with_mpi.f90:281-510
 * farms one four_run per member) in one persistent launch.  dsi[c] receives
 * crystal c's intensity (host buffer, num(1)*num(2)*num(3) of grids[c]);
 * when i_target != NULL, chi2[c] and the gradients of member c are returned
 * as well (grad_pos[c], grad_occ[c] may be NULL).  The population graph
 * covers EXACT64 phases on the tensor-core engine without <F>, lots,
 * DISCAMB or anomalous scattering; with any of those (or the CUDA-core
 * engine) the members run one after another through dgpu_four_run and
 * dgpu_chi2_grad, with the same outputs, and dgpu_batch_last_ms is the wall
 * time of that loop.                                                        */
int dgpu_batch_run(dgpu_ctx *ctx, int32_t ncrystal, const dgpu_crystal *crystals,
                   const dgpu_grid *grids, const dgpu_opts *opts,
                   double *const *dsi,
                   const double *const *i_target, const double *const *weight,
                   double *chi2, double *const *grad_pos, double *const *grad_occ);

/* Device time of the last dgpu_batch_run call's graph launch, ms. */
double dgpu_batch_last_ms(const dgpu_ctx *ctx);

/* Nodes (kernels, copies, memsets) and kernel nodes of the graph the last
 * dgpu_batch_run call launched (kernels may be NULL); 0 when it ran member
 * by member.  Measurement aid; no counterpart in the reference. */
int64_t dgpu_batch_graph_nodes(const dgpu_ctx *ctx, int64_t *kernels);

/* Device time of the tensor-core type-sum kernel alone in the last
 * dgpu_four_run / dgpu_four_run_device call that used the tensor-core
 * engine, ms (CUDA events on the context's stream around that launch).
 * Measurement aid; no counterpart in the reference. */
double dgpu_tc_last_kernel_ms(const dgpu_ctx *ctx);

#ifdef __cplusplus
}
#endif
#endif /* DISCUS_GPU_H */
