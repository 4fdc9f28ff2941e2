/*
 * springsteel_gpu.h — C ABI of the GB300 transform backend for Springsteel.jl
 * RL / RLZ cylindrical grids.
 *
 * The library owns every device buffer of a grid: the physical array
 * (np × nvars × nslots, column-major, exactly the reference's
 * `grid.physical` layout) and the spectral array (nspec × nvars, the
 * reference's `grid.spectral` layout).  Both stay resident in HBM between
 * calls; host copies happen only through the explicit upload/download entry
 * points.  No C++ exception, torch type or CUDA type crosses this boundary:
 * streams are passed as `void*` (a cudaStream_t, NULL = the grid's own
 * stream) and every entry point returns an `int32_t` status code.
 *
 * Reference boundary replaced (file:line within Springsteel.jl):
 *   createGrid                  src/factory.jl:1104-1143 (RL :646-685, RLZ :688-740)
 *   spectralTransform!(RL)      src/transforms_cylindrical.jl:153-222
 *   gridTransform!(RL)          src/transforms_cylindrical.jl:254-428
 *   spectralTransform!(RLZ)     src/transforms_cylindrical.jl:524-618
 *   gridTransform!(RLZ)         src/transforms_cylindrical.jl:654-853
 *   applyFilter!                src/filtering.jl:262-428
 *   _set_wavenumber_ahat!       src/multipatch_registry.jl:45-62
 *   solve / solve! (Krylov)     src/solver.jl:1002-1009, src/solver_problem.jl:207-222,474-529
 * A handle is not thread-safe (same contract as Fourier1D, src/Fourier.jl:111-112);
 * distinct handles may be used from distinct host threads.
 */
#ifndef SPRINGSTEEL_GPU_H
#define SPRINGSTEEL_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SS_ABI_VERSION 2

/* ---- status codes (no exceptions cross the ABI) ------------------------ */
enum {
    SS_OK = 0,
    SS_BAD_ARG = 1,
    SS_BAD_SHAPE = 2,
    SS_NOT_SPD = 3,          /* mirrors PosDefException, src/banded_cholesky.jl:175-177 */
    SS_UNSUPPORTED_BC = 4,   /* mirrors DomainError, src/Chebyshev.jl:1174 */
    SS_CUDA_ERROR = 5,
    SS_DEVICE_TIMEOUT = 6,
    SS_NAN_DETECTED = 7,     /* reserved: not returned (NaN inputs propagate, as in the reference) */
    SS_NOT_CONVERGED = 8,    /* reserved: ss_solve reports convergence in ss_solve_stats, as the
                                reference's Krylov backend returns its stats instead of throwing */
    SS_OUT_OF_MEMORY = 9,
    SS_NO_DEVICE = 10
};

/* ---- geometry / precision --------------------------------------------- */
enum { SS_GEOM_RL = 1, SS_GEOM_RLZ = 2 };
enum {
    SS_PREC_F64 = 0,         /* every stage in IEEE binary64 (parity with the reference's Float64) */
    SS_PREC_F32_REFINED = 1, /* binary32 bulk; FP64 factor + one FP64-accurate refinement in SA */
    SS_PREC_F64_FAST = 2     /* binary64 data, FFT/DCT bulk in double-float (two binary32, 48-bit
                                significand) on the FP32 pipes: ~2^-48 rounding, so derivative
                                slots carry ~1e-11 relative error instead of ~1e-14 */
};
enum { SS_DTYPE_F64 = 0, SS_DTYPE_F32 = 1 };
enum { SS_QUAD_GAUSS = 0, SS_QUAD_REGULAR = 1 };

/* ---- boundary conditions ---------------------------------------------- */
/* Cubic B-spline BC, the GammaBC kinds of src/CubicBSpline.jl:287-291.
 * alpha/beta carry α1/β1 (rank 1) or α2/β2 (rank 2) of Ooyama (2002) Table 1,
 * exactly as the reference's BC Dicts do (src/CubicBSpline.jl:41-122,
 * converted from BoundaryConditions by src/factory.jl:343-375). */
enum {
    SS_SBC_R0 = 0,        /* NaturalBC                            */
    SS_SBC_RANK1 = 1,     /* α1, β1: R1T0 (-4,-1), R1T1 (0,1), R1T2 (2,-1), Robin */
    SS_SBC_RANK2 = 2,     /* α2, β2: R2T10 (1,-0.5), R2T20 (-1,0)  */
    SS_SBC_PERIODIC = 3,  /* PERIODIC: rankL 1 / rankR 2 wrap-around fold; dense LLᵀ factor
                             (DenseSplineFactor), kept as band + last 3 rows */
    SS_SBC_R3 = 4,        /* ZerosBC                              */
    SS_SBC_R3X = 5        /* FixedBC: R3 fold plus background ahat */
};
typedef struct ss_spline_bc {
    int32_t kind;
    int32_t _pad;
    double alpha;
    double beta;
} ss_spline_bc;

/* Chebyshev BC kinds of src/Chebyshev.jl:949-963 (_bc_type). */
enum { SS_CBC_R0 = 0, SS_CBC_R1T0 = 1, SS_CBC_R1T1 = 2 };

/* ---- grid parameters: mirror of SpringsteelGridParameters ------------- */
/* src/Springsteel.jl:425-465.  Per-variable dictionaries become arrays of
 * nvars entries (variable v = index v-1 of the reference's vars Dict).    */
typedef struct ss_grid_params {
    int32_t geometry;        /* SS_GEOM_RL | SS_GEOM_RLZ                      */
    int32_t precision;       /* SS_PREC_*                                     */
    int32_t num_cells;
    int32_t mubar;           /* default 3                                     */
    int32_t quadrature;      /* SS_QUAD_GAUSS (mubar 1..5) | SS_QUAD_REGULAR  */
    int32_t nvars;
    int32_t kDim;            /* Chebyshev points (RLZ only)                   */
    int32_t b_kDim;          /* 0 → min(kDim, floor((2kDim-1)/3)+1)          */
    int32_t patchOffsetL;    /* (spectralIndexL-1)*mubar                      */
    int32_t _pad0;
    double iMin, iMax;
    double kMin, kMax;
    const double *l_q;                 /* nvars entries, NULL → 2.0             */
    const ss_spline_bc *BCL;           /* nvars entries, NULL → R0              */
    const ss_spline_bc *BCR;           /* nvars entries, NULL → R0              */
    const int32_t *BCB;                /* nvars entries, NULL → SS_CBC_R0       */
    const int32_t *BCT;                /* nvars entries, NULL → SS_CBC_R0       */
    const int32_t *max_wavenumber;     /* nvars entries, NULL → -1 (ring kmax = ri);
                                          RL: one ring set per variable              */
    /* RLZ rings are shared by all variables (src/factory.jl:730-738).  Their
     * kmax is the reference's var_kmax: the "default" entry of max_wavenumber,
     * overridden by each variable's own entry in the order the caller's vars
     * Dict iterates, so the last variable (in that order) that has an entry of
     * its own wins.  A caller that knows which variables have their own entry
     * passes that value in ring_kmax with ring_kmax_set = 1; with
     * ring_kmax_set = 0 the rings take max_wavenumber[nvars-1] (the loop's
     * result when every variable has its own entry). */
    int32_t ring_kmax_set;
    int32_t ring_kmax;
} ss_grid_params;

/* Derived dimensions (src/factory.jl:153-175, 290-298, 658-661, 700-706). */
typedef struct ss_dims {
    int64_t iDim;            /* num_cells*mubar                               */
    int64_t b_iDim;          /* num_cells+3                                   */
    int64_t jDim;            /* Σ_r (4+4 ri)                                  */
    int64_t b_jDim;          /* Σ_r (1+2 ri)                                  */
    int64_t kDim;            /* Chebyshev points (1 for RL)                   */
    int64_t b_kDim;          /* Chebyshev modes (1 for RL)                    */
    int64_t kDim_wn;         /* iDim+patchOffsetL: largest wavenumber         */
    int64_t nvars;
    int64_t nslots;          /* 5 (RL) or 7 (RLZ) derivative slots           */
    int64_t n_physical;      /* rows of physical: jDim (RL), kDim*jDim (RLZ) */
    int64_t n_spectral;      /* rows of spectral: b_kDim*b_iDim*(1+2 kDim_wn) */
    int64_t n_blocks;        /* spectral blocks of b_iDim rows per variable   */
} ss_dims;

typedef struct ss_grid ss_grid;

/* ---- library ----------------------------------------------------------- */
int32_t ss_version(void);
/* Message of the last failing call on this host thread (never NULL). */
const char *ss_last_error_string(void);

/* createGrid (src/factory.jl:1104-1143): builds the FP64 spline templates
 * (P+Q fold and banded Cholesky factor, src/CubicBSpline.jl:733-783 and
 * src/banded_cholesky.jl:99-197), ring/column tables, and allocates the
 * device-resident physical and spectral arrays, zero-filled. */
int32_t ss_grid_create(const ss_grid_params *params, ss_grid **out);
int32_t ss_grid_destroy(ss_grid *grid);
int32_t ss_grid_dims(const ss_grid *grid, ss_dims *out);
/* The grid's own CUDA stream (cudaStream_t), for callers that time or order work. */
int32_t ss_grid_stream(const ss_grid *grid, void **stream_out);
/* Device pointers of grid.physical / grid.spectral (element type: F64 for
 * SS_PREC_F64, F32 for SS_PREC_F32_REFINED). Owned by the grid. */
int32_t ss_grid_device_physical(ss_grid *grid, void **dptr);
int32_t ss_grid_device_spectral(ss_grid *grid, void **dptr);

/* Host ↔ device copies.  `host` is borrowed for the call only; `dtype` is the
 * host element type (converted on the device when it differs from the grid's).
 * slot = 1..nslots copies one derivative slot (np × nvars); slot = 0 copies
 * the whole physical array.  The copy is ordered on `stream`; the call
 * returns after the host buffer may be reused (it synchronizes the stream). */
int32_t ss_upload_physical(ss_grid *grid, const void *host, int32_t dtype,
                           int32_t slot, void *stream);
int32_t ss_download_physical(ss_grid *grid, void *host, int32_t dtype,
                             int32_t slot, void *stream);
int32_t ss_upload_spectral(ss_grid *grid, const void *host, int32_t dtype, void *stream);
int32_t ss_download_spectral(ss_grid *grid, void *host, int32_t dtype, void *stream);

/* spectralTransform!(grid): physical slot 1 → spectral (B-vectors), then the
 * spectral filter epilogue (applyFilter!).  Asynchronous on `stream`. */
int32_t ss_spectral_transform(ss_grid *grid, void *stream);
/* gridTransform!(grid): spectral → all physical slots
 * (RL: f, ∂r, ∂rr, ∂λ, ∂λλ; RLZ adds ∂z, ∂zz).  Asynchronous on `stream`. */
int32_t ss_grid_transform(ss_grid *grid, void *stream);

/* The same transforms with the physical array in host memory, as the
 * reference's spectralTransform!(grid) / gridTransform!(grid) operate on
 * grid.physical (src/transforms_cylindrical.jl:159-222, 259-428).  The grid's
 * rings are split into radial chunks of about equal point counts; each
 * chunk's columns move between host and device on a second stream while the
 * next chunk computes (one strided copy per chunk).  `host_slot1` holds
 * physical slot 1 (np × nvars), `host_all` receives every slot (nslots × nvars
 * × np), both in `dtype`.  from_host returns once the host buffer may be
 * reused (the transform itself stays queued on `stream`); to_host returns with
 * the result in `host_all`.  Page-locked host buffers give full overlap; with
 * a `dtype` other than the grid's the calls copy and transform in sequence. */
int32_t ss_spectral_transform_from_host(ss_grid *grid, const void *host_slot1, int32_t dtype,
                                        void *stream);
int32_t ss_grid_transform_to_host(ss_grid *grid, void *host_all, int32_t dtype, void *stream);

/* Spectral filter weights (applyFilter!, src/filtering.jl:262-428): the host
 * evaluates the reference's _filter_weight per wavenumber (kDim_wn+1 values)
 * and per Chebyshev mode (b_kDim values); NULL clears that filter. */
int32_t ss_grid_set_filter(ss_grid *grid, int32_t var, const double *fourier_w,
                           const double *chebyshev_w);

/* Per-wavenumber R3X background coefficients (src/multipatch_registry.jl:45-62).
 * `block` is the spectral block index (0 = k0, 2k-1 = k real, 2k = k imag,
 * plus z_b*(1+2 kDim_wn) for RLZ); ahat has b_iDim entries.  A grid without
 * any registered ahat uses zeros, as the reference does. */
int32_t ss_grid_set_ahat(ss_grid *grid, int32_t var, int32_t block, const double *ahat);
int32_t ss_grid_clear_ahat(ss_grid *grid);

int32_t ss_grid_synchronize(ss_grid *grid);

/* ---- grid archives: save_grid / load_grid (src/io.jl:410-439) ---------
 * The reference archives params, spectral and physical in a JLD2 file with a
 * format-version tag and rebuilds the grid with createGrid(params).  Without
 * an HDF5/JLD2 library in this build the same components go into a flat
 * little-endian file:
 *   "SSGRID01" (8 bytes: magic and format version 01)
 *   uint32 R, uint32 U        byte counts of the two blocks that follow
 *   R bytes  parameter record: int32 geometry, precision, num_cells, mubar,
 *            quadrature, nvars, kDim, b_kDim, patchOffsetL, ring_kmax_set,
 *            ring_kmax, dtype (SS_DTYPE_*), filtered; double iMin, iMax, kMin,
 *            kMax; per variable: double l_q, BCL and BCR as ss_spline_bc
 *            (int32 kind, int32 0, double alpha, double beta), int32 BCB,
 *            BCT, max_wavenumber, 0; int64 n_spectral, n_physical, nslots,
 *            nvars, nfw, ncw; nfw + ncw doubles of spectral filter weights
 *            (Fourier [var][k ≤ kDim_wn], then Chebyshev [var][z_b])
 *   U bytes  caller block (the host mirror stores its variable names)
 *   spectral (n_spectral × nvars) then physical (n_physical × nvars × nslots),
 *            column-major as grid.spectral / grid.physical, in the grid's
 *            storage type.
 * The arrays stream between HBM and the file through page-locked staging
 * buffers, each chunk's copy overlapping the previous chunk's file write
 * (read, loading).  The R3X background registry is not archived, as in the
 * reference (it is not part of params).  Every call returns once the file
 * or the grid is complete. */
int32_t ss_grid_save(ss_grid *grid, const char *path, const void *user, int64_t user_bytes, void *stream);
/* load_grid: a new grid from the archived parameters and arrays (and filter). */
int32_t ss_grid_load(const char *path, ss_grid **out, void *stream);
/* The archived arrays into an existing grid of the same shape and storage type. */
int32_t ss_grid_load_arrays(ss_grid *grid, const char *path, void *stream);
/* The caller block of an archive: copies min(cap, size) bytes, size in *user_bytes. */
int32_t ss_grid_archive_user(const char *path, void *buf, int64_t cap, int64_t *user_bytes);

/* Tile pipeline (src/tiling.jl).  ss_spline_transform is splineTransform!(
 * sharedSpectral, tile) (RL :1490-1516, RLZ :1862-1892): SAtransform(spline, b)
 * of every wavenumber (and Chebyshev-mode) block of `d_shared_spectral`, a
 * device array in the tile's own spectral layout and storage type (NULL: the
 * tile's spectral array itself, in place), written as spline coefficients a
 * into the tile's spectral array.  The two-argument SAtransform applies no R3X
 * background.  ss_tile_transform is tileTransform!(sharedSpectral, tile,
 * physical, spectral) (RL :1540-1660, RLZ :1915-2046): the tile's spectral
 * array holds coefficients a; SI / SIx / SIxx, the ring inverse with its λ
 * derivatives and, for RLZ, the Chebyshev inverse with its z derivatives fill
 * every physical slot — gridTransform! without its SAtransform!.  Both queue
 * on `stream` (NULL: the grid's stream). */
int32_t ss_spline_transform(ss_grid *grid, const void *d_shared_spectral, void *stream);
int32_t ss_tile_transform(ss_grid *grid, void *stream);

/* regularGridTransform(grid, r_pts, λ_pts[, z_pts]) (src/transforms_cylindrical.jl:929-1020
 * RL, 1168-1287 RLZ): the device-resident spectral array evaluated on the tensor
 * product of n_r radii, n_lam azimuths and (RLZ) n_z levels: per wavenumber (and
 * Chebyshev mode) SAtransform! of the spectral block, SI / SIx / SIxx at r, the
 * Fourier series at λ with the R2HC factor 2 for k ≥ 1, and for RLZ CAtransform!
 * plus the Chebyshev series at z.  Computed in FP64 for every precision; `out`
 * is a host array of n_r·n_lam·n_z rows (r outer, λ then z inner) × nvars × 5 (RL)
 * or 7 (RLZ) slots, column-major like grid.physical.  z_pts is ignored for RL.
 * No R3X background (ahat) is applied: the reference runs SAtransform! on the
 * grid's spline objects, whose ahat is zero unless multipatch coupling set it.
 * Returns once `out` holds the result. */
int32_t ss_regular_grid_transform(ss_grid *grid, const double *r_pts, int32_t n_r, const double *lam_pts,
                                  int32_t n_lam, const double *z_pts, int32_t n_z, double *out, void *stream);

/* evaluate_unstructured(grid, pts; out_of_bounds) (src/interpolation.jl:1735-1850;
 * RL :1628-1656, RLZ :1670-1718): the device-resident spectral array evaluated at
 * npts arbitrary points.  `pts` is column-major npts × 2 (r, λ) or npts × 3
 * (r, λ, z); `out` a host array npts × nvars (column-major).  Per point:
 * SAtransform! of every block (FP64, no R3X background, as regularGridTransform),
 * the 4-tap spline value at r, the Fourier series at λ with the factor 2 for
 * k ≥ 1, and for RLZ CAtransform! plus the Chebyshev series at z (clamped to the
 * column).  Points with r outside [iMin, iMax] (or z outside [kMin, kMax]) get
 * NaN (out_of_bounds 0), make the call fail with SS_BAD_ARG (1), or get `fill` (2).
 * Returns once `out` holds the result. */
int32_t ss_evaluate_unstructured(ss_grid *grid, const double *pts, int64_t npts, double *out,
                                 int32_t out_of_bounds, double fill, void *stream);
/* relocate_grid(grid, (dx, dy); boundary, taper_width) fast path
 * (src/relocation.jl:144-439): every gridpoint (r, λ[, z]) of `target` takes the
 * source's value at the shifted position x = r cos λ + dx, y = r sin λ + dy; then
 * spectralTransform! and gridTransform! of the target.  Points mapped beyond
 * [iMin, iMax] take NaN (boundary 0), the value at the clamped radius (1, :nearest)
 * or the azimuthal mean there (2, :azimuthal_mean); taper_width > 0 blends the
 * last taper_width cells toward the azimuthal mean with a cosine weight.
 * `target` has the source's parameters; target == source relocates in place
 * (relocate_grid!: the source is read before the target is written).  The work
 * is queued on `stream` (NULL: the target's stream) once the source's stream
 * has drained. */
int32_t ss_relocate_grid(ss_grid *target, ss_grid *source, double dx, double dy, int32_t boundary,
                         int32_t taper_width, void *stream);

/* ---- stage timing (the library's own instrumentation; no reference
 * counterpart: the reference times whole calls with BenchmarkTools,
 * bench/bench_grids.jl:20-38).  With profiling on, CUDA events bracket every
 * stage on the stream it runs on; reading synchronizes and returns the
 * accumulated milliseconds and the kernel launches of each stage since the
 * last ss_grid_profile(grid, 1). */
enum {
    SS_STAGE_CHEB_FWD = 0,   /* CBtransform! columns            */
    SS_STAGE_RING_FWD = 1,   /* FBtransform! rings              */
    SS_STAGE_SB = 2,         /* SBtransform! per spectral slot  */
    SS_STAGE_SA_SI = 3,      /* SAtransform! + SI/SIx/SIxx      */
    SS_STAGE_RING_INV = 4,   /* FAtransform! + FI/FIx/FIxx      */
    SS_STAGE_CHEB_INV = 5,   /* CAtransform! + CI/CIx/CIxx      */
    SS_NSTAGES = 6
};
/* ---- many grids: batches under a CUDA graph ----------------------------
 * No single reference counterpart: the reference transforms grids one call
 * at a time (multipatch layers "can be transformed in parallel",
 * src/multipatch.jl:659-661, but run serially :771-784).
 * Without SS_BATCH_FUSED a batch enqueues every grid's own stage launches on
 * forked streams.  With SS_BATCH_FUSED the RL grids' stages are fused across
 * grids: every stage is one launch per shared-memory class (ring stages) or one
 * launch (SB, SA) whose CTAs each run one grid's record from a device work
 * list — 64 uneven grids take about ten launches per round trip instead of
 * ~700; RLZ grids keep their own launch sequences.  Results are bit-identical
 * to single-grid calls.  With use_graph the sequence is captured once into a
 * CUDA graph and replayed (captured again after ss_grid_set_ahat /
 * ss_grid_clear_ahat / ss_grid_set_filter on a member grid).
 * SS_BATCH_AUTOTUNE times candidate tile shapes at creation on the grids' own
 * data: per grid the ring-kernel CTA size (64/128/256) without fusion; with
 * fusion the ring CTA size (128/256) and the items per ring CTA (×1, ×2). */
enum { SS_BATCH_AUTOTUNE = 1, SS_BATCH_FUSED = 2 };
typedef struct ss_batch ss_batch;
int32_t ss_batch_create(ss_grid *const *grids, int32_t n, int32_t flags, ss_batch **out);
int32_t ss_batch_destroy(ss_batch *batch);
/* what: 1 spectralTransform!, 2 gridTransform!, 3 both */
int32_t ss_batch_run(ss_batch *batch, int32_t what, int32_t use_graph, void *stream);
int32_t ss_batch_synchronize(ss_batch *batch);
int32_t ss_batch_ring_threads(const ss_batch *batch, int32_t index, int32_t *fwd, int32_t *inv);
/* Kernel launches of a fused batch for `what` (0 without SS_BATCH_FUSED); its
 * RLZ grids, which keep their own sequences, are not counted. */
int32_t ss_batch_fused_launches(const ss_batch *batch, int32_t what, int32_t *launches);

/* ---- RL multi-patch chain ---------------------------------------------
 * PatchChain(grids) (src/multipatch.jl:825-848) and multiGridTransform!
 * (src/multipatch.jl:769-786) with the per-wavenumber R3X coupling of
 * update_interface! (_rl_kernel!, src/multipatch.jl:417-478).  Grids are
 * given in spatial order; at each interface the coarser patch is primary
 * (NaturalBC side), the finer secondary (FixedBC side); DX ratio 1:1 or 2:1. */
typedef struct ss_chain ss_chain;
int32_t ss_chain_create(ss_grid *const *grids, int32_t n, ss_chain **out);
/* PatchEmbedded(grids) (src/multipatch.jl:891-925): grids nested outermost
 * first, each inner grid 2:1 finer than its parent and FixedBC (R3X) at both
 * ends; multiGridTransform! feeds each inner grid R3X data from its parent
 * at both ends (stacked interfaces at the parent's nodes under the inner
 * boundaries).  Destroyed and run like a chain. */
int32_t ss_chain_create_embedded(ss_grid *const *grids, int32_t n, ss_chain **out);
int32_t ss_chain_destroy(ss_chain *chain);
int32_t ss_multi_grid_transform(ss_chain *chain, void *stream);

/* ---- radial tiles ------------------------------------------------------
 * sumSpectralTile! (set = 0) / the write of setSpectralTile! (set = 1),
 * src/tiling.jl:1040-1330: add (or write) a tile's spectral blocks into the
 * patch at the tile's spectralIndexL; the 3 overlapping coefficients of
 * adjacent tiles form the halo sum.  ss_tile_copy_physical moves the tile's
 * rings of a physical slot (0 = all) between patch and tile (direction 0:
 * patch → tile, 1: tile → patch). */
int32_t ss_tile_sum_spectral(ss_grid *patch, const ss_grid *tile, int32_t set, void *stream);
int32_t ss_tile_copy_physical(ss_grid *patch, ss_grid *tile, int32_t slot, int32_t direction, void *stream);
int32_t ss_grid_zero_spectral(ss_grid *grid, void *stream);

/* ---- forward RL transform that allocates nothing ------------------------
 * No counterpart in the reference.  spectralTransform! of an RL grid in FP64
 * for callers that cannot call cudaMalloc where they transform (inside an
 * open stream capture, under a host framework's own device-memory pool, in a
 * loop that must not enter the allocator).  Input (physical slot 1,
 * n_physical × nvars) and output (spectral, n_spectral × nvars) are the
 * caller's device arrays; the ring-coefficient scratch is a fixed 8 MiB static
 * device array (1,048,576 FP64 values, reserved on every GPU that loads the
 * library until exit), so grids needing more (nvars × Σ(1+2ri) > 1,048,576)
 * get SS_BAD_SHAPE.  d_physical_slot1 must be 16-byte aligned (cudaMalloc
 * pointers are), else SS_BAD_ARG.  The first call on a device resolves the array's device
 * address; make that call before any stream capture.  Calls share the array:
 * calls that overlap on the GPU race.  Asynchronous on `stream`. */
int32_t ss_spectral_transform_noalloc(const ss_grid *grid, const double *d_physical_slot1,
                                      double *d_spectral, void *stream);

int32_t ss_grid_profile(ss_grid *grid, int32_t enable);
int32_t ss_grid_profile_read(ss_grid *grid, double *ms, int64_t *launches);

/* ---- FFT plan inspection (host only: no GPU needed) ----------------------
 * The plan grid creation builds for the complex DFT of length n (n = L/2 of a
 * ring of L = 4 + 4 ri points) in `precision`, with the same limits and tuning
 * overrides (SS_FFT_MAX_PRIME, SS_FFT_RADER, SS_FFT_RADER_PAD).  kind 0: Stockham
 * passes with radices rad[0..nrad) (odd primes above 13 as direct prime passes);
 * 1: one Rader pass for the prime rad[0] = rader_p, then rad[1..nrad), its
 * (p − 1)-point cyclic convolution taken by inner DFTs of length rader_inner —
 * p − 1, or a smooth length ≥ 2p − 3 holding the zero-padded convolution — with
 * radices inner_rad[0..inner_nrad); 2: Bluestein with a smooth length bluestein_m
 * (radices in rad[]). */
typedef struct {
    int32_t n, kind, nrad, rad[24];
    int32_t rader_p, rader_inner, inner_nrad, inner_rad[24];
    int32_t bluestein_m, max_prime, pad_prime, _pad;
} ss_fft_plan_info;
int32_t ss_fft_plan(int32_t n, int32_t precision, ss_fft_plan_info *out);

/* ---- elliptic solve on RL grids ------------------------------------------
 * Replaces SpringsteelProblem(grid, L*u => f; backend, preconditioner) and
 * solve / solve! (src/solver_problem.jl:311-339, :474-529; Krylov backend
 * :99-109, :172-179, :207-222) for L = ∂rr + (1/r)∂r + (1/r²)∂λλ − k²(r) on an
 * RL grid, whose Kron assembly the reference does not support
 * (src/solver.jl:339-363).  Per Fourier wavenumber m the radial Galerkin
 * system G_m x = Γ_m b_m is built from the reference's spline matrices
 * (src/CubicBSpline.jl:1729-1816) and Γ fold (src/solver.jl:721-756), with
 * u'(0) = 0 (m = 0), u(0) = 0 (m ≥ 1) and u(R) = 0.
 * ss_problem_create: k2 = k²(r) at the iDim mish points (native FP64 RL grid).
 * ss_solve: f is read from physical slot 1; u and its derivatives are written
 * to every physical slot (gridTransform! layout); spectral holds the
 * coefficients a.  Methods: direct banded LU, GMRES with the :diag (Jacobi)
 * right preconditioner, flexible GMRES with the learned MLP preconditioner
 * (z = D⁻¹(v + N(v))); its unconverged systems fall back to Jacobi GMRES, then
 * to the direct solve (stats->fallback_systems). */
typedef struct ss_problem ss_problem;
typedef struct ss_mlp ss_mlp;
enum { SS_SOLVER_DIRECT = 0, SS_SOLVER_GMRES_JACOBI = 1, SS_SOLVER_FGMRES_MLP = 2 };
typedef struct {
    int32_t method, systems, converged, max_iterations, fallback_systems, _pad;
    double mean_iterations, max_rel_residual; /* ‖c − G x‖ / ‖c‖ per radial system */
    double ms;                                /* device time of the radial solve stage */
} ss_solve_stats;
int32_t ss_problem_create(ss_grid *grid, const double *k2, ss_problem **out);
int32_t ss_problem_destroy(ss_problem *problem);
int32_t ss_problem_dims(const ss_problem *problem, int32_t *nsys, int32_t *nmax, int32_t *K, int32_t *bandwidth);
int32_t ss_problem_operator_band(const ss_problem *problem, int32_t m, double *band, int32_t *n, int32_t *kl);
int32_t ss_problem_set_mlp(ss_problem *problem, ss_mlp *mlp, int32_t max_wavenumber);
int32_t ss_solve(ss_problem *problem, int32_t method, double tol, int32_t max_iter, int32_t restart,
                 ss_solve_stats *stats, void *stream);
int32_t ss_problem_export(const ss_problem *problem, double *rhs, double *x, double *res, int32_t *iters);
int32_t ss_problem_collect_training(ss_problem *problem, ss_mlp *mlp, const double *points, const double *blobs,
                                   const int32_t *offsets, int32_t nfields, int32_t max_wavenumber);
int32_t ss_problem_collect_random(ss_problem *problem, ss_mlp *mlp, int32_t nsets, uint64_t seed, int32_t smooth,
                                  int32_t max_wavenumber);

/* ---- learned preconditioner network --------------------------------------
 * No reference counterpart (the reference's preconditioners are :none and
 * :diag).  3 dense layers 256 → 256 → 256 → 256, ReLU between, BF16 weights
 * and activations with FP32 accumulation on the tensor cores (tcgen05); FP32
 * master weights and Adam state.  Parameters are W[layer][out][in] and
 * b[layer][out] as FP32 host arrays (3·256·256 and 3·256 values).  Row
 * arrays are rows × 256 FP32.  ss_mlp_gradients takes rows a multiple of
 * 128, the target rows and the used width per row, and returns dL/dW, dL/db
 * of L = (1/rows) Σ_rows Σ_{i<n} (out_i − target_i)². */
typedef struct {
    int32_t epochs, _pad;
    int64_t steps, rows;
    double first_epoch_loss, last_epoch_loss, ms;
} ss_train_stats;
int32_t ss_mlp_create(int32_t device, uint64_t seed, ss_mlp **out);
int32_t ss_mlp_destroy(ss_mlp *mlp);
int32_t ss_mlp_set_params(ss_mlp *mlp, const float *W, const float *b);
int32_t ss_mlp_get_params(const ss_mlp *mlp, float *W, float *b);
int32_t ss_mlp_forward(ss_mlp *mlp, const float *in, float *out, int64_t rows);
int32_t ss_mlp_gradients(ss_mlp *mlp, const float *in, const float *target, const int32_t *n, int64_t rows,
                         float *dW, float *db, double *loss);
int32_t ss_mlp_dataset_rows(const ss_mlp *mlp, int64_t *rows);
int32_t ss_mlp_dataset_clear(ss_mlp *mlp);
int32_t ss_mlp_train(ss_mlp *mlp, int32_t epochs, int32_t batch, float lr, uint64_t seed, ss_train_stats *stats);

#ifdef __cplusplus
}
#endif
#endif /* SPRINGSTEEL_GPU_H */
