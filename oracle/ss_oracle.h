/*
 * ss_oracle.h — FP64 CPU restatement of Springsteel.jl's RL/RLZ transform
 * hot path.  TEST INFRASTRUCTURE ONLY: the oracle is the checker for the
 * GPU library and the timed CPU baseline; no product code links it.
 *
 * Parity pinning: Julia is not installed where this oracle is built, so the
 * reference cannot be executed.  The oracle is pinned against every
 * known-answer test the reference's own test suite holds for this path
 * (test/basis.jl, test/banded_cholesky.jl, test/transforms.jl) and its
 * FFT/DCT against an independent implementation (scipy.fft / pocketfft).
 * Coefficient values beyond those KATs are not pinned by the reference's
 * tests (its tests check round trips only).
 */
#ifndef SS_ORACLE_H
#define SS_ORACLE_H
#include "springsteel_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct or_grid or_grid;

const char *or_last_error(void);
void or_set_threads(int n);

/* grid-level drivers */
int32_t or_grid_create(const ss_grid_params *p, or_grid **out);
void or_grid_destroy(or_grid *g);
int32_t or_grid_dims(const or_grid *g, ss_dims *d);
/* physical: (n_physical, nvars, nslots) column-major; only slot 1 is read. */
int32_t or_spectral_transform(or_grid *g, const double *physical, double *spectral);
/* writes all nslots slots of physical */
int32_t or_grid_transform(or_grid *g, const double *spectral, double *physical);
int32_t or_grid_set_ahat(or_grid *g, int32_t var, int32_t block, const double *ahat);
int32_t or_grid_set_filter(or_grid *g, int32_t var, const double *fw, const double *cw);
/* gridpoints (getGridpoints): out has n_physical rows × (2 RL | 3 RLZ) columns, column-major */
int32_t or_grid_points(const or_grid *g, double *out);
/* mish points of the radial spline, ring angles, Chebyshev levels */
int32_t or_grid_radial_points(const or_grid *g, double *out);   /* iDim */
int32_t or_grid_ring_points(const or_grid *g, int32_t r, double *out);  /* r 1-based, L_r */
int32_t or_grid_column_points(const or_grid *g, double *out);   /* kDim */
/* FP64 band factor rows of a variable's spline (4 × Minterior, column-major) */
int32_t or_grid_factor(const or_grid *g, int32_t var, double *L4, int32_t *n_out);

/* RL multi-patch chain (PatchChain + multiGridTransform!, src/multipatch.jl) */
typedef struct or_chain or_chain;
int32_t or_chain_create(or_grid **grids, int32_t n, or_chain **out);
int32_t or_chain_create_embedded(or_grid **grids, int32_t n, or_chain **out);
void or_chain_destroy(or_chain *c);
/* spectral[i] / physical[i]: arrays of patch i (layouts as or_grid_transform) */
int32_t or_multi_grid_transform(or_chain *c, const double **spectral, double **physical);

/* Elliptic per-wavenumber solve on RL grids (no reference counterpart: built
 * from the reference's B-spline pieces; see ss_oracle.c) */
typedef struct or_elliptic or_elliptic;
int32_t or_elliptic_create(or_grid *g, const double *k2, or_elliptic **out);
void or_elliptic_destroy(or_elliptic *e);
int32_t or_elliptic_operator(const or_elliptic *e, int32_t m, double *G, int32_t *n_out);
int32_t or_elliptic_solve_spectral(const or_elliptic *e, double *spec);
int32_t or_grid_transform_coeffs(or_grid *g, const double *acoef, double *phys);
/* splineTransform! of every spectral block (no R3X background) */
int32_t or_grid_spline_transform(const or_grid *g, const double *shared, double *acoef);

/* ---- 1-D primitives for the known-answer tests -------------------------- */
typedef struct or_spline or_spline;
int32_t or_spline_create(double xmin, double xmax, int32_t num_cells, int32_t mubar,
                         int32_t quadrature, double l_q, const ss_spline_bc *bcl,
                         const ss_spline_bc *bcr, or_spline **out);
void or_spline_destroy(or_spline *s);
int32_t or_spline_info(const or_spline *s, int32_t *bDim, int32_t *mishDim, int32_t *Minterior);
double or_basis(const or_spline *s, int32_t m, double x, int32_t derivative);
int32_t or_spline_mish(const or_spline *s, double *x);
int32_t or_spline_sb(const or_spline *s, const double *u, double *b);
int32_t or_spline_sa(const or_spline *s, const double *b, const double *ahat, double *a);
int32_t or_spline_si(const or_spline *s, const double *a, int32_t derivative, double *u);
int32_t or_spline_si_points(const or_spline *s, const double *a, const double *pts, int32_t n,
                            int32_t derivative, double *u);
int32_t or_spline_gamma_dense(const or_spline *s, double *G);   /* Min × bDim col-major */
int32_t or_spline_pq_dense(const or_spline *s, double *PQ);     /* bDim × bDim col-major */
int32_t or_spline_set_ahat_r3x(const or_spline *s, double u0, double u1, double u2,
                               int32_t side, double *ahat);

/* banded Cholesky (src/banded_cholesky.jl) on a dense symmetric n×n matrix */
int32_t or_band_chol(const double *A, int32_t n, double *L4);
int32_t or_band_solve(const double *L4, int32_t n, const double *b, double *x);

/* Fourier ring (yDim, kmax, bDim, ymin) */
int32_t or_r2hc(const double *x, int32_t n, double *out);
int32_t or_hc2r(const double *x, int32_t n, double *out);
int32_t or_fourier_fb(int32_t yDim, int32_t kmax, int32_t bDim, double ymin,
                      const double *u, double *b);
int32_t or_fourier_fa(int32_t yDim, int32_t kmax, int32_t bDim, double ymin,
                      const double *b, double *a);
int32_t or_fourier_fi(int32_t yDim, int32_t kmax, const double *a, int32_t derivative,
                      double *u);

/* Chebyshev column */
int32_t or_redft00(const double *x, int32_t n, double *out);
int32_t or_cheb_cb(int32_t zDim, int32_t bDim, const double *u, double *b);
int32_t or_cheb_gamma(int32_t zDim, int32_t bcb, int32_t bct, double *G, int32_t *is_matrix);
int32_t or_cheb_ca(int32_t zDim, int32_t bDim, int32_t bcb, int32_t bct, const double *b,
                   double *a);
int32_t or_cheb_ci(int32_t zDim, double zmin, double zmax, const double *a,
                   int32_t derivative, double *u);
int32_t or_cheb_mish(int32_t zDim, double zmin, double zmax, double *z);

#ifdef __cplusplus
}
#endif
#endif
