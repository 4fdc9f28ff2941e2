// ss_kernels.h — launch parameters of the transform kernels (plain PODs
// passed by value to the kernels).
#pragma once

#include <cstdlib>

#include <cuda_runtime.h>

#include "ss_internal.h"
#include "ss_df64.cuh"

namespace ss {

struct RingLaunch {
    const int *ring_list;      // ring indices (0-based r-1) of this launch, largest first
    const RingDesc *rings;     // descriptors; variable v uses rings[v*ring_var_stride + r]
    int64_t ring_var_stride;   // iDim for RL (per-variable kmax), 0 for RLZ (shared rings)
    const FftPlan *plans;
    const void *pool;          // twiddle pool (compute layout)
    const void *phase;         // cos(k ymin), sin(k ymin) pool (compute layout)
    const void *in;
    void *out;
    int64_t in_item_stride;    // RL forward: physical stride between variables (np)
    int64_t frows;             // packed coefficient rows per item: Σ_r (1+2ri)
    int64_t jDim;
    int64_t np;
    int nitems, nvars, bk, rlz;
    int ib;                    // items per CTA (≤ kRingBatchMax): one batched DFT per pass
};
constexpr int kRingBatchMax = 16;
constexpr size_t kRingBatchBytes = 128 * 1024;  // shared-memory budget of one ring batch
// items per CTA for a launch of `nrings` rings of buffer length ≤ `buf` complex
// entries, needing `per_item` shared-memory bytes each: sequences until each of
// the CTA's `threads` has about 16 complex entries per pass, within the
// shared-memory budget, while the launch keeps at least `min_ctas` CTAs (each
// bucket of rings is its own launch).  Measured on the 200-cell FP64 and
// 400-cell binary32 grids (ring_inverse + ring_forward): 42.3 / 77.6 ms at 2
// entries and 64 KB, 42.1 / 76.6 at 4, 41.8 / 74.2 at 8 and 96 KB, 41.2 / 71.7 at
// 16 and 128 KB (the same at 200 KB), 50.5 / 97.5 at 32 and 160 KB.
// (tuning overrides: SS_RING_WORK entries per thread, SS_RING_BATCH_KB budget)
// `fused`: the multi-grid batch planner, which keeps 2 entries per thread and a 64 KB
// budget (its autotuner scales the result by 1, 2 or 4 itself).
inline int ring_batch(size_t per_item, int nitems, int nrings, int min_ctas, int threads, int buf,
                      bool fused = false) {
    static const int work_env = [] {
        const char *e = std::getenv("SS_RING_WORK");
        const int v = e ? std::atoi(e) : 0;
        return (v >= 1 && v <= 64) ? v : 16;
    }();
    static const size_t budget_env = [] {
        const char *e = std::getenv("SS_RING_BATCH_KB");
        const int v = e ? std::atoi(e) : 0;
        return (v >= 16 && v <= 220) ? (size_t)v * 1024 : kRingBatchBytes;
    }();
    const int work = fused ? 2 : work_env;
    const size_t budget = fused ? (size_t)64 * 1024 : budget_env;
    size_t ib = budget / (per_item > 0 ? per_item : 1);
    const size_t by_work = (size_t)(work * threads) / (size_t)(buf > 0 ? buf : 1);
    if (ib > by_work) ib = by_work;
    if (ib < 1) ib = 1;
    if (ib > (size_t)kRingBatchMax) ib = kRingBatchMax;
    if (ib > (size_t)nitems) ib = nitems > 0 ? nitems : 1;
    while (ib > 1 && (long long)nrings * ((nitems + (long long)ib - 1) / (long long)ib) < min_ctas) ib--;
    return (int)ib;
}

// SB projection CTA: 32 slots × kSbOut outputs; its F rows are staged in shared
// memory for mubar ≤ kSbMaxMubar
constexpr int kSbOut = 32;
constexpr int kSbMaxMubar = 4;

struct SbLaunch {
    const void *F;
    void *spec;
    const SplineDev *spl;      // per variable
    const int64_t *fofs;       // packed row start of ring r
    const double *fw, *cw;     // filter weights (per variable), may be null
    int64_t frows, nspec;
    int iDim, b, mubar, pOL, K, nslots_z, bk, filtered;
};

struct SaLaunch {
    const void *spec;
    void *G;
    const SplineDev *spl;
    const int64_t *fofs;
    const double *ahat;        // [v][block][b] or null
    int64_t frows, nspec, nblocks;
    int iDim, b, ld, pOL, nslots_z, bk, nitems;
    int coeffs;                // 1: spectral holds spline coefficients a (skip SAtransform!)
    void *aout;                // non-null: write the coefficients a (storage type, spectral
                               // layout) here and skip SI (splineTransform!)
    float *sx, *sy;            // binary32 grids: the slot-parallel solve's scratch arrays
};

struct ChebLaunch {
    const void *in;
    void *out;
    const ChebDev *cheb;       // per variable
    const RingDesc *rings;     // ring start table (jofs, L)
    const int *col_ring;       // ring index of every column (ring point)
    int64_t jDim, np;
    int64_t col0, col1;        // columns (ring points) [col0, col1) of this launch
    int iDim, bk, nvars;
};

// RL chain coupling (update_interface!, src/multipatch.jl:417-478)
struct ChainLaunch {
    const void *spec;          // primary spectral (P)
    const SplineDev *spl;      // primary splines (per variable)
    double *coupled;           // [v][q][3] coupled border coefficients
    double *state;             // secondary spline-object ahat: [v][3][b_s] (k0, real, imag)
    const double *pstate;      // the primary's spline-object ahat [v][3][b_p] (used when the primary is
                               // itself R3X, an inner grid of an embedded multigrid)
    double *reg;               // secondary per-wavenumber registry: [v][nblocks_s][b_s]
    int64_t nspec_p, nblocks_s;
    int b_p, b_s, ld, nq, nvars, side;  // side of the secondary: 0 left, 1 right
    int bk;                    // Chebyshev levels (RLZ; 1 for RL)
    int zblk_p, zblk_s;        // spectral blocks per level, 1 + 2 kDim_wn, of primary / secondary
    int node[3];
    double C[9];
};
// tile halo sum (sumSpectralTile!, src/tiling.jl:1048-1136)
struct TileLaunch {
    void *patch;               // patch spectral (P)
    const void *tile;          // tile spectral (P)
    int64_t nspec_p, nspec_t;
    int b_p, b_t, blocks_p, blocks_t, bk, nvars, offset, set;
};

// One CTA of a fused multi-grid launch: the launch record it runs (an index
// into the launch's record array in device memory) and its block coordinates
// in the grid of CTAs that record would have on its own.
struct BatchWork {
    int rec;
    int bx, by, bz;
};

void fft_init_constants();

template <typename P>
cudaError_t launch_chain_couple(const ChainLaunch &C, size_t smem, cudaStream_t st);
cudaError_t launch_chain_assemble(const ChainLaunch &C, cudaStream_t st);
template <typename P>
cudaError_t launch_tile_sum(const TileLaunch &T, cudaStream_t st);

// P: storage type of physical/spectral; T: compute type (double | df64 | float)
template <typename P, typename T>
cudaError_t launch_ring_forward(const RingLaunch &L, int nrings, int nitems, size_t smem, int threads,
                                cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_ring_inverse(const RingLaunch &L, int nrings, int nitems, size_t smem, int threads,
                                cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_sb_project(const SbLaunch &S, int nitems, cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_sa_si(const SaLaunch &A, int nitems, size_t smem, cudaStream_t st);
// binary32 grids: slot-parallel solve over the scratch arrays X, Y, each
// nitems × b × nslots_z floats (ss_sa_f32.cu)
template <typename P>
cudaError_t launch_sa_si_f32(const SaLaunch &A, int nitems, float *X, float *Y, cudaStream_t st);
// fused launches over the CTAs of many grids' records (nwork CTAs)
template <typename P, typename T>
cudaError_t launch_ring_forward_fused(const RingLaunch *recs, const BatchWork *work, int nwork, size_t smem,
                                      int threads, cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_ring_inverse_fused(const RingLaunch *recs, const BatchWork *work, int nwork, size_t smem,
                                      int threads, cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_sb_project_fused(const SbLaunch *recs, const BatchWork *work, int nwork, cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_sa_si_fused(const SaLaunch *recs, const BatchWork *work, int nwork, size_t smem, cudaStream_t st);
template <typename P>
cudaError_t launch_sa_si_f32_fused(const SaLaunch *recs, const BatchWork *work, int nwork, cudaStream_t st);
template <typename P, typename T>
cudaError_t launch_cheb_forward(const ChebLaunch &C, size_t smem, cudaStream_t st, int N);
template <typename P, typename T>
cudaError_t launch_cheb_inverse(const ChebLaunch &C, size_t smem, cudaStream_t st, int N);

}  // namespace ss
