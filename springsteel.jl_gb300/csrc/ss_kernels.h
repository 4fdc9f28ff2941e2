// ss_kernels.h — launch parameters of the transform kernels (plain PODs
// passed by value to the kernels).
#pragma once

#include <cuda_runtime.h>

#include "ss_internal.h"

namespace ss {

struct RingLaunch {
    const int *ring_list;      // ring indices (0-based r-1) of this launch, largest first
    const RingDesc *rings;     // descriptors; variable v uses rings[v*ring_var_stride + r]
    int64_t ring_var_stride;   // iDim for RL (per-variable kmax), 0 for RLZ (shared rings)
    const FftPlan *plans;
    const double2 *pool;       // FP64 twiddle pool
    const double2 *phase;      // cos(k ymin), sin(k ymin) pool
    const void *in;
    void *out;
    int64_t in_item_stride;    // RL forward: physical stride between variables (np)
    int64_t frows;             // packed coefficient rows per item: Σ_r (1+2ri)
    int64_t jDim;
    int64_t np;
    int nitems, nvars, bk, rlz;
};

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
};

struct ChebLaunch {
    const void *in;
    void *out;
    const ChebDev *cheb;       // per variable
    const RingDesc *rings;     // ring start table (jofs) for column → ring lookup
    int64_t jDim, np;
    int iDim, bk, nvars;
};

void fft_init_constants();

template <typename T>
cudaError_t launch_ring_forward(const RingLaunch &L, int nrings, int nitems, size_t smem, cudaStream_t st);
template <typename T>
cudaError_t launch_ring_inverse(const RingLaunch &L, int nrings, int nitems, size_t smem, cudaStream_t st);
template <typename T>
cudaError_t launch_sb_project(const SbLaunch &P, int nitems, cudaStream_t st);
template <typename T>
cudaError_t launch_sa_si(const SaLaunch &P, int nitems, size_t smem, cudaStream_t st);
template <typename T>
cudaError_t launch_cheb_forward(const ChebLaunch &P, size_t smem, cudaStream_t st);
template <typename T>
cudaError_t launch_cheb_inverse(const ChebLaunch &P, size_t smem, cudaStream_t st);

}  // namespace ss
