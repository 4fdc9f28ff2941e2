// ss_mlp.h — the learned per-wavenumber preconditioner network (internal).
//
// Three dense layers of width 256 (256 → 256 → 256 → 256, ReLU between),
// BF16 weights and activations, FP32 accumulation in tensor memory
// (tcgen05.mma kind::f16, one 128 × 256 tile per CTA).  FP32 master weights and
// Adam moments live beside the BF16 copies for training.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "springsteel_gpu.h"

namespace ss {

constexpr int kMlpWidth = 256;
constexpr int kMlpLayers = 3;
constexpr int kMlpTileM = 128;
constexpr int kMlpChunkK = 64;

// GEMM epilogues: C[M][256] = A[M][K] · B[256][K]ᵀ
enum {
    GEMM_STORE = 0,   // Cf = acc (+ bias)
    GEMM_RELU = 1,    // Z = acc + bias → Cf (optional), relu(Z) → Yb / Yt (bf16)
    GEMM_DRELU = 2,   // G = acc ⊙ [Zin > 0] → Yb / Yt (bf16)
    GEMM_ATOMIC = 3   // Cf += acc (split-K partial sums)
};

struct GemmArgs {
    const __nv_bfloat16 *A;
    const __nv_bfloat16 *B;
    int64_t lda, ldb;      // row strides in elements (K-contiguous rows)
    int M, ksplit;         // rows (multiple of 128); K elements per CTA along gridDim.y
    int mode, _pad;
    const float *bias;     // [256] or null
    float *Cf;             // fp32 output [M][ldc]
    int64_t ldc;
    __nv_bfloat16 *Yb;     // bf16 output [M][256]
    __nv_bfloat16 *Yt;     // bf16 transposed output [256][ldt]
    int64_t ldt;
    const float *Zin;      // [M][256] pre-activations for GEMM_DRELU
    int *err;              // device error word (bounded waits that gave up)
};

int32_t launch_gemm_tc(const GemmArgs &g, int splits, cudaStream_t st);

}  // namespace ss

struct ss_mlp {
    int device = 0;
    uint64_t seed = 0;
    // FP32 masters and Adam moments: [layer][256][256] weights, [layer][256] biases
    float *W = nullptr, *b = nullptr, *mW = nullptr, *vW = nullptr, *mb = nullptr, *vb = nullptr;
    float *dW = nullptr, *db = nullptr;
    __nv_bfloat16 *Wb = nullptr, *Wt = nullptr;  // bf16 [layer][out][in] and [layer][in][out]
    int64_t adam_t = 0;
    // activations for up to cap rows
    int64_t cap = 0;
    __nv_bfloat16 *X0 = nullptr, *X0t = nullptr, *Y1 = nullptr, *Y1t = nullptr, *Y2 = nullptr, *Y2t = nullptr;
    __nv_bfloat16 *G3 = nullptr, *G3t = nullptr, *G2 = nullptr, *G2t = nullptr, *G1 = nullptr, *G1t = nullptr;
    float *Z1 = nullptr, *Z2 = nullptr, *O = nullptr;
    __nv_bfloat16 *T = nullptr;  // targets of the current batch
    int32_t *nrow = nullptr;      // used width per row of the current batch
    float *loss = nullptr;        // [1]
    int *err = nullptr;
    // training set resident in HBM
    int64_t ds_rows = 0, ds_cap = 0;
    __nv_bfloat16 *ds_X = nullptr, *ds_T = nullptr;
    int32_t *ds_n = nullptr, *perm = nullptr;
    int mlp_max_wavenumber = 1 << 30;
    cudaStream_t stream = nullptr;
};

namespace ss {
// forward pass of rows already in mlp->X0 (bf16 [rows][256]); output fp32 into out [rows][256]
int32_t mlp_forward(ss_mlp *m, const __nv_bfloat16 *in, float *out, int64_t rows, cudaStream_t st);
int32_t mlp_reserve(ss_mlp *m, int64_t rows);
int32_t mlp_dataset_reserve(ss_mlp *m, int64_t rows);
}  // namespace ss
