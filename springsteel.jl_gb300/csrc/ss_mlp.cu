// ss_mlp.cu — BF16 tensor-core MLP (tcgen05.mma, accumulators in tensor
// memory) for the learned preconditioner: inference, backward pass and Adam.
//
// One GEMM kernel serves every product of the network:
//     C[M][256] = A[M][K] · B[256][K]ᵀ      (A, B bf16, K-contiguous rows)
// A CTA owns a 128 × 256 FP32 accumulator (256 TMEM columns).  K advances in
// chunks of 64: 128 threads stage the A (16 KB) and B (32 KB) chunks into
// shared memory in the no-swizzle K-major core-matrix layout (8 rows × 16 B
// per core matrix; core matrices along K 128 B apart, 8-row groups 1 KB
// apart), one thread issues four tcgen05.mma (M=128, N=256, K=16) per chunk
// and commits them to an mbarrier, while the block stages the next chunk into
// the other buffer.  The epilogue reads TMEM with tcgen05.ld (warp w owns
// lanes 32w..32w+31 = rows) and applies bias/ReLU/ReLU'/split-K atomics.
// Every wait is bounded (about two seconds); a wait that gives up records an
// error word, waits again (bounded) for the MMAs in flight, frees TMEM and
// returns.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "ss_internal.h"
#include "ss_mlp.h"

using namespace ss;

#define CUDA_TRY(expr)                                                                      \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            set_error("%s failed: %s", #expr, cudaGetErrorString(_e));                      \
            return (_e == cudaErrorMemoryAllocation) ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;   \
        }                                                                                   \
    } while (0)

namespace ss {

constexpr int kGemmThreads = 128;
constexpr uint32_t kChunkA = kMlpTileM * kMlpChunkK * 2;   // 16 KB
constexpr uint32_t kChunkB = kMlpWidth * kMlpChunkK * 2;   // 32 KB
constexpr size_t kGemmSmem = 2 * (kChunkA + kChunkB) + 1024;  // + alignment slack
constexpr long long kWaitNs = 2000000000LL;

// instruction descriptor, kind::f16: D = F32 (bits 4-5), A = B = BF16 (bits
// 7-9, 10-12), both K-major (bits 15, 16 clear), N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t kIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(kMlpWidth >> 3) << 17) |
                            ((uint32_t)(kMlpTileM >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4 (bits 0-13), leading byte
// offset >> 4 (16-29), stride byte offset >> 4 (32-45), version 1 (46-47),
// base offset 0, no swizzle (layout type 0 in bits 61-63)
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

__device__ __forceinline__ long long global_ns() {
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// bounded wait for the phase with the given parity; false after ~2 s
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    const uint32_t a = smem_u32(bar);
    const long long t0 = global_ns();
    while (true) {
        uint32_t ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (global_ns() - t0 > kWaitNs) return false;
    }
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float *v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
        "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// stage rows [row0, row0 + rows) × K chunk [k0, k0 + 64) into core-matrix layout
__device__ __forceinline__ void stage_chunk(uint8_t *dst, const __nv_bfloat16 *src, int64_t ld, int64_t row0,
                                            int rows, int64_t k0) {
    const int pieces = rows * 8;
    for (int p = threadIdx.x; p < pieces; p += kGemmThreads) {
        const int row = p >> 3, kg = p & 7;
        const uint4 v = __ldg(reinterpret_cast<const uint4 *>(src + (row0 + row) * ld + k0 + kg * 8));
        *reinterpret_cast<uint4 *>(dst + (((row >> 3) * 8 + kg) * 128 + (row & 7) * 16)) = v;
    }
}

__global__ void __launch_bounds__(kGemmThreads) gemm_tc_kernel(GemmArgs g) {
    extern __shared__ __align__(1024) uint8_t smem_dyn[];
    __shared__ __align__(8) uint64_t bars[2];
    __shared__ uint32_t tmem_slot;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
    uint8_t *const sA0 = base, *const sB0 = base + 2 * kChunkA;  // buffer b: sA0 + b·kChunkA, sB0 + b·kChunkB
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)blockIdx.x * kMlpTileM;
    const int64_t kbeg = (int64_t)blockIdx.y * g.ksplit;
    const int nchunks = g.ksplit / kMlpChunkK;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kMlpWidth)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;

    bool ok = true;
    uint32_t phase0 = 0u, phase1 = 0u;
    stage_chunk(sA0, g.A, g.lda, m0, kMlpTileM, kbeg);
    stage_chunk(sB0, g.B, g.ldb, 0, kMlpWidth, kbeg);
    for (int c = 0; c < nchunks; c++) {
        const int bf = c & 1;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(sA0 + bf * kChunkA), b0 = smem_u32(sB0 + bf * kChunkB);
#pragma unroll
            for (int s = 0; s < kMlpChunkK / 16; s++) {
                const uint64_t ad = smem_desc(a0 + s * 256, 128, 1024);
                const uint64_t bd = smem_desc(b0 + s * 256, 128, 1024);
                const uint32_t acc = (c > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bars[bf]))
                         : "memory");
        }
        if (c + 1 < nchunks) {
            const int nb = (c + 1) & 1;
            if (c >= 1) {  // the MMAs of chunk c − 1 read buffer nb
                uint32_t &ph = nb ? phase1 : phase0;
                ok = mbar_wait(&bars[nb], ph) && ok;
                ph ^= 1u;
            }
            stage_chunk(sA0 + nb * kChunkA, g.A, g.lda, m0, kMlpTileM, kbeg + (int64_t)(c + 1) * kMlpChunkK);
            stage_chunk(sB0 + nb * kChunkB, g.B, g.ldb, 0, kMlpWidth, kbeg + (int64_t)(c + 1) * kMlpChunkK);
        }
    }
    {
        const int lb = (nchunks - 1) & 1;
        const uint32_t ph = lb ? phase1 : phase0;
        bool done = mbar_wait(&bars[lb], ph);
        if (!done) done = mbar_wait(&bars[lb], ph);  // one more bounded wait for MMAs in flight
        ok = ok && done;
    }
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    if (!ok && lane == 0) atomicExch(g.err, 1);

    // epilogue: thread (warp w, lane l) owns row m0 + 32w + l
    const int64_t row = m0 + warp * 32 + lane;
    for (int cc = 0; cc < kMlpWidth / 32; cc++) {
        float v[32];
        tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(cc * 32), v);
        if (!ok) continue;
        const int c0 = cc * 32;
        if (g.mode == GEMM_STORE) {
            float *o = g.Cf + row * g.ldc + c0;
#pragma unroll
            for (int i = 0; i < 32; i += 4) {
                float4 q = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                if (g.bias) {
                    q.x += g.bias[c0 + i]; q.y += g.bias[c0 + i + 1];
                    q.z += g.bias[c0 + i + 2]; q.w += g.bias[c0 + i + 3];
                }
                *reinterpret_cast<float4 *>(o + i) = q;
            }
        } else if (g.mode == GEMM_ATOMIC) {
            float *o = g.Cf + row * g.ldc + c0;
#pragma unroll
            for (int i = 0; i < 32; i++) atomicAdd(o + i, v[i]);
        } else {
            __nv_bfloat16 y[32];
            if (g.mode == GEMM_RELU) {
#pragma unroll
                for (int i = 0; i < 32; i++) {
                    const float z = v[i] + (g.bias ? g.bias[c0 + i] : 0.f);
                    v[i] = z;
                    y[i] = __float2bfloat16(z > 0.f ? z : 0.f);
                }
                if (g.Cf) {
                    float *o = g.Cf + row * g.ldc + c0;
#pragma unroll
                    for (int i = 0; i < 32; i += 4)
                        *reinterpret_cast<float4 *>(o + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
                }
            } else {  // GEMM_DRELU
                const float *zi = g.Zin + row * kMlpWidth + c0;
#pragma unroll
                for (int i = 0; i < 32; i++) y[i] = __float2bfloat16(zi[i] > 0.f ? v[i] : 0.f);
            }
            if (g.Yb) {
                uint4 *o = reinterpret_cast<uint4 *>(g.Yb + row * kMlpWidth + c0);
                const uint4 *s = reinterpret_cast<const uint4 *>(y);
#pragma unroll
                for (int i = 0; i < 4; i++) o[i] = s[i];
            }
            if (g.Yt) {
#pragma unroll
                for (int i = 0; i < 32; i++) g.Yt[(int64_t)(c0 + i) * g.ldt + row] = y[i];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMlpWidth) : "memory");
}

// ---------------------------------------------------------------- fused inference
// All three layers in one launch: a CTA keeps its 128 input rows (64 KB bf16)
// in shared memory, stages each layer's 256 × 256 weights (128 KB), issues 16
// tcgen05.mma (K = 16 each) into TMEM, and writes the ReLU'd bf16 activations
// back over its input tile for the next layer.  256 threads: warps w and w + 4
// share TMEM lanes 32(w mod 4)… and split the 256 columns in halves.
constexpr int kInferThreads = 256;
constexpr uint32_t kTileX = kMlpTileM * kMlpWidth * 2;     // 64 KB
constexpr uint32_t kTileW = kMlpWidth * kMlpWidth * 2;     // 128 KB
constexpr size_t kInferSmem = kTileX + kTileW + 1024;

// full-K (256) core-matrix layout: 8-row groups 4 KB apart, core matrices along K 128 B apart
__device__ __forceinline__ uint32_t cm_offset(int row, int col) {
    return (uint32_t)((((row >> 3) * 32 + (col >> 3)) * 128) + (row & 7) * 16 + (col & 7) * 2);
}

// rows × 256 bf16 into the core-matrix layout by 16-byte cp.async pieces, every
// piece of the thread in flight at once (completed by cp_async_wait_all)
__device__ __forceinline__ void stage_full_async(uint8_t *dst, const __nv_bfloat16 *src, int64_t row0, int rows) {
    const int pieces = rows * 32;
    for (int p = threadIdx.x; p < pieces; p += kInferThreads) {
        const int row = p >> 5, kg = p & 31;
        const __nv_bfloat16 *g = src + (row0 + row) * kMlpWidth + kg * 8;
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst + cm_offset(row, kg * 8))), "l"(g)
                     : "memory");
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

__global__ void __launch_bounds__(kInferThreads) mlp_infer_kernel(const __nv_bfloat16 *in, const __nv_bfloat16 *Wb,
                                                                  const float *bias, float *out, int *err) {
    extern __shared__ __align__(1024) uint8_t smem_dyn[];
    __shared__ __align__(8) uint64_t bar;
    __shared__ uint32_t tmem_slot;
    uint8_t *base = reinterpret_cast<uint8_t *>((reinterpret_cast<uintptr_t>(smem_dyn) + 1023) & ~uintptr_t(1023));
    uint8_t *sX = base, *sW = base + kTileX;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int64_t m0 = (int64_t)blockIdx.x * kMlpTileM;
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_slot)),
                     "r"(kMlpWidth)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_slot;
    stage_full_async(sX, in, m0, kMlpTileM);
    stage_full_async(sW, Wb, 0, kMlpWidth);
    bool ok = true;
    uint32_t phase = 0u;
    const int row = (warp & 3) * 32 + lane, cbase = (warp >> 2) * (kMlpWidth / 2);
    for (int l = 0; l < kMlpLayers; l++) {
        // this layer's weights (and, first, the input rows) have landed; the
        // generic-proxy writes (cp.async, the previous epilogue's activations)
        // are made visible to the tensor core's async proxy
        cp_async_wait_all();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (threadIdx.x == 0 && ok) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            const uint32_t a0 = smem_u32(sX), b0 = smem_u32(sW);
#pragma unroll
            for (int s = 0; s < kMlpWidth / 16; s++) {
                const uint64_t ad = smem_desc(a0 + s * 256, 128, 4096);
                const uint64_t bd = smem_desc(b0 + s * 256, 128, 4096);
                const uint32_t acc = s > 0 ? 1u : 0u;
                asm volatile(
                    "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                    " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                    "l"(ad), "l"(bd), "r"(kIdesc), "r"(acc)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                             smem_u32(&bar))
                         : "memory");
        }
        bool done = mbar_wait(&bar, phase);
        if (!done) done = mbar_wait(&bar, phase);
        ok = ok && done;
        phase ^= 1u;
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        // the MMAs have read sW: the next layer's weights stream in under the epilogue
        if (ok && l + 1 < kMlpLayers) stage_full_async(sW, Wb + (size_t)(l + 1) * kMlpWidth * kMlpWidth, 0, kMlpWidth);
        const float *bl = bias + l * kMlpWidth;
        for (int cc = 0; cc < kMlpWidth / 64; cc++) {
            const int c0 = cbase + cc * 32;
            float v[32];
            tmem_ld32(tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0, v);
            if (!ok) continue;
            if (l + 1 < kMlpLayers) {
                __align__(16) __nv_bfloat16 y[32];
#pragma unroll
                for (int i = 0; i < 32; i++) {
                    const float z = v[i] + bl[c0 + i];
                    y[i] = __float2bfloat16(z > 0.f ? z : 0.f);
                }
#pragma unroll
                for (int q = 0; q < 4; q++)
                    *reinterpret_cast<uint4 *>(sX + cm_offset(row, c0 + 8 * q)) = reinterpret_cast<const uint4 *>(y)[q];
            } else {
                float *o = out + (m0 + row) * kMlpWidth + c0;
#pragma unroll
                for (int i = 0; i < 32; i += 4)
                    *reinterpret_cast<float4 *>(o + i) =
                        make_float4(v[i] + bl[c0 + i], v[i + 1] + bl[c0 + i + 1], v[i + 2] + bl[c0 + i + 2],
                                    v[i + 3] + bl[c0 + i + 3]);
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();  // activations written, TMEM read: the next layer may overwrite both
    }
    if (!ok && lane == 0) atomicExch(err, 1);
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kMlpWidth) : "memory");
}

int32_t launch_gemm_tc(const GemmArgs &g, int splits, cudaStream_t st) {
    if (g.M <= 0 || g.M % kMlpTileM || g.ksplit <= 0 || g.ksplit % kMlpChunkK || splits < 1) {
        set_error("GEMM shape M=%d ksplit=%d not tiled by 128 x 64", g.M, g.ksplit);
        return SS_BAD_SHAPE;
    }
    if ((g.lda % 8) || (g.ldb % 8) || ((uintptr_t)g.A & 15) || ((uintptr_t)g.B & 15)) {
        set_error("GEMM operands must be 16-byte aligned rows");
        return SS_BAD_SHAPE;
    }
    static bool attr = false;
    if (!attr) {
        CUDA_TRY(cudaFuncSetAttribute(gemm_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGemmSmem));
        attr = true;
    }
    dim3 grid(g.M / kMlpTileM, splits);
    gemm_tc_kernel<<<grid, kGemmThreads, kGemmSmem, st>>>(g);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

// ---------------------------------------------------------------- small kernels
__global__ void f32_to_bf16_rows(const float *in, __nv_bfloat16 *out, __nv_bfloat16 *outT, int64_t rows,
                                 int64_t ldt) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= rows * kMlpWidth) return;
    const int64_t r = i / kMlpWidth, c = i % kMlpWidth;
    const __nv_bfloat16 v = __float2bfloat16(in[i]);
    out[i] = v;
    if (outT) outT[c * ldt + r] = v;
}

__global__ void zero_rows_bf16(__nv_bfloat16 *p, int64_t n) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = __float2bfloat16(0.f);
}

// loss = (1/B) Σ_rows Σ_{i<n} (o − t)²; dO = (2/B)(o − t) → G / Gᵀ (bf16)
__global__ void mse_loss_kernel(const float *O, const __nv_bfloat16 *T, const int32_t *nrow, int64_t B, int64_t ldt,
                                __nv_bfloat16 *G, __nv_bfloat16 *Gt, float *loss) {
    const int64_t r = blockIdx.x;
    const int c = threadIdx.x;
    const int n = nrow[r];
    float d = 0.f;
    if (c < n) d = O[r * kMlpWidth + c] - __bfloat162float(T[r * kMlpWidth + c]);
    const __nv_bfloat16 gv = __float2bfloat16(2.f * d / (float)B);
    G[r * kMlpWidth + c] = gv;
    Gt[(int64_t)c * ldt + r] = gv;
    float s = d * d;
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float red[8];
    if ((c & 31) == 0) red[c >> 5] = s;
    __syncthreads();
    if (c == 0) {
        float t = 0.f;
        for (int i = 0; i < kMlpWidth / 32; i++) t += red[i];
        atomicAdd(loss, t / (float)B);
    }
}

// db[c] = Σ_r Gt[c][r]
__global__ void colsum_kernel(const __nv_bfloat16 *Gt, int64_t ldt, int64_t B, float *db) {
    const int c = blockIdx.x;
    float s = 0.f;
    for (int64_t r = threadIdx.x; r < B; r += blockDim.x) s += __bfloat162float(Gt[(int64_t)c * ldt + r]);
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    __shared__ float red[32];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int i = 0; i < (int)(blockDim.x >> 5); i++) t += red[i];
        db[c] = t;
    }
}

__global__ void adam_kernel(float *W, float *b, const float *dW, const float *db, float *mW, float *vW, float *mb,
                            float *vb, __nv_bfloat16 *Wb, __nv_bfloat16 *Wt, float lr, float c1, float c2) {
    const int64_t nW = (int64_t)kMlpLayers * kMlpWidth * kMlpWidth;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    if (i < nW) {
        const float gr = dW[i];
        const float m = b1 * mW[i] + (1.f - b1) * gr, v = b2 * vW[i] + (1.f - b2) * gr * gr;
        mW[i] = m;
        vW[i] = v;
        const float p = W[i] - lr * (m / c1) / (sqrtf(v / c2) + eps);
        W[i] = p;
        const int64_t l = i / (kMlpWidth * kMlpWidth), o = (i / kMlpWidth) % kMlpWidth, k = i % kMlpWidth;
        const __nv_bfloat16 pb = __float2bfloat16(p);
        Wb[i] = pb;
        Wt[l * kMlpWidth * kMlpWidth + k * kMlpWidth + o] = pb;
    } else if (i < nW + kMlpLayers * kMlpWidth) {
        const int64_t j = i - nW;
        const float gr = db[j];
        const float m = b1 * mb[j] + (1.f - b1) * gr, v = b2 * vb[j] + (1.f - b2) * gr * gr;
        mb[j] = m;
        vb[j] = v;
        b[j] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
    }
}

__global__ void refresh_bf16_kernel(const float *W, __nv_bfloat16 *Wb, __nv_bfloat16 *Wt) {
    const int64_t nW = (int64_t)kMlpLayers * kMlpWidth * kMlpWidth;
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nW) return;
    const int64_t l = i / (kMlpWidth * kMlpWidth), o = (i / kMlpWidth) % kMlpWidth, k = i % kMlpWidth;
    const __nv_bfloat16 pb = __float2bfloat16(W[i]);
    Wb[i] = pb;
    Wt[l * kMlpWidth * kMlpWidth + k * kMlpWidth + o] = pb;
}

// batch rows from the resident training set by a permutation
__global__ void gather_rows_kernel(const __nv_bfloat16 *X, const __nv_bfloat16 *T, const int32_t *n,
                                   const int32_t *perm, int64_t B, int64_t ldt, __nv_bfloat16 *X0,
                                   __nv_bfloat16 *X0t, __nv_bfloat16 *Tb, int32_t *nb) {
    const int64_t r = blockIdx.x;
    const int c = threadIdx.x;
    const int64_t src = perm[r];
    const __nv_bfloat16 x = X[src * kMlpWidth + c];
    X0[r * kMlpWidth + c] = x;
    X0t[(int64_t)c * ldt + r] = x;
    Tb[r * kMlpWidth + c] = T[src * kMlpWidth + c];
    if (c == 0) nb[r] = n[src];
}

// ---------------------------------------------------------------- host helpers
static int32_t dalloc(void **p, size_t bytes) {
    if (cudaMalloc(p, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc(%zu) failed", bytes);
        return SS_OUT_OF_MEMORY;
    }
    cudaMemset(*p, 0, bytes ? bytes : 16);
    return SS_OK;
}

static int32_t check_err(ss_mlp *m) {
    int e = 0;
    CUDA_TRY(cudaMemcpy(&e, m->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (e) {
        CUDA_TRY(cudaMemset(m->err, 0, sizeof(int)));
        set_error("tensor-core GEMM wait gave up");
        return SS_DEVICE_TIMEOUT;
    }
    return SS_OK;
}

int32_t mlp_reserve(ss_mlp *m, int64_t rows) {
    rows = (rows + kMlpTileM - 1) / kMlpTileM * kMlpTileM;
    if (rows <= m->cap) return SS_OK;
    void *bufs[] = {m->X0, m->X0t, m->Y1, m->Y1t, m->Y2, m->Y2t, m->G3, m->G3t, m->G2, m->G2t, m->G1, m->G1t,
                    m->Z1, m->Z2, m->O, m->T, m->nrow};
    cudaDeviceSynchronize();
    for (void *p : bufs)
        if (p) cudaFree(p);
    const size_t hb = (size_t)rows * kMlpWidth * 2, fb = (size_t)rows * kMlpWidth * 4;
    __nv_bfloat16 **hbp[] = {&m->X0, &m->X0t, &m->Y1, &m->Y1t, &m->Y2, &m->Y2t,
                             &m->G3, &m->G3t, &m->G2, &m->G2t, &m->G1, &m->G1t, &m->T};
    for (auto pp : hbp) {
        *pp = nullptr;
        int32_t st = dalloc((void **)pp, hb);
        if (st) { m->cap = 0; return st; }
    }
    float **fbp[] = {&m->Z1, &m->Z2, &m->O};
    for (auto pp : fbp) {
        *pp = nullptr;
        int32_t st = dalloc((void **)pp, fb);
        if (st) { m->cap = 0; return st; }
    }
    m->nrow = nullptr;
    int32_t st = dalloc((void **)&m->nrow, (size_t)rows * 4);
    if (st) { m->cap = 0; return st; }
    m->cap = rows;
    return SS_OK;
}

int32_t mlp_dataset_reserve(ss_mlp *m, int64_t rows) {
    if (rows <= m->ds_cap) return SS_OK;
    int64_t cap = std::max<int64_t>(rows, m->ds_cap * 2);
    cap = (cap + kMlpTileM - 1) / kMlpTileM * kMlpTileM;
    __nv_bfloat16 *X = nullptr, *T = nullptr;
    int32_t *n = nullptr, *perm = nullptr;
    int32_t st = dalloc((void **)&X, (size_t)cap * kMlpWidth * 2);
    if (!st) st = dalloc((void **)&T, (size_t)cap * kMlpWidth * 2);
    if (!st) st = dalloc((void **)&n, (size_t)cap * 4);
    if (!st) st = dalloc((void **)&perm, (size_t)cap * 4);
    if (st) { cudaFree(X); cudaFree(T); cudaFree(n); cudaFree(perm); return st; }
    if (m->ds_rows) {
        CUDA_TRY(cudaMemcpy(X, m->ds_X, (size_t)m->ds_rows * kMlpWidth * 2, cudaMemcpyDeviceToDevice));
        CUDA_TRY(cudaMemcpy(T, m->ds_T, (size_t)m->ds_rows * kMlpWidth * 2, cudaMemcpyDeviceToDevice));
        CUDA_TRY(cudaMemcpy(n, m->ds_n, (size_t)m->ds_rows * 4, cudaMemcpyDeviceToDevice));
    }
    cudaFree(m->ds_X); cudaFree(m->ds_T); cudaFree(m->ds_n); cudaFree(m->perm);
    m->ds_X = X; m->ds_T = T; m->ds_n = n; m->perm = perm;
    m->ds_cap = cap;
    return SS_OK;
}

static GemmArgs gemm(const __nv_bfloat16 *A, int64_t lda, const __nv_bfloat16 *B, int64_t ldb, int M, int ksplit,
                     int mode, int *err) {
    GemmArgs g{};
    g.A = A; g.lda = lda; g.B = B; g.ldb = ldb; g.M = M; g.ksplit = ksplit; g.mode = mode; g.err = err;
    return g;
}

static const size_t kWL = (size_t)kMlpWidth * kMlpWidth;

int32_t mlp_forward(ss_mlp *m, const __nv_bfloat16 *in, float *out, int64_t rows, cudaStream_t st) {
    int32_t r = mlp_reserve(m, rows);
    if (r) return r;
    const int M = (int)((rows + kMlpTileM - 1) / kMlpTileM * kMlpTileM);
    if (((uintptr_t)in & 15) || ((uintptr_t)out & 15)) { set_error("MLP rows must be 16-byte aligned"); return SS_BAD_SHAPE; }
    static bool attr = false;
    if (!attr) {
        CUDA_TRY(cudaFuncSetAttribute(mlp_infer_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInferSmem));
        attr = true;
    }
    mlp_infer_kernel<<<M / kMlpTileM, kInferThreads, kInferSmem, st>>>(in, m->Wb, m->b, out, m->err);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

// one forward/backward pass over the batch in X0/X0t/T/nrow (B rows, multiple of 128);
// leaves gradients in dW/db and the loss in m->loss
static int32_t mlp_fwd_bwd(ss_mlp *m, int64_t B, cudaStream_t st) {
    int32_t r;
    const int M = (int)B;
    const int64_t ldt = m->cap;
    // forward, keeping pre-activations and transposed activations
    GemmArgs g = gemm(m->X0, kMlpWidth, m->Wb, kMlpWidth, M, kMlpWidth, GEMM_RELU, m->err);
    g.bias = m->b; g.Cf = m->Z1; g.ldc = kMlpWidth; g.Yb = m->Y1; g.Yt = m->Y1t; g.ldt = ldt;
    if ((r = launch_gemm_tc(g, 1, st))) return r;
    g = gemm(m->Y1, kMlpWidth, m->Wb + kWL, kMlpWidth, M, kMlpWidth, GEMM_RELU, m->err);
    g.bias = m->b + kMlpWidth; g.Cf = m->Z2; g.ldc = kMlpWidth; g.Yb = m->Y2; g.Yt = m->Y2t; g.ldt = ldt;
    if ((r = launch_gemm_tc(g, 1, st))) return r;
    g = gemm(m->Y2, kMlpWidth, m->Wb + 2 * kWL, kMlpWidth, M, kMlpWidth, GEMM_STORE, m->err);
    g.bias = m->b + 2 * kMlpWidth; g.Cf = m->O; g.ldc = kMlpWidth;
    if ((r = launch_gemm_tc(g, 1, st))) return r;
    CUDA_TRY(cudaMemsetAsync(m->loss, 0, sizeof(float), st));
    mse_loss_kernel<<<(unsigned)B, kMlpWidth, 0, st>>>(m->O, m->T, m->nrow, B, ldt, m->G3, m->G3t, m->loss);
    CUDA_TRY(cudaGetLastError());
    // backward
    CUDA_TRY(cudaMemsetAsync(m->dW, 0, kMlpLayers * kWL * sizeof(float), st));
    int ks = 256;
    while (B % ks) ks /= 2;
    if (ks < kMlpChunkK) { set_error("batch must be a multiple of 128"); return SS_BAD_SHAPE; }
    const int splits = (int)(B / ks);
    const __nv_bfloat16 *Gt[3] = {m->G1t, m->G2t, m->G3t};
    const __nv_bfloat16 *Xt[3] = {m->X0t, m->Y1t, m->Y2t};
    for (int l = 2; l >= 0; l--) {
        // dW_l = G_lᵀ · X_l  (A = G_lᵀ [256][B], B = X_lᵀ [256][B])
        g = gemm(Gt[l], ldt, Xt[l], ldt, kMlpWidth, ks, GEMM_ATOMIC, m->err);
        g.Cf = m->dW + l * kWL; g.ldc = kMlpWidth;
        if ((r = launch_gemm_tc(g, splits, st))) return r;
        colsum_kernel<<<kMlpWidth, 256, 0, st>>>(Gt[l], ldt, B, m->db + l * kMlpWidth);
        CUDA_TRY(cudaGetLastError());
        if (l == 0) break;
        // G_{l-1} = (G_l · W_l) ⊙ [Z_{l-1} > 0]   (B operand = W_lᵀ [in][out])
        const __nv_bfloat16 *Gl = l == 2 ? m->G3 : m->G2;
        g = gemm(Gl, kMlpWidth, m->Wt + l * kWL, kMlpWidth, M, kMlpWidth, GEMM_DRELU, m->err);
        g.Zin = l == 2 ? m->Z2 : m->Z1;
        g.Yb = l == 2 ? m->G2 : m->G1;
        g.Yt = l == 2 ? m->G2t : m->G1t;
        g.ldt = ldt;
        if ((r = launch_gemm_tc(g, 1, st))) return r;
    }
    return SS_OK;
}

static int32_t mlp_adam(ss_mlp *m, float lr, cudaStream_t st) {
    m->adam_t++;
    const float c1 = 1.f - powf(0.9f, (float)m->adam_t), c2 = 1.f - powf(0.999f, (float)m->adam_t);
    const int64_t total = (int64_t)kMlpLayers * (kWL + kMlpWidth);
    adam_kernel<<<(unsigned)((total + 255) / 256), 256, 0, st>>>(m->W, m->b, m->dW, m->db, m->mW, m->vW, m->mb,
                                                                  m->vb, m->Wb, m->Wt, lr, c1, c2);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

static int32_t upload_batch(ss_mlp *m, const float *in, const float *target, const int32_t *n, int64_t rows,
                            int64_t B, cudaStream_t st) {
    std::vector<__nv_bfloat16> hx((size_t)B * kMlpWidth, __float2bfloat16(0.f)), ht(hx);
    std::vector<int32_t> hn((size_t)B, 0);
    for (int64_t i = 0; i < rows * kMlpWidth; i++) hx[i] = __float2bfloat16(in[i]);
    if (target)
        for (int64_t i = 0; i < rows * kMlpWidth; i++) ht[i] = __float2bfloat16(target[i]);
    if (n) std::copy(n, n + rows, hn.begin());
    CUDA_TRY(cudaMemcpyAsync(m->X0, hx.data(), hx.size() * 2, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(m->T, ht.data(), ht.size() * 2, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(m->nrow, hn.data(), hn.size() * 4, cudaMemcpyHostToDevice, st));
    // transposed copy of the input for the first layer's weight gradient
    std::vector<__nv_bfloat16> hxt((size_t)kMlpWidth * m->cap, __float2bfloat16(0.f));
    for (int64_t r = 0; r < B; r++)
        for (int c = 0; c < kMlpWidth; c++) hxt[(size_t)c * m->cap + r] = hx[(size_t)r * kMlpWidth + c];
    CUDA_TRY(cudaMemcpyAsync(m->X0t, hxt.data(), hxt.size() * 2, cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return SS_OK;
}

}  // namespace ss

// ---------------------------------------------------------------- C ABI
extern "C" int32_t ss_mlp_create(int32_t device, uint64_t seed, ss_mlp **out) {
    if (!out) { set_error("null argument"); return SS_BAD_ARG; }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        cudaGetLastError();
        set_error("no CUDA device");
        return SS_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) { set_error("device %d out of range", device); return SS_BAD_ARG; }
    cudaSetDevice(device);
    ss_mlp *m = new ss_mlp();
    m->device = device;
    m->seed = seed;
    const size_t nW = kMlpLayers * kWL, nb = kMlpLayers * kMlpWidth;
    int32_t st = SS_OK;
    float **fp[] = {&m->W, &m->mW, &m->vW, &m->dW};
    for (auto pp : fp)
        if (!st) st = dalloc((void **)pp, nW * 4);
    float **bp[] = {&m->b, &m->mb, &m->vb, &m->db};
    for (auto pp : bp)
        if (!st) st = dalloc((void **)pp, nb * 4);
    if (!st) st = dalloc((void **)&m->Wb, nW * 2);
    if (!st) st = dalloc((void **)&m->Wt, nW * 2);
    if (!st) st = dalloc((void **)&m->loss, 4);
    if (!st) st = dalloc((void **)&m->err, 4);
    if (st) { ss_mlp_destroy(m); return st; }
    if (cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking) != cudaSuccess) {
        ss_mlp_destroy(m);
        set_error("stream creation failed");
        return SS_CUDA_ERROR;
    }
    // He-normal hidden layers, zero output layer (the network starts as the identity correction 0)
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, std::sqrt(2.f / kMlpWidth));
    std::vector<float> W(nW, 0.f), b(nb, 0.f);
    for (size_t i = 0; i < 2 * kWL; i++) W[i] = nd(rng);
    st = ss_mlp_set_params(m, W.data(), b.data());
    if (st) { ss_mlp_destroy(m); return st; }
    *out = m;
    return SS_OK;
}

extern "C" int32_t ss_mlp_destroy(ss_mlp *m) {
    if (!m) return SS_OK;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    void *bufs[] = {m->W, m->b, m->mW, m->vW, m->mb, m->vb, m->dW, m->db, m->Wb, m->Wt, m->X0, m->X0t,
                    m->Y1, m->Y1t, m->Y2, m->Y2t, m->G3, m->G3t, m->G2, m->G2t, m->G1, m->G1t, m->Z1, m->Z2,
                    m->O, m->T, m->nrow, m->loss, m->err, m->ds_X, m->ds_T, m->ds_n, m->perm};
    for (void *p : bufs)
        if (p) cudaFree(p);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
    return SS_OK;
}

extern "C" int32_t ss_mlp_set_params(ss_mlp *m, const float *W, const float *b) {
    if (!m || !W || !b) { set_error("null argument"); return SS_BAD_ARG; }
    cudaSetDevice(m->device);
    CUDA_TRY(cudaMemcpy(m->W, W, kMlpLayers * kWL * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(m->b, b, kMlpLayers * kMlpWidth * 4, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(m->mW, 0, kMlpLayers * kWL * 4));
    CUDA_TRY(cudaMemset(m->vW, 0, kMlpLayers * kWL * 4));
    CUDA_TRY(cudaMemset(m->mb, 0, kMlpLayers * kMlpWidth * 4));
    CUDA_TRY(cudaMemset(m->vb, 0, kMlpLayers * kMlpWidth * 4));
    m->adam_t = 0;
    refresh_bf16_kernel<<<(unsigned)((kMlpLayers * kWL + 255) / 256), 256>>>(m->W, m->Wb, m->Wt);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaDeviceSynchronize());
    return SS_OK;
}

extern "C" int32_t ss_mlp_get_params(const ss_mlp *m, float *W, float *b) {
    if (!m) { set_error("null argument"); return SS_BAD_ARG; }
    cudaSetDevice(m->device);
    CUDA_TRY(cudaDeviceSynchronize());
    if (W) CUDA_TRY(cudaMemcpy(W, m->W, kMlpLayers * kWL * 4, cudaMemcpyDeviceToHost));
    if (b) CUDA_TRY(cudaMemcpy(b, m->b, kMlpLayers * kMlpWidth * 4, cudaMemcpyDeviceToHost));
    return SS_OK;
}

extern "C" int32_t ss_mlp_forward(ss_mlp *m, const float *in, float *out, int64_t rows) {
    if (!m || !in || !out || rows <= 0) { set_error("bad argument"); return SS_BAD_ARG; }
    cudaSetDevice(m->device);
    int32_t r = mlp_reserve(m, rows);
    if (r) return r;
    const int64_t B = (rows + kMlpTileM - 1) / kMlpTileM * kMlpTileM;
    if ((r = upload_batch(m, in, nullptr, nullptr, rows, B, m->stream))) return r;
    if ((r = mlp_forward(m, m->X0, m->O, B, m->stream))) return r;
    CUDA_TRY(cudaMemcpyAsync(out, m->O, (size_t)rows * kMlpWidth * 4, cudaMemcpyDeviceToHost, m->stream));
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    return check_err(m);
}

extern "C" int32_t ss_mlp_gradients(ss_mlp *m, const float *in, const float *target, const int32_t *n, int64_t rows,
                                    float *dW, float *db, double *loss) {
    if (!m || !in || !target || !n || rows <= 0) { set_error("bad argument"); return SS_BAD_ARG; }
    if (rows % kMlpTileM) { set_error("rows must be a multiple of 128"); return SS_BAD_SHAPE; }
    for (int64_t i = 0; i < rows; i++)
        if (n[i] < 0 || n[i] > kMlpWidth) { set_error("row width out of range"); return SS_BAD_ARG; }
    cudaSetDevice(m->device);
    int32_t r = mlp_reserve(m, rows);
    if (r) return r;
    if ((r = upload_batch(m, in, target, n, rows, rows, m->stream))) return r;
    if ((r = mlp_fwd_bwd(m, rows, m->stream))) return r;
    CUDA_TRY(cudaStreamSynchronize(m->stream));
    if ((r = check_err(m))) return r;
    if (dW) CUDA_TRY(cudaMemcpy(dW, m->dW, kMlpLayers * kWL * 4, cudaMemcpyDeviceToHost));
    if (db) CUDA_TRY(cudaMemcpy(db, m->db, kMlpLayers * kMlpWidth * 4, cudaMemcpyDeviceToHost));
    if (loss) {
        float l = 0.f;
        CUDA_TRY(cudaMemcpy(&l, m->loss, 4, cudaMemcpyDeviceToHost));
        *loss = l;
    }
    return SS_OK;
}

extern "C" int32_t ss_mlp_dataset_rows(const ss_mlp *m, int64_t *rows) {
    if (!m || !rows) { set_error("null argument"); return SS_BAD_ARG; }
    *rows = m->ds_rows;
    return SS_OK;
}

extern "C" int32_t ss_mlp_dataset_clear(ss_mlp *m) {
    if (!m) { set_error("null argument"); return SS_BAD_ARG; }
    m->ds_rows = 0;
    return SS_OK;
}

// Adam over the resident training set: `epochs` shuffled passes in batches of
// `batch` rows (multiple of 128); the mean batch loss of the last epoch is returned.
extern "C" int32_t ss_mlp_train(ss_mlp *m, int32_t epochs, int32_t batch, float lr, uint64_t seed,
                                ss_train_stats *stats) {
    if (!m || epochs < 0 || batch <= 0 || batch % kMlpTileM) {
        set_error("batch must be a positive multiple of 128");
        return SS_BAD_ARG;
    }
    if (m->ds_rows < batch) { set_error("training set (%lld rows) smaller than one batch", (long long)m->ds_rows); return SS_BAD_SHAPE; }
    cudaSetDevice(m->device);
    int32_t r = mlp_reserve(m, batch);
    if (r) return r;
    cudaStream_t st = m->stream;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, st);
    std::mt19937_64 rng(seed);
    std::vector<int32_t> perm((size_t)m->ds_rows);
    const int64_t nb = m->ds_rows / batch;
    double last = 0.0, first = 0.0;
    std::vector<float> losses((size_t)nb);
    float *d_losses = nullptr;
    if ((r = dalloc((void **)&d_losses, (size_t)nb * 4))) return r;
    int64_t steps = 0;
    for (int e = 0; e < epochs; e++) {
        for (int64_t i = 0; i < m->ds_rows; i++) perm[i] = (int32_t)i;
        std::shuffle(perm.begin(), perm.end(), rng);
        CUDA_TRY(cudaMemcpyAsync(m->perm, perm.data(), perm.size() * 4, cudaMemcpyHostToDevice, st));
        for (int64_t bi = 0; bi < nb; bi++) {
            gather_rows_kernel<<<batch, kMlpWidth, 0, st>>>(m->ds_X, m->ds_T, m->ds_n, m->perm + bi * batch, batch,
                                                            m->cap, m->X0, m->X0t, m->T, m->nrow);
            CUDA_TRY(cudaGetLastError());
            if ((r = mlp_fwd_bwd(m, batch, st))) { cudaFree(d_losses); return r; }
            if ((r = mlp_adam(m, lr, st))) { cudaFree(d_losses); return r; }
            CUDA_TRY(cudaMemcpyAsync(d_losses + bi, m->loss, 4, cudaMemcpyDeviceToDevice, st));
            steps++;
        }
        CUDA_TRY(cudaMemcpyAsync(losses.data(), d_losses, (size_t)nb * 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        double s = 0.0;
        for (float l : losses) s += l;
        last = s / (double)nb;
        if (e == 0) first = last;
    }
    cudaEventRecord(e1, st);
    CUDA_TRY(cudaEventSynchronize(e1));
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d_losses);
    if ((r = check_err(m))) return r;
    if (stats) {
        stats->epochs = epochs;
        stats->steps = steps;
        stats->rows = m->ds_rows;
        stats->first_epoch_loss = first;
        stats->last_epoch_loss = last;
        stats->ms = ms;
    }
    return SS_OK;
}
