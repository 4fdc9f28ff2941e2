// ss_sa_f32.cu — SAtransform! + SI for binary32 grids (SS_PREC_F32_REFINED).
//
// SAtransform! (src/CubicBSpline.jl:1368-1396) solves, per spectral slot, the
// banded system Γ(P+Q)Γᵀ x = Γ b and unfolds a = Γᵀ x (+ ahat); SIxcoeff/
// SIxxcoeff evaluate f, ∂r, ∂rr at the mish points from 4-tap windows of a.
// In binary32 the solve runs on the FP32-rounded Cholesky factor, followed by
// one refinement step in FP64: the residual r = Γb − A x against the FP64
// open-form band and the correction solve x += L⁻ᵀL⁻¹ r with the FP64 factor
// (FP64 arithmetic throughout; the forward sweep's intermediate is kept in
// binary32 between the two sweeps, an error of order 2^-24·|c| ≈ 2^-48·|x|).
//
// Layout: one thread per spectral slot, 128 consecutive slots per CTA, every
// thread solving.  The per-slot vectors live in two slot-interleaved scratch
// arrays X, Y ([item][row][slot], a warp's rows are 128-byte coalesced), the
// band window in registers; rows are prefetched in blocks so that the
// substitution recurrences do not wait on one load per row.  Sweeps:
//   1  stage b in 32-row chunks through shared memory; b̃ = b − PQ·ahat;
//      Γ fold → X; forward substitution L y = Γb → Y
//   2  backward substitution Lᵀ x = y, in place in Y
//   3  residual r = Γb − A x (FP64) fused with the FP64 forward substitution
//      of the correction → X
//   4  FP64 backward substitution of the correction, x + c, unfold a = Γᵀ x + ahat
//      written shifted by rankL into Y (descending rows, so every row is read
//      before it is overwritten), boundary rows last
//   5  SI / SIx / SIxx at the mish points of every ring that carries the slot,
//      with a sliding 4-coefficient window → G
// With coefficient input (spectral holds a), sweep 1 copies b into Y and
// sweeps 2-4 are skipped.
#include <cuda_runtime.h>

#include "ss_kernels.h"
#include "ss_types.cuh"

namespace ss {

constexpr int kSaSlots = 128;  // slots (threads) per CTA; 6 resident CTAs leave 80 registers for
                               // the FP64 residual window (measured 18.3 ms against 19.6 ms at 8
                               // CTAs with a binary32 window, 400-cell binary32 grid)
constexpr int kSaChunk = 32;   // rows per shared-memory staging chunk
constexpr int kSaBlk = 8;      // rows per prefetch block in the substitution sweeps

template <typename P>
__device__ __forceinline__ void sa_si_f32_body(const SaLaunch &A, float *X, float *Y, const int bx, const int by) {
    __shared__ float tile[kSaSlots][kSaChunk + 1];
    const int item = by;
    const int v = item / A.bk, zb = item % A.bk;
    const SplineDev &sp = A.spl[v];
    const int Md = A.b, n = sp.Min, rL = sp.rankL;
    const int s0 = bx * kSaSlots, t = threadIdx.x, s = s0 + t;
    const int nsl = min(kSaSlots, A.nslots_z - s0);
    const bool act = t < nsl;
    const size_t ns = (size_t)A.nslots_z;
    // this thread's column of the scratch arrays: row i at [i * ns]
    float *Xc = X + (size_t)item * Md * ns + s;
    float *Yc = Y + (size_t)item * Md * ns + s;
    const P *spec = (const P *)A.spec + (size_t)v * A.nspec + ((size_t)zb * A.nslots_z + s0) * Md;
    const double *ah = (!A.coeffs && sp.r3x && A.ahat)
                           ? A.ahat + ((size_t)v * A.nblocks + (size_t)zb * A.nslots_z + s) * Md
                           : nullptr;
    const float *Lf = sp.L4f, *Df = sp.dinvf;
    const float aL = (float)sp.aL, bL = (float)sp.bL, aR = (float)sp.aR, bR = (float)sp.bR;
    // b̃_m = b_m − (PQ·ahat)_m (full P+Q band, half-width 3)
    auto pq_ahat = [&](int m) -> double {
        double acc = 0.0;
        for (int j = max(0, m - 3); j <= min(Md - 1, m + 3); j++) acc += sp.PQb[m * 7 + (j - m + 3)] * ah[j];
        return acc;
    };

    // ---- sweep 1
    float bM1 = 0.f, bM2 = 0.f, b0 = 0.f, b1 = 0.f;
    if (act && !A.coeffs) {  // the right-end Γ terms need the last two rows first
        bM1 = (float)spec[(size_t)t * Md + Md - 1];
        bM2 = (float)spec[(size_t)t * Md + Md - 2];
        if (ah) {
            bM1 = (float)((double)bM1 - pq_ahat(Md - 1));
            bM2 = (float)((double)bM2 - pq_ahat(Md - 2));
        }
    }
    float y1 = 0.f, y2 = 0.f, y3 = 0.f;
    double g0d = 0.0, g1d = 0.0, gm2d = 0.0, gm1d = 0.0;  // Γb rows 0, 1, n−2, n−1 in FP64 (the residual's)
    for (int m0 = 0; m0 < Md; m0 += kSaChunk) {
        const int mc = min(kSaChunk, Md - m0);
        __syncthreads();
        for (int e = t; e < nsl * kSaChunk; e += kSaSlots) {
            const int sl = e / kSaChunk, mm = e % kSaChunk;
            tile[sl][mm] = mm < mc ? (float)spec[(size_t)sl * Md + m0 + mm] : 0.f;
        }
        __syncthreads();
        if (!act) continue;
        if (A.coeffs) {
            for (int mm = 0; mm < mc; mm++) Yc[(size_t)(m0 + mm) * ns] = tile[t][mm];
            continue;
        }
        for (int mm = 0; mm < mc; mm++) {
            const int m = m0 + mm;
            float bm = tile[t][mm];
            if (ah) bm = (float)((double)bm - pq_ahat(m));
            if (m == 0) b0 = bm;
            if (m == 1) b1 = bm;
            const int i = m - rL;
            if (i < 0 || i >= n) continue;
            // Γ fold (src/CubicBSpline.jl:427-463): row i = b_{i+rankL} + boundary terms
            float gb = bm;
            if (i <= 1 || i >= n - 2) {  // boundary rows: the fold in FP64 for the residual
                double gd = (double)bm;
                if (i == 0) {
                    if (sp.lk == BC_A1) gd += sp.aL * (double)b0;
                    else if (sp.lk == BC_A2) gd += sp.aL * (double)b0 + sp.bL * (double)b1;
                }
                if (i == 1 && sp.lk == BC_A1) gd += sp.bL * (double)b0;
                if (i == n - 1) {
                    if (sp.rk == BC_A1) gd += sp.aR * (double)bM1;
                    else if (sp.rk == BC_A2) gd += sp.aR * (double)bM1 + sp.bR * (double)bM2;
                }
                if (i == n - 2 && sp.rk == BC_A1) gd += sp.bR * (double)bM1;
                if (i == 0) g0d = gd;
                if (i == 1) g1d = gd;
                if (i == n - 2) gm2d = gd;
                if (i == n - 1) gm1d = gd;
                gb = (float)gd;
            }
            Xc[(size_t)i * ns] = gb;
            float acc = gb;
            if (i >= 3) acc -= Lf[(i - 3) * 4 + 3] * y3;
            if (i >= 2) acc -= Lf[(i - 2) * 4 + 2] * y2;
            if (i >= 1) acc -= Lf[(i - 1) * 4 + 1] * y1;
            const float yi = acc * Df[i];
            Yc[(size_t)i * ns] = yi;
            y3 = y2; y2 = y1; y1 = yi;
        }
    }
    if (!act) return;

    if (!A.coeffs) {
        // ---- sweep 2: Lᵀ x = y in place (src/banded_cholesky.jl:216-231)
        float x1 = 0.f, x2 = 0.f, x3 = 0.f;
        for (int hi = n - 1; hi >= 0; hi -= kSaBlk) {
            float yv[kSaBlk];
#pragma unroll
            for (int k = 0; k < kSaBlk; k++) yv[k] = hi - k >= 0 ? Yc[(size_t)(hi - k) * ns] : 0.f;
#pragma unroll
            for (int k = 0; k < kSaBlk; k++) {
                const int i = hi - k;
                if (i < 0) break;
                float acc = yv[k];
                if (i + 1 < n) acc -= Lf[i * 4 + 1] * x1;
                if (i + 2 < n) acc -= Lf[i * 4 + 2] * x2;
                if (i + 3 < n) acc -= Lf[i * 4 + 3] * x3;
                const float xi = acc * Df[i];
                Yc[(size_t)i * ns] = xi;
                x3 = x2; x2 = x1; x1 = xi;
            }
        }

        // ---- sweep 3: r = Γb − A x in FP64, window w[q] = x_{i+q−3}; FP64 forward
        //      substitution of the correction L c' = r with the FP64 factor → X
        const double *Ld = sp.L4, *Dd = sp.dinv, *Ab = sp.Aband;
        // the window is kept in FP64: each x_j is converted once, when it enters
        // (conversions to FP64 share the FP64 pipe with the residual's FMAs)
        double w[7];
#pragma unroll
        for (int q = 0; q < 7; q++) {
            const int j = q - 3;
            w[q] = (j >= 0 && j < n) ? (double)Yc[(size_t)j * ns] : 0.0;
        }
        double z1 = 0.0, z2 = 0.0, z3 = 0.0;
        for (int lo = 0; lo < n; lo += kSaBlk) {
            float gv[kSaBlk], xn[kSaBlk];
#pragma unroll
            for (int k = 0; k < kSaBlk; k++) {
                const int i = lo + k;
                gv[k] = i < n ? Xc[(size_t)i * ns] : 0.f;
                xn[k] = i + 4 < n ? Yc[(size_t)(i + 4) * ns] : 0.f;
            }
#pragma unroll
            for (int k = 0; k < kSaBlk; k++) {
                const int i = lo + k;
                if (i >= n) break;
                double acc = i == 0 ? g0d : (i == 1 ? g1d : (i == n - 2 ? gm2d : (i == n - 1 ? gm1d : (double)gv[k])));
#pragma unroll
                for (int q = 0; q < 7; q++) {
                    const int j = i + q - 3;
                    if (j < 0 || j >= n) continue;
                    acc -= __ldg(Ab + min(i, j) * 4 + abs(q - 3)) * w[q];
                }
                if (i >= 3) acc -= __ldg(Ld + (i - 3) * 4 + 3) * z3;
                if (i >= 2) acc -= __ldg(Ld + (i - 2) * 4 + 2) * z2;
                if (i >= 1) acc -= __ldg(Ld + (i - 1) * 4 + 1) * z1;
                const double zi = acc * __ldg(Dd + i);
                Xc[(size_t)i * ns] = (float)zi;
                z3 = z2; z2 = z1; z1 = zi;
#pragma unroll
                for (int q = 0; q < 6; q++) w[q] = w[q + 1];
                w[6] = (double)xn[k];
            }
        }

        // ---- sweep 4: Lᵀ c = c' in FP64 with the FP64 factor, x + c, a_{i+rankL} =
        //      x_i (+ ahat) → Y row i + rankL
        float x0 = 0.f, xs1 = 0.f, xn1 = 0.f, xn2 = 0.f;
        double c1 = 0.0, c2 = 0.0, c3 = 0.0;
        for (int hi = n - 1; hi >= 0; hi -= kSaBlk) {
            float cv[kSaBlk], xv[kSaBlk];
#pragma unroll
            for (int k = 0; k < kSaBlk; k++) {
                const int i = hi - k;
                cv[k] = i >= 0 ? Xc[(size_t)i * ns] : 0.f;
                xv[k] = i >= 0 ? Yc[(size_t)i * ns] : 0.f;
            }
#pragma unroll
            for (int k = 0; k < kSaBlk; k++) {
                const int i = hi - k;
                if (i < 0) break;
                double acc = (double)cv[k];
                if (i + 1 < n) acc -= __ldg(Ld + i * 4 + 1) * c1;
                if (i + 2 < n) acc -= __ldg(Ld + i * 4 + 2) * c2;
                if (i + 3 < n) acc -= __ldg(Ld + i * 4 + 3) * c3;
                const double ci = acc * __ldg(Dd + i);
                c3 = c2; c2 = c1; c1 = ci;
                const float xf = xv[k] + (float)ci;  // the binary32 result: one conversion
                if (i == n - 1) xn1 = xf;
                if (i == n - 2) xn2 = xf;
                if (i == 1) xs1 = xf;
                if (i == 0) x0 = xf;
                const int m = i + rL;
                Yc[(size_t)m * ns] = ah ? (float)((double)xf + ah[m]) : xf;
            }
        }
        // boundary rows of Γᵀ x (src/CubicBSpline.jl:465-500): m < rankL, m ≥ rankL + n
        for (int m = 0; m < rL; m++) {
            float a = 0.f;
            if (sp.lk == BC_A1 && m == 0) a = aL * x0 + bL * xs1;
            if (sp.lk == BC_A2) a = m == 0 ? aL * x0 : (m == 1 ? bL * x0 : 0.f);
            Yc[(size_t)m * ns] = ah ? (float)((double)a + ah[m]) : a;
        }
        for (int m = rL + n; m < Md; m++) {
            float a = 0.f;
            if (sp.rk == BC_A1 && m == Md - 1) a = aR * xn1 + bR * xn2;
            if (sp.rk == BC_A2) a = m == Md - 1 ? aR * xn1 : (m == Md - 2 ? bR * xn1 : 0.f);
            Yc[(size_t)m * ns] = ah ? (float)((double)a + ah[m]) : a;
        }
    }

    // ---- sweep 5: f, ∂r, ∂rr at the mish points of the rings carrying slot s
    // (ring ri carries slots s < 1 + 2 ri; si_m0 is nondecreasing in r)
    int cur = -8;
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
    for (int r = max(0, (s - 1) / 2 - A.pOL); r < A.iDim; r++) {
        const int ri = r + 1 + A.pOL;
        if (s >= 1 + 2 * ri) continue;
        const int m0 = sp.si_m0[r];
        if (m0 == cur + 1) {
            a0 = a1; a1 = a2; a2 = a3;
            a3 = Yc[(size_t)(m0 + 3) * ns];
        } else if (m0 != cur) {
            a0 = Yc[(size_t)m0 * ns];
            a1 = Yc[(size_t)(m0 + 1) * ns];
            a2 = Yc[(size_t)(m0 + 2) * ns];
            a3 = Yc[(size_t)(m0 + 3) * ns];
        }
        cur = m0;
        const size_t orow = A.fofs[r] + s;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const int64_t wi = ((int64_t)d * A.iDim + r) * 4;
            const float u = ld_real<float>(sp.siw_t, wi) * a0 + ld_real<float>(sp.siw_t, wi + 1) * a1 +
                            ld_real<float>(sp.siw_t, wi + 2) * a2 + ld_real<float>(sp.siw_t, wi + 3) * a3;
            ((float *)A.G)[((size_t)d * A.nitems + item) * A.frows + orow] = u;
        }
    }
}

template <typename P>
__global__ void __launch_bounds__(kSaSlots, 6) sa_si_f32_kernel(SaLaunch A, float *X, float *Y) {
    sa_si_f32_body<P>(A, X, Y, blockIdx.x, blockIdx.y);
}

// fused multi-grid launch: CTA blockIdx.x runs work[blockIdx.x]; the record
// (with its own scratch arrays) is staged in shared memory
template <typename P>
__global__ void __launch_bounds__(kSaSlots, 6) sa_si_f32_fused_kernel(const SaLaunch *recs, const BatchWork *work) {
    __shared__ __align__(16) SaLaunch A;
    const BatchWork w = work[blockIdx.x];
    for (int i = threadIdx.x; i < (int)(sizeof(SaLaunch) / 4); i += blockDim.x)
        reinterpret_cast<int *>(&A)[i] = __ldg(reinterpret_cast<const int *>(recs + w.rec) + i);
    __syncthreads();
    sa_si_f32_body<P>(A, A.sx, A.sy, w.bx, w.by);
}

template <typename P>
cudaError_t launch_sa_si_f32_fused(const SaLaunch *recs, const BatchWork *work, int nwork, cudaStream_t st) {
    if (nwork <= 0) return cudaSuccess;
    sa_si_f32_fused_kernel<P><<<nwork, kSaSlots, 0, st>>>(recs, work);
    return cudaGetLastError();
}
template cudaError_t launch_sa_si_f32_fused<float>(const SaLaunch *, const BatchWork *, int, cudaStream_t);

template <typename P>
cudaError_t launch_sa_si_f32(const SaLaunch &A, int nitems, float *X, float *Y, cudaStream_t st) {
    const dim3 grid((A.nslots_z + kSaSlots - 1) / kSaSlots, nitems);
    sa_si_f32_kernel<P><<<grid, kSaSlots, 0, st>>>(A, X, Y);
    return cudaGetLastError();
}
template cudaError_t launch_sa_si_f32<float>(const SaLaunch &, int, float *, float *, cudaStream_t);

}  // namespace ss
