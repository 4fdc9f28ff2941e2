// ss_kernels.cu — sm_103a kernels of the RL/RLZ transform path.
//
// Data flow of one variable (RL: b_kDim = 1, no column stages):
//   spectralTransform!  (src/transforms_cylindrical.jl:159-222, 530-618)
//     cheb_forward   physical slot 1 columns (kz) → C[r][zb][l]      (CBtransform!)
//     ring_forward   ring R2HC + 1/L + phase rotation → F rows       (FBtransform!)
//     sb_project     12-tap B-spline projection per slot → spectral  (SBtransform!)
//   gridTransform!     (src/transforms_cylindrical.jl:259-428, 659-853)
//     sa_si          Γ fold + banded LLᵀ solve + Γᵀ (+ahat), then f, ∂r, ∂rr at the
//                    mish points → G rows                             (SAtransform!, SI*)
//     ring_inverse   phase rotation back + HC2R for f, ∂λ, ∂λλ, ∂r, ∂rr
//     cheb_inverse   CA (Γ fold) + DCT-I for each ring output; f column also ∂z, ∂zz
//
// Every kernel is a template over the storage type P of physical/spectral
// (double | float) and the compute type T (double | df64 | float); the
// intermediate buffers C, F, G, H hold T values.
//
// Packed coefficient rows: ring r (ri = r + patchOffsetL) owns 1+2ri entries
// [DC, re1, im1, re2, im2, …] — the order of the reference's spectral slots.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>

#include "ss_fft.cuh"
#include "ss_kernels.h"
#include "ss_spline_dev.cuh"

namespace ss {

// ------------------------------------------------------------ constants
void fft_init_constants() {
    static bool done[64] = {false};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev >= 0 && dev < 64 && done[dev]) return;
    double c[14][14] = {}, s[14][14] = {};
    float cf[14][14] = {}, sf[14][14] = {};
    float2 cx[14][14] = {}, sx[14][14] = {};
    for (int R = 2; R < 14; R++)
        for (int j = 0; j < R; j++) {
            // cos(2π j/R), sin(2π j/R), reduced to the first half turn
            int jj = (2 * j > R) ? R - j : j;
            double a = 2.0 * 3.14159265358979323846 * jj / R;
            c[R][j] = std::cos(a);
            s[R][j] = (2 * j > R) ? -std::sin(a) : std::sin(a);
            cf[R][j] = (float)c[R][j];
            sf[R][j] = (float)s[R][j];
            cx[R][j] = make_float2((float)c[R][j], (float)(c[R][j] - (double)(float)c[R][j]));
            sx[R][j] = make_float2((float)s[R][j], (float)(s[R][j] - (double)(float)s[R][j]));
        }
    cudaMemcpyToSymbol(c_rcos_d, c, sizeof c);
    cudaMemcpyToSymbol(c_rsin_d, s, sizeof s);
    cudaMemcpyToSymbol(c_rcos_f, cf, sizeof cf);
    cudaMemcpyToSymbol(c_rsin_f, sf, sizeof sf);
    cudaMemcpyToSymbol(c_rcos_x, cx, sizeof cx);
    cudaMemcpyToSymbol(c_rsin_x, sx, sizeof sx);
    if (dev >= 0 && dev < 64) done[dev] = true;
}

// Resident 256-thread CTAs the ring kernels are compiled for: binary32
// butterflies fit 64 registers (4 CTAs per SM); binary64 and double-float need more.
template <typename T>
constexpr int kRingMinBlocks = std::is_same<T, float>::value ? 4 : 2;
// sequences per unit of the kernels' element-wise load / pack / store sweeps
constexpr int kSweepSeqs = 1;

// ====================================================================
// ring_forward: one CTA per (ring, batch of up to L.ib items); item = v*bk + zb
// (RLZ) or v (RL).  The items of a batch share the ring's plan and twiddles;
// their sequences sit fft_seq_stride(plan) complex entries apart in each
// ping-pong buffer (each buffer holds L.ib × fft_buffer_len(plan) entries).
// The grid is (item batches, rings): CTAs scheduled together mostly work on
// the same ring and share its plan, twiddle and phase tables in L1/L2
// (measured on GB300: 6.5% less ring_inverse time than ring-fastest order
// for the binary32 400-cell grid, 4% for the binary64 200-cell grid).
// ====================================================================
template <typename P, typename T>
__device__ __forceinline__ void ring_forward_body(const RingLaunch &L, const int bx, const int by) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int kmx[kRingBatchMax];
    const int ring = L.ring_list[by];  // consecutive CTAs: item batches of one ring
    const int item0 = bx * L.ib;
    const int nb = min(L.ib, L.nitems - item0);
    const RingDesc rd = L.rings[(size_t)(L.rlz ? 0 : item0) * L.ring_var_stride + ring];
    const FftPlan &pl = L.plans[rd.plan];
    const int buf = fft_buffer_len(pl), sq = fft_seq_stride(pl);
    cpx<T> *A = reinterpret_cast<cpx<T> *>(smem_raw);
    cpx<T> *B = A + (size_t)L.ib * buf;
    __shared__ int64_t ioff[kRingBatchMax];  // element offset of each item's ring in the input
    const int Lr = rd.L, N = Lr / 2;
    if (threadIdx.x < nb) {
        const int item = item0 + threadIdx.x;
        kmx[threadIdx.x] = L.rings[(size_t)(L.rlz ? 0 : item) * L.ring_var_stride + ring].kmax;
        ioff[threadIdx.x] = L.rlz ? (int64_t)(item / L.bk) * L.bk * L.jDim + (int64_t)L.bk * rd.jofs +
                                        (int64_t)(item % L.bk) * Lr
                                  : (int64_t)item * L.in_item_stride + rd.jofs;
    }
    __syncthreads();
    for (UnitWalk uw_(N); uw_.g < (nb); uw_.next()) {
        const int n = uw_.n, b = uw_.g;
        // ring offsets and lengths are even: (point 2n, point 2n+1) is one aligned pair
        if (L.rlz) {
            A[(size_t)b * sq + n] = reinterpret_cast<const cpx<T> *>((const T *)L.in + ioff[b])[n];
        } else {
            const cpx<P> v = reinterpret_cast<const cpx<P> *>((const P *)L.in + ioff[b])[n];
            A[(size_t)b * sq + n] = {to_compute<T>(v.x), to_compute<T>(v.y)};
        }
    }
    __syncthreads();
    cpx<T> *Zb = dft<-1, T>(A, B, pl, L.pool, nb, L.ib);

    const T invL = T(1.0f) / T((float)Lr);
    const int nk = rd.ri + 1;
    const int G = (nb + kSweepSeqs - 1) / kSweepSeqs;
    for (UnitWalk uw_(nk); uw_.g < (G); uw_.next()) {
        const int k = uw_.n, g = uw_.g;
        cpx<T> uw = c_zero<T>(), cs = c_zero<T>();
        if (k > 0) {
            uw = ld_cplx<T>(L.pool, rd.utw + k);
            cs = ld_cplx<T>(L.phase, rd.phase + (k - 1));
        }
#pragma unroll
        for (int t = 0; t < kSweepSeqs; t++) {
            const int b = g * kSweepSeqs + t;
            if (b >= nb) break;
            const cpx<T> *Z = Zb + (size_t)b * sq;
            T *out = (T *)L.out + (size_t)(item0 + b) * L.frows + rd.fofs;
            const cpx<T> zk = Z[k];
            const cpx<T> zn = c_conj(Z[(N - k) % N]);
            if (k == 0) {
                out[0] = (zk.x + zk.y) * invL;
                continue;
            }
            T bre = T(0.0f), bim = T(0.0f);
            if (k <= kmx[b]) {
                cpx<T> e = {scale_f(zk.x + zn.x, 0.5f), scale_f(zk.y + zn.y, 0.5f)};
                cpx<T> d = {scale_f(zk.x - zn.x, 0.5f), scale_f(zk.y - zn.y, 0.5f)};
                cpx<T> o = {d.y, -d.x};  // d / i
                cpx<T> X = c_add(e, c_mul(uw, o));
                T re = X.x * invL, im = X.y * invL;
                bre = cs.x * re + cs.y * im;
                bim = -(cs.y * re) + cs.x * im;
            }
            out[2 * k - 1] = bre;
            out[2 * k] = bim;
        }
    }
}

template <typename P, typename T>
__global__ void __launch_bounds__(256, kRingMinBlocks<T>) ring_forward_kernel(RingLaunch L) {
    ring_forward_body<P, T>(L, blockIdx.x, blockIdx.y);
}

// ====================================================================
// ring_inverse: one CTA per (ring, batch of items).  For d = 0 (value), 1 (∂r),
// 2 (∂rr) read the ring's coefficient rows, undo the phase rotation
// (FAtransform!), and run HC2R for the variants: d=0 → f, ∂λ, ∂λλ; d=1 → ∂r;
// d=2 → ∂rr.
// ====================================================================
template <typename P, typename T>
__device__ __forceinline__ void ring_inverse_body(const RingLaunch &L, const int bx, const int by) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int kmx[kRingBatchMax];
    const int ring = L.ring_list[by];  // consecutive CTAs: item batches of one ring
    const int item0 = bx * L.ib;
    const int nb = min(L.ib, L.nitems - item0);
    const RingDesc rd = L.rings[(size_t)(L.rlz ? 0 : item0) * L.ring_var_stride + ring];
    const FftPlan &pl = L.plans[rd.plan];
    const int buf = fft_buffer_len(pl), sq = fft_seq_stride(pl);
    const int nk = rd.ri + 1;  // Xs stride: kmax ≤ ri
    cpx<T> *A = reinterpret_cast<cpx<T> *>(smem_raw);
    cpx<T> *B = A + (size_t)L.ib * buf;
    cpx<T> *Xs = B + (size_t)L.ib * buf;  // rotated spectra X_k, k = 0..kmax, per item
    __shared__ int64_t ooff[kRingBatchMax];  // element offset of each item's ring in one output plane
    const int Lr = rd.L, N = Lr / 2;
    if (threadIdx.x < nb) {
        const int item = item0 + threadIdx.x;
        kmx[threadIdx.x] = L.rings[(size_t)(L.rlz ? 0 : item) * L.ring_var_stride + ring].kmax;
        // RLZ: H[variant][v][r][zb][l]; RL: physical[slot][v][point]
        ooff[threadIdx.x] = L.rlz ? (int64_t)(item / L.bk) * L.bk * L.jDim + (int64_t)L.bk * rd.jofs +
                                        (int64_t)(item % L.bk) * Lr
                                  : (int64_t)item * L.np + rd.jofs;
    }
    __syncthreads();
    const int G = (nb + kSweepSeqs - 1) / kSweepSeqs;

    for (int d = 0; d < 3; d++) {
        // FAtransform!: a_re = c br - s bi, a_im = s br + c bi (phase_filter.jl:154-190)
        for (UnitWalk uw_(nk); uw_.g < (G); uw_.next()) {
        const int k = uw_.n, g = uw_.g;
            const cpx<T> cs = k > 0 ? ld_cplx<T>(L.phase, rd.phase + (k - 1)) : c_zero<T>();
#pragma unroll
            for (int t = 0; t < kSweepSeqs; t++) {
                const int b = g * kSweepSeqs + t;
                if (b >= nb) break;
                if (k > kmx[b]) continue;
                const T *gr = (const T *)L.in + ((size_t)d * L.nitems + item0 + b) * L.frows + rd.fofs;
                cpx<T> *X = Xs + (size_t)b * nk;
                if (k == 0) {
                    X[0] = {gr[0], T(0.0f)};
                } else {
                    const T br = gr[2 * k - 1], bi = gr[2 * k];
                    X[k] = {cs.x * br - cs.y * bi, cs.y * br + cs.x * bi};
                }
            }
        }
        __syncthreads();
        const int nvar = (d == 0) ? 3 : 1;
        for (int dl = 0; dl < nvar; dl++) {
            // packed spectrum Zp_k = E_k + i O_k, k < N (HC2R of length L via a length-N
            // inverse DFT).  With N = 2(ri + 1) > 2·kmax, entry k ≤ N/2 sees only X_k and
            // entry N − k only conj(X_k): for x = (iκ)^dl X_k (FIxcoefficients, κ = k)
            // and z = x·conj(W_L^k), Zp_k = x + i z and Zp_{N−k} = conj(x) + i conj(z) —
            // one spectrum load and one twiddle per pair
            const int NH = N / 2;
            for (UnitWalk uw_(NH + 1); uw_.g < (G); uw_.next()) {
                const int k = uw_.n, g = uw_.g;
                const cpx<T> uw = c_conj(ld_cplx<T>(L.pool, rd.utw + k));
                const float ka = (float)k;
#pragma unroll
                for (int t = 0; t < kSweepSeqs; t++) {
                    const int b = g * kSweepSeqs + t;
                    if (b >= nb) break;
                    cpx<T> x = c_zero<T>();
                    if (k <= kmx[b]) x = Xs[(size_t)b * nk + k];
                    if (dl == 1) {
                        x = {scale_f(x.y, -ka), scale_f(x.x, ka)};
                    } else if (dl == 2) {
                        x = {scale_f(scale_f(x.x, -ka), ka), scale_f(scale_f(x.y, -ka), ka)};
                    }
                    const cpx<T> z = c_mul(x, uw);
                    cpx<T> *Ab = A + (size_t)b * sq;
                    Ab[k] = {x.x - z.y, x.y + z.x};
                    if (k > 0 && k < NH) Ab[N - k] = {x.x + z.y, z.x - x.y};
                }
            }
            __syncthreads();
            cpx<T> *zb0 = dft<1, T>(A, B, pl, L.pool, nb, L.ib);
            int slot;  // 1-based physical slot
            if (d == 0) slot = (dl == 0) ? 1 : (dl == 1 ? 4 : 5);
            else slot = (d == 1) ? 2 : 3;
            const int var = (d == 0) ? dl : (d == 1 ? 3 : 4);  // H variant: 0 f, 1 ∂λ, 2 ∂λλ, 3 ∂r, 4 ∂rr
            const int64_t plane = L.rlz ? (int64_t)var * L.nvars * L.bk * L.jDim : (int64_t)(slot - 1) * L.nvars * L.np;
            for (UnitWalk uw_(N); uw_.g < (nb); uw_.next()) {
        const int n = uw_.n, b = uw_.g;
                const cpx<T> w = zb0[(size_t)b * sq + n];
                // even plane and ring offsets: points (2n, 2n+1) are one aligned pair
                if (L.rlz) {
                    reinterpret_cast<cpx<T> *>((T *)L.out + plane + ooff[b])[n] = w;
                } else {
                    reinterpret_cast<cpx<P> *>((P *)L.out + plane + ooff[b])[n] = {to_storage<P>(w.x), to_storage<P>(w.y)};
                }
            }
            __syncthreads();
        }
    }
}

template <typename P, typename T>
__global__ void __launch_bounds__(256, kRingMinBlocks<T>) ring_inverse_kernel(RingLaunch L) {
    ring_inverse_body<P, T>(L, blockIdx.x, blockIdx.y);
}

// ====================================================================
// sb_project: spectral[(zb*(1+2K) + s)*b + mi] = Σ_taps w(mi,tap) F[row][s]
// CTA = 32 slots × kSbOut outputs mi (8 rows of threads).  The F rows that the
// CTA's tap windows span (mubar·(kSbOut − 1) + 4·mubar of them) are staged once
// in shared memory with coalesced loads, zero where a ring has no such slot
// (k > ri: the reference zero-fills); each output then reads its 4·mubar taps
// from there.  Grids with mubar > kSbMaxMubar read F from global memory.
// ====================================================================
template <typename P, typename T>
__device__ __forceinline__ void sb_project_body(const SbLaunch &S, const int bx, const int by, const int bz) {
    constexpr int MO = kSbOut, FROWS = MO * kSbMaxMubar + 4 * kSbMaxMubar;
    __shared__ T fs[FROWS][32];
    __shared__ T tile[32][MO + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int s0 = bx * 32, m0 = by * MO;
    const int item = bz;
    const int v = item / S.bk, zb = item % S.bk;
    const int s = s0 + tx;
    const SplineDev &sp = S.spl[v];
    const int taps = 4 * S.mubar;
    const T *F = (const T *)S.F + (size_t)item * S.frows;
    if (S.mubar <= kSbMaxMubar) {
        const int rbase = S.mubar * (m0 - 3);  // tap 0 of output m0
        const int nrows = S.mubar * (MO - 1) + taps;
        for (int rr = ty; rr < nrows; rr += 8) {
            const int row = rbase + rr;  // radial mish index (0-based ring r-1)
            T val = T(0.0f);
            if (row >= 0 && row < S.iDim && s < S.nslots_z && s < 1 + 2 * (row + 1 + S.pOL)) val = F[S.fofs[row] + s];
            fs[rr][tx] = val;
        }
        __syncthreads();
        for (int q = 0; q < MO / 8; q++) {
            const int ml = ty + 8 * q, mi = m0 + ml;
            T acc = T(0.0f);
            if (mi < S.b) {
                const T *f = &fs[S.mubar * ml][tx];
                for (int t = 0; t < taps; t++) acc = acc + ld_real<T>(sp.sbw_t, (int64_t)mi * taps + t) * f[t * 32];
            }
            tile[tx][ml] = acc;
        }
    } else {
        for (int q = 0; q < MO / 8; q++) {
            const int mi = m0 + ty + 8 * q;
            T acc = T(0.0f);
            if (mi < S.b && s < S.nslots_z) {
                const int row0 = S.mubar * (mi - 3);
                for (int t = 0; t < taps; t++) {
                    const int row = row0 + t;
                    if (row < 0 || row >= S.iDim) continue;
                    const int ri = row + 1 + S.pOL;
                    if (s >= 1 + 2 * ri) continue;
                    acc = acc + ld_real<T>(sp.sbw_t, (int64_t)mi * taps + t) * F[S.fofs[row] + s];
                }
            }
            tile[tx][ty + 8 * q] = acc;
        }
    }
    __syncthreads();
    P *spec = (P *)S.spec + (size_t)v * S.nspec + (size_t)zb * S.nslots_z * S.b;
    const double *fw = S.fw ? S.fw + (size_t)v * (S.K + 1) : nullptr;
    const double *cw = S.cw ? S.cw + (size_t)v * S.bk : nullptr;
    const int tid = ty * 32 + tx;
    for (int e = tid; e < 32 * MO; e += 256) {
        const int sl = e / MO, ml = e % MO;
        const int ss = s0 + sl, mi = m0 + ml;
        if (ss < S.nslots_z && mi < S.b) {
            T val = tile[sl][ml];
            if (S.filtered) {
                const double wgt = (fw ? fw[(ss + 1) / 2] : 1.0) * (cw ? cw[zb] : 1.0);
                if (wgt != 1.0) val = (wgt == 0.0) ? T(0.0f) : val * to_compute<T>(wgt);
            }
            spec[(size_t)ss * S.b + mi] = to_storage<P>(val);
        }
    }
}

template <typename P, typename T>
__global__ void __launch_bounds__(256) sb_project_kernel(SbLaunch S) {
    sb_project_body<P, T>(S, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ====================================================================
// sa_si: per 32-slot tile, SAtransform! (src/CubicBSpline.jl:1368-1396)
//   FP64 modes: Γ b → L⁻ᵀL⁻¹ → Γᵀ (+ahat) in binary64;
//   FP32 mode:  binary32 solve with the FP32-rounded factor, then one FP64
//               refinement step: residual r = Γb − A x against the FP64
//               open-form matrix, correction solve with the FP64 factor,
//               x += dx;
// then the 4-tap SI/SIx/SIxx at the mish points in the compute type.
// ====================================================================
template <typename P, typename T>
__device__ __forceinline__ void sa_si_body(const SaLaunch &A, const int bx, const int by) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr bool kF32 = std::is_same<T, float>::value;
    using S = typename std::conditional<kF32, float, double>::type;  // solve type
    const int item = by;
    const int v = item / A.bk, zb = item % A.bk;
    const SplineDev &sp = A.spl[v];
    const int b = A.b, ld = A.ld, n = sp.Min;
    S *X = reinterpret_cast<S *>(smem_raw);  // 32 × ld
    S *Ls = X + 32 * ld;                     // 4n factor
    S *Di = Ls + 4 * n;                      // n reciprocals
    S *R = Di + n;                           // 32 × ld: FP32 residuals / df64 coefficients for SI
    constexpr bool kSameX = kF32 || std::is_same<T, double>::value;
    T *XT = kSameX ? reinterpret_cast<T *>(X) : reinterpret_cast<T *>(R);
    const int s0 = bx * 32;
    const P *spec = (const P *)A.spec + (size_t)v * A.nspec + ((size_t)zb * A.nslots_z + s0) * b;
    const int nsl = min(32, A.nslots_z - s0);
    for (int e = threadIdx.x; e < nsl * b; e += blockDim.x) X[(e / b) * ld + (e % b)] = (S)spec[e];
    for (int e = threadIdx.x; e < 4 * n; e += blockDim.x) Ls[e] = kF32 ? (S)sp.L4f[e] : (S)sp.L4[e];
    for (int e = threadIdx.x; e < n; e += blockDim.x) Di[e] = kF32 ? (S)sp.dinvf[e] : (S)sp.dinv[e];
    __syncthreads();

    if (threadIdx.x < nsl && A.coeffs) {
        if constexpr (!kSameX) {
            S *x = X + threadIdx.x * ld;
            T *xt = XT + threadIdx.x * ld;
            for (int i = 0; i < b; i++) xt[i] = to_compute<T>((double)x[i]);
        }
    } else if (threadIdx.x < nsl) {
        S *x = X + threadIdx.x * ld;
        const int Md = b;
        const double *ah = (sp.r3x && A.ahat)
                               ? A.ahat + ((size_t)v * A.nblocks + (size_t)zb * A.nslots_z + s0 + threadIdx.x) * b
                               : nullptr;
        if (ah) {
            // b̃ = b − PQ·ahat (PQ = full P+Q, band 3); row i only changes b_i
            for (int i = 0; i < Md; i++) {
                double acc = 0.0;
                for (int j = max(0, i - 3); j <= min(Md - 1, i + 3); j++) acc += sp.PQb[i * 7 + (j - i + 3)] * ah[j];
                x[i] = (S)((double)x[i] - acc);
            }
        }
        gamma_fold(sp, x, Md, n);
        if constexpr (kF32) {
            S *r = R + threadIdx.x * ld;
            for (int i = 0; i < n; i++) r[i] = x[i];  // keep Γb
            band_solve(Ls, Di, x, n, sp.periodic ? sp.tailf : nullptr);
            // one refinement step in FP64: residual r = Γb − A x against the FP64
            // open-form band (and, periodic, its corners), correction L Lᵀ c = r
            // with the FP64 factor (forward sweep into r, rounded to binary32
            // between the sweeps), x ← x + c rounded once
            const int r0 = sp.periodic ? n - 3 : n;
            double y1 = 0.0, y2 = 0.0, y3 = 0.0;
            for (int i = 0; i < n; i++) {
                double acc = (double)r[i];
                for (int j = max(0, i - 3); j <= min(n - 1, i + 3); j++)
                    acc -= __ldg(sp.Aband + min(i, j) * 4 + abs(i - j)) * (double)x[j];
                if (sp.periodic) {  // A[n−3+q][c] and its transpose, beyond the band
                    for (int c = 0; c < 3; c++) {
                        if (i >= r0) acc -= __ldg(sp.acorner + (i - r0) * 3 + c) * (double)x[c];
                        if (i < 3) acc -= __ldg(sp.acorner + c * 3 + i) * (double)x[r0 + c];
                    }
                }
                if (i >= r0) {
                    for (int j = 0; j < i; j++) acc -= __ldg(sp.tail + (size_t)(i - r0) * n + j) * (double)r[j];
                } else {
                    if (i >= 3) acc -= __ldg(sp.L4 + (i - 3) * 4 + 3) * y3;
                    if (i >= 2) acc -= __ldg(sp.L4 + (i - 2) * 4 + 2) * y2;
                    if (i >= 1) acc -= __ldg(sp.L4 + (i - 1) * 4 + 1) * y1;
                }
                const double yi = acc * __ldg(sp.dinv + i);
                r[i] = (S)yi;
                y3 = y2; y2 = y1; y1 = yi;
            }
            double c1 = 0.0, c2 = 0.0, c3 = 0.0, ct[3] = {0.0, 0.0, 0.0};  // ct: the tail rows' c
            for (int i = n - 1; i >= 0; i--) {
                double acc = (double)r[i];
                if (i + 1 < n) acc -= __ldg(sp.L4 + i * 4 + 1) * c1;
                if (i + 2 < n) acc -= __ldg(sp.L4 + i * 4 + 2) * c2;
                if (i + 3 < n) acc -= __ldg(sp.L4 + i * 4 + 3) * c3;
                if (sp.periodic)
                    for (int q = max(r0, i + 4); q < n; q++) acc -= __ldg(sp.tail + (size_t)(q - r0) * n + i) * ct[q - r0];
                const double ci = acc * __ldg(sp.dinv + i);
                if (i >= r0) ct[i - r0] = ci;
                c3 = c2; c2 = c1; c1 = ci;
                x[i] = (S)((double)x[i] + ci);
            }
        } else {
            band_solve(Ls, Di, x, n, sp.periodic ? sp.tail : nullptr);
        }
        gamma_unfold(sp, x, Md, n);
        if (ah)
            for (int i = 0; i < Md; i++) x[i] = (S)((double)x[i] + ah[i]);
        if constexpr (!kSameX) {
            T *xt = XT + threadIdx.x * ld;
            for (int i = 0; i < Md; i++) xt[i] = to_compute<T>((double)x[i]);
        }
    }
    __syncthreads();
    if (A.aout) {  // splineTransform!: the coefficients themselves, in the spectral layout
        P *out = (P *)A.aout + (size_t)v * A.nspec + ((size_t)zb * A.nslots_z + s0) * b;
        for (int e = threadIdx.x; e < nsl * b; e += blockDim.x) out[e] = (P)X[(e / b) * ld + (e % b)];
        return;
    }

    // SI at the iDim mish points for the slots each ring carries
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int s = s0 + lane;
    const T *xa = XT + lane * ld;
    for (int r = grp; r < A.iDim; r += 4) {
        const int ri = r + 1 + A.pOL;
        if (lane >= nsl || s >= 1 + 2 * ri) continue;
        const int m0 = sp.si_m0[r];
        const T a0 = xa[m0], a1 = xa[m0 + 1], a2 = xa[m0 + 2], a3 = xa[m0 + 3];
        const size_t orow = A.fofs[r] + s;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const int64_t w = ((int64_t)d * A.iDim + r) * 4;
            T u = ld_real<T>(sp.siw_t, w) * a0 + ld_real<T>(sp.siw_t, w + 1) * a1 +
                  ld_real<T>(sp.siw_t, w + 2) * a2 + ld_real<T>(sp.siw_t, w + 3) * a3;
            ((T *)A.G)[((size_t)d * A.nitems + item) * A.frows + orow] = u;
        }
    }
}

template <typename P, typename T>
__global__ void __launch_bounds__(128) sa_si_kernel(SaLaunch A) {
    sa_si_body<P, T>(A, blockIdx.x, blockIdx.y);
}

// ====================================================================
// cheb_forward: DCT-I of each kz-point column, scaled 1/(2(kz-1)), first bk modes
// (CBtransform!, src/Chebyshev.jl:417-426).  CTA = 64 consecutive columns.
// ====================================================================
// K consecutive shared-memory values (16-byte aligned rows: vector loads for float/double)
template <typename T, int K>
__device__ __forceinline__ void load_row(const T *p, T (&v)[K]) {
    if constexpr (std::is_same<T, float>::value && K % 4 == 0) {
#pragma unroll
        for (int q = 0; q < K / 4; q++) {
            const float4 x = reinterpret_cast<const float4 *>(p)[q];
            v[4 * q] = x.x; v[4 * q + 1] = x.y; v[4 * q + 2] = x.z; v[4 * q + 3] = x.w;
        }
    } else if constexpr (std::is_same<T, double>::value && K % 2 == 0) {
#pragma unroll
        for (int q = 0; q < K / 2; q++) {
            const double2 x = reinterpret_cast<const double2 *>(p)[q];
            v[2 * q] = x.x; v[2 * q + 1] = x.y;
        }
    } else {
#pragma unroll
        for (int c = 0; c < K; c++) v[c] = p[c];
    }
}

// ====================================================================
// cheb_forward, register-tiled: the CTA's 64 columns are staged (cp.async),
// folded into xe[j][c] = x_j + x_{N-1-j} and xo[j][c] = x_j − x_{N-1-j}
// (j < half; the middle point once), then out[k][c] = Σ_j FW[k][j] x{e,o}[j][c]
// as two small GEMMs (even and odd k) with 4 × 4 register tiles; the same
// per-output summation order (j ascending) as cheb_forward.  Results are staged
// k-major and stored per ring row (C[r][zb][l]) with consecutive columns
// contiguous.
// ====================================================================
template <typename P, typename T>
__global__ void __launch_bounds__(128) cheb_forward_tiled_kernel(ChebLaunch C) {
    constexpr int COLS = 64, TK = 4, TC = 4, CT = COLS / TC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t col_base[COLS];
    __shared__ int col_L[COLS];
    const int v = blockIdx.y;
    const ChebDev &cb = C.cheb[v];
    const int N = cb.N, bk = cb.bk, half = cb.half;
    const int ke = (bk + 1) / 2, ko = bk / 2;
    const int KEP = (ke + TK - 1) / TK * TK, KOP = (ko > 0 ? (ko + TK - 1) / TK : 1) * TK;
    const int ldx = N | 1;
    T *xe = reinterpret_cast<T *>(smem_raw);      // half × COLS
    T *xo = xe + (size_t)half * COLS;              // half × COLS
    T *fe = xo + (size_t)half * COLS;              // half × KEP: FW[2i][j] at fe[j][i]
    T *fo = fe + (size_t)half * KEP;               // half × KOP: FW[2i+1][j] at fo[j][i]
    T *xs = fo + (size_t)half * KOP;               // COLS × ldx staged columns; later bk × COLS outputs
    T *os = xs;
    // tables once per CTA (host-transposed: coalesced)
    for (int e = threadIdx.x; e < half * KEP; e += blockDim.x) fe[e] = ld_real<T>(cb.fwd_et_t, e);
    for (int e = threadIdx.x; e < half * KOP; e += blockDim.x) fo[e] = ld_real<T>(cb.fwd_ot_t, e);
    const int64_t nblk = (C.col1 - C.col0 + COLS - 1) / COLS;
    for (int64_t blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
    const int64_t c0 = C.col0 + blk * COLS;
    const int ncol = (int)((C.col1 - c0) < COLS ? (C.col1 - c0) : COLS);
    const P *in = (const P *)C.in + (size_t)v * C.np + c0 * N;
    // (point z, column c) walked with carries: no division per element
    if constexpr (std::is_same<P, T>::value) {
        for (UnitWalk u(N); u.g < ncol; u.next()) cp_async<sizeof(T)>(xs + u.g * ldx + u.n, in + u.g * N + u.n);
    } else {
        for (UnitWalk u(N); u.g < ncol; u.next()) xs[u.g * ldx + u.n] = to_compute<T>(in[u.g * N + u.n]);
    }
    for (int c = threadIdx.x; c < COLS; c += blockDim.x) {
        if (c < ncol) {
            const int64_t q = c0 + c;
            const RingDesc &rd = C.rings[C.col_ring[q]];
            col_base[c] = (int64_t)C.bk * rd.jofs + (q - rd.jofs);
            col_L[c] = rd.L;
        }
    }
    if constexpr (std::is_same<P, T>::value) cp_async_wait_all();
    __syncthreads();
    for (int e = threadIdx.x; e < half * COLS; e += blockDim.x) {
        const int j = e / COLS, c = e % COLS;
        T a = T(0.0f), b = T(0.0f);
        if (c < ncol) {
            const T *x = xs + c * ldx;
            const int jj = N - 1 - j;
            if (jj == j) { a = x[j]; b = x[j]; }
            else { a = x[j] + x[jj]; b = x[j] - x[jj]; }
        }
        xe[e] = a;
        xo[e] = b;
    }
    __syncthreads();
    const int KT = KEP / TK + KOP / TK;
    for (int t = threadIdx.x; t < KT * CT; t += blockDim.x) {
        const int ct = t % CT, kt = t / CT;
        const bool odd = kt >= KEP / TK;
        const int i0 = (odd ? kt - KEP / TK : kt) * TK, cc = ct * TC;
        const T *ft = odd ? fo : fe;
        const T *xt = odd ? xo : xe;
        const int KP = odd ? KOP : KEP;
        T acc[TK][TC];
#pragma unroll
        for (int i = 0; i < TK; i++)
#pragma unroll
            for (int c = 0; c < TC; c++) acc[i][c] = T(0.0f);
        for (int j = 0; j < half; j++) {
            T w[TK], x[TC];
            load_row<T, TK>(ft + (size_t)j * KP + i0, w);
            load_row<T, TC>(xt + (size_t)j * COLS + cc, x);
#pragma unroll
            for (int i = 0; i < TK; i++)
#pragma unroll
                for (int c = 0; c < TC; c++) acc[i][c] = acc[i][c] + w[i] * x[c];
        }
        // os aliases xs, which only the fold pass (before the last barrier) read
#pragma unroll
        for (int i = 0; i < TK; i++) {
            const int k = 2 * (i0 + i) + (odd ? 1 : 0);
            if (k < bk)
#pragma unroll
                for (int c = 0; c < TC; c++) os[(size_t)k * COLS + cc + c] = acc[i][c];
        }
    }
    __syncthreads();
    T *out = (T *)C.out + (size_t)v * C.bk * C.jDim;
    for (UnitWalk u(ncol); u.g < bk; u.next()) {  // column u.n of mode u.g
        const int k = u.g, c = u.n;
        out[col_base[c] + (int64_t)k * col_L[c]] = os[(size_t)k * COLS + c];
    }
    __syncthreads();  // os and col_base are rewritten by the next block
    }  // column blocks
}

template <typename T>
size_t cheb_forward_tiled_smem(int N, int bk) {
    const int half = (N + 1) / 2, ke = (bk + 1) / 2, ko = bk / 2;
    const int KEP = (ke + 3) / 4 * 4, KOP = (ko > 0 ? (ko + 3) / 4 : 1) * 4;
    const size_t stage = std::max((size_t)64 * (N | 1), (size_t)bk * 64);
    return ((size_t)2 * half * 64 + (size_t)half * (KEP + KOP) + stage) * sizeof(T);
}

// ====================================================================
// cheb_inverse as one GEMM per output: CA (Γ fold), the CIx recurrence and
// the folded DCT-I are linear, so each output column is u = M_d b with
// M_d = IDCT·(D/dscale)^d·G composed on the host in FP64 (ChebDev::inv_m_t).
// A CTA gathers the bk ring outputs of its 64 columns (cp.async, k-major) and
// runs, per output, Ue = Me·B and Uo = Mo·B with 4 × 4 register tiles (matrix
// rows read through L1, broadcast within a warp; B from shared memory), then
// u[j] = Ue + Uo, u[N-1-j] = Ue − Uo, staged for a coalesced store.  No serial
// per-column phase remains.  grid = (column blocks, variables, 5 ring variants);
// variant 0 (f) also writes ∂z and ∂zz.
// ====================================================================
template <typename P, typename T>
__global__ void __launch_bounds__(128) cheb_inverse_m_kernel(ChebLaunch C) {
    constexpr int COLS = 64, TJ = 4, TC = 4, CT = COLS / TC;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t col_base[COLS];
    __shared__ int col_L[COLS];
    const int v = blockIdx.y, var = blockIdx.z;
    const ChebDev &cb = C.cheb[v];
    const int N = cb.N, bk = cb.bk, half = cb.half;
    const int JT = (half + TJ - 1) / TJ, JP = JT * TJ;
    const int ldn = N | 1;
    const int nr = cb.nrank, Ke = (bk + 1) / 2 + nr, Ko = bk / 2 + nr;
    T *xe = reinterpret_cast<T *>(smem_raw);  // Ke × COLS: even inputs b_{2i'}, then s = Uᵀ b
    T *xo = xe + (size_t)Ke * COLS;            // Ko × COLS: odd inputs b_{2i'+1}, then s
    T *us = xo + (size_t)Ko * COLS;            // COLS × ldn outputs
    T *ms = us + (size_t)COLS * ldn;           // 2 × kcap × JP: M_d of both output halves
    const int64_t c0 = C.col0 + (int64_t)blockIdx.x * COLS;
    const int ncol = (int)((C.col1 - c0) < COLS ? (C.col1 - c0) : COLS);
    for (int c = threadIdx.x; c < COLS; c += blockDim.x) {
        if (c < ncol) {
            const int64_t q = c0 + c;
            const RingDesc &rd = C.rings[C.col_ring[q]];
            col_base[c] = (int64_t)C.bk * rd.jofs + (q - rd.jofs);
            col_L[c] = rd.L;
        }
    }
    __syncthreads();
    const T *H = (const T *)C.in + ((size_t)var * C.nvars + v) * C.bk * C.jDim;
    for (int e = threadIdx.x; e < bk * COLS; e += blockDim.x) {
        const int zb = e / COLS, col = e % COLS;
        T *dst = ((zb & 1) ? xo : xe) + (size_t)(zb >> 1) * COLS + col;
        if (col < ncol) cp_async<sizeof(T)>(dst, H + col_base[col] + (int64_t)zb * col_L[col]);
        else *dst = T(0.0f);
    }
    cp_async_wait_all();
    __syncthreads();
    // s_p = Σ_i gu[p][i] b_i (the rank term of the Γ fold), appended to both input
    // sets: one (column, p) per thread, even and odd inputs as two partial sums
    for (int t = threadIdx.x; t < COLS * nr; t += blockDim.x) {
        const int c = t % COLS, p = t / COLS;
        const int64_t g0 = (int64_t)p * bk;
        T se = T(0.0f), so = T(0.0f);
        for (int i2 = 0; 2 * i2 < bk; i2++) {
            se = se + ld_real<T>(cb.gu_t, g0 + 2 * i2) * xe[(size_t)i2 * COLS + c];
            if (2 * i2 + 1 < bk) so = so + ld_real<T>(cb.gu_t, g0 + 2 * i2 + 1) * xo[(size_t)i2 * COLS + c];
        }
        const T acc = se + so;
        xe[(size_t)((bk + 1) / 2 + p) * COLS + c] = acc;
        xo[(size_t)(bk / 2 + p) * COLS + c] = acc;
    }
    __syncthreads();
    const int nd = (var == 0) ? 3 : 1;
    const T *mtab = (const T *)cb.inv_m_t;
    for (int dd = 0; dd < nd; dd++) {
        // M_d of both halves into shared memory (16-byte copies: JP and kcap·JP are
        // multiples of 4 entries, so every row start is 16-byte aligned)
        {
            const int nm = 2 * cb.kcap * JP, per16 = 16 / (int)sizeof(T);
            const T *src = mtab + (int64_t)(dd * 2) * cb.kcap * JP;
            if (dd > 0) __syncthreads();  // the previous derivative's tiles have read ms
            for (int e = threadIdx.x * per16; e < nm; e += blockDim.x * per16) cp_async<16>(ms + e, src + e);
            cp_async_wait_all();
            __syncthreads();
        }
        // output half pe reads the inputs of parity (pe + dd) mod 2
        const int64_t me = 0, mo = (int64_t)cb.kcap * JP;
        const T *ie = (dd & 1) ? xo : xe, *io = (dd & 1) ? xe : xo;
        const int Kie = (dd & 1) ? Ko : Ke, Kio = (dd & 1) ? Ke : Ko;
        for (int t = threadIdx.x; t < JT * CT; t += blockDim.x) {
            const int ct = t % CT, jt = t / CT;
            const int j0 = jt * TJ, cc = ct * TC;
            T E[TJ][TC], O[TJ][TC];
#pragma unroll
            for (int i = 0; i < TJ; i++)
#pragma unroll
                for (int c = 0; c < TC; c++) { E[i][c] = T(0.0f); O[i][c] = T(0.0f); }
            for (int k = 0; k < Kie; k++) {
                T w[TJ], b[TC];
#pragma unroll
                load_row<T, TJ>(ms + me + (size_t)k * JP + j0, w);
                load_row<T, TC>(ie + (size_t)k * COLS + cc, b);
#pragma unroll
                for (int i = 0; i < TJ; i++)
#pragma unroll
                    for (int c = 0; c < TC; c++) E[i][c] = E[i][c] + w[i] * b[c];
            }
            for (int k = 0; k < Kio; k++) {
                T w[TJ], b[TC];
#pragma unroll
                load_row<T, TJ>(ms + mo + (size_t)k * JP + j0, w);
                load_row<T, TC>(io + (size_t)k * COLS + cc, b);
#pragma unroll
                for (int i = 0; i < TJ; i++)
#pragma unroll
                    for (int c = 0; c < TC; c++) O[i][c] = O[i][c] + w[i] * b[c];
            }
#pragma unroll
            for (int i = 0; i < TJ; i++) {
                const int j = j0 + i;
                if (j < half)
#pragma unroll
                    for (int c = 0; c < TC; c++) {
                        T *u = us + (size_t)(cc + c) * ldn;
                        u[j] = E[i][c] + O[i][c];
                        if (N - 1 - j != j) u[N - 1 - j] = E[i][c] - O[i][c];
                    }
            }
        }
        __syncthreads();
        int slot;
        if (var == 0) slot = (dd == 0) ? 1 : (dd == 1 ? 6 : 7);
        else slot = (var == 1) ? 4 : (var == 2 ? 5 : (var == 3 ? 2 : 3));
        P *dst = (P *)C.out + ((size_t)(slot - 1) * C.nvars + v) * C.np + c0 * N;
        const float inv_n = 1.0f / (float)N;
        for (int e = threadIdx.x; e < ncol * N; e += blockDim.x) {
            const int col = div_small(e, N, inv_n);
            dst[e] = to_storage<P>(us[col * ldn + (e - col * N)]);
        }
        __syncthreads();
    }
}

// TJ consecutive values from registers to global memory: 16-byte stores when the
// run is 16-byte aligned (`vec`), else one store per value
template <typename P, int TJ>
__device__ __forceinline__ void store_run(P *dst, const P (&u)[TJ], bool vec) {
    if constexpr ((TJ * sizeof(P)) % 16 == 0) {
        if (vec) {
#pragma unroll
            for (int q = 0; q < TJ * (int)sizeof(P) / 16; q++) {
                if constexpr (sizeof(P) == 4)
                    reinterpret_cast<float4 *>(dst)[q] = make_float4(u[4 * q], u[4 * q + 1], u[4 * q + 2], u[4 * q + 3]);
                else
                    reinterpret_cast<double2 *>(dst)[q] = make_double2(u[2 * q], u[2 * q + 1]);
            }
            return;
        }
    }
#pragma unroll
    for (int i = 0; i < TJ; i++) dst[i] = u[i];
}

// ====================================================================
// cheb_inverse, persistent: the same composed matrices u = M_d b as
// cheb_inverse_m_kernel, with M_0, M_1, M_2 of both output halves resident in
// shared memory for the CTA's life.  grid = (CTAs per variable, variables);
// each CTA walks work items (64-column block, ring variant), variants fastest,
// and gathers the next item's bk ring outputs (16-byte cp.async: four binary32
// or two binary64 columns of one ring row per copy) into the second buffer
// while it computes the current one.  The register tiles are TJ z-outputs ×
// TC columns, consecutive threads on consecutive z, so each u[j] run and its
// mirror u[N−1−j] leave registers as 16-byte stores covering whole sectors.
// Summation order per output is that of cheb_inverse_m_kernel (bit-identical).
// ====================================================================
// Columns per block of the persistent Chebyshev inverse.  (Measured on the
// 400-cell binary32 grid: tiles whose parity halves sit on lane pairs joined by
// shuffles ran slower — 23.5 ms with 8 × 8 tiles over 128 columns, 21.3 ms with
// 8 × 4 over 64 — than 4 × 4 tiles of both halves, 20.7 ms.)
template <typename T>
__host__ __device__ constexpr int cheb_inv_cols() { return 64; }

template <typename P, typename T>
__global__ void __launch_bounds__(128) cheb_inverse_p_kernel(ChebLaunch C) {
    // binary64 columns are short (kz = 32: JT = 4): 2-column tiles keep all 128
    // threads busy; binary32 (kz = 64: JT = 8) takes 4-column tiles
    constexpr int COLS = cheb_inv_cols<T>(), TJ = 4, TC = std::is_same<T, float>::value ? 4 : 2, CT = COLS / TC;
    constexpr int VEC = 16 / (int)sizeof(T);  // compute-type values per 16-byte copy
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int64_t col_base[COLS / VEC];
    __shared__ int col_L[COLS / VEC];
    const int v = blockIdx.y;
    const ChebDev &cb = C.cheb[v];
    const int N = cb.N, bk = cb.bk, half = cb.half;
    const int JT = (half + TJ - 1) / TJ, JP = JT * TJ;  // JP = pad4(half), the host layout
    const int nr = cb.nrank, ke = (bk + 1) / 2, ko = bk / 2, Ke = ke + nr, Ko = ko + nr;
    const int kcap = cb.kcap;
    T *ms = reinterpret_cast<T *>(smem_raw);    // [d][pe][kcap][JP]
    T *xbuf = ms + (size_t)6 * kcap * JP;       // 2 × [(Ke + Ko) × COLS]: even rows, then odd rows
    const int XS = (Ke + Ko) * COLS;
    const int64_t nblk = (C.col1 - C.col0 + COLS - 1) / COLS;
    const int64_t nitem = ((nblk - blockIdx.x + gridDim.x - 1) / gridDim.x) * 5;  // this CTA's items
    if (blockIdx.x >= nblk) return;
    constexpr int VP = 16 / (int)sizeof(P);
    const bool vec_ok = (N % VP) == 0 && (C.np % VP) == 0;
    {
        const int nm = 6 * kcap * JP;  // kcap·JP is a multiple of 4 entries: 16-byte rows
        const T *src = (const T *)cb.inv_m_t;
        for (int e = threadIdx.x * VEC; e < nm; e += blockDim.x * VEC) cp_async<16>(ms + e, src + e);
    }
    // column metadata of a block (one entry per VEC-column group: a group never
    // straddles a ring, whose starts and lengths are multiples of 4)
    auto meta = [&](int64_t blk) {
        const int64_t c0 = C.col0 + blk * COLS;
        for (int g = threadIdx.x; g < COLS / VEC; g += blockDim.x) {
            const int64_t q = c0 + (int64_t)g * VEC;
            if (q < C.col1) {
                const RingDesc &rd = C.rings[C.col_ring[q]];
                col_base[g] = (int64_t)C.bk * rd.jofs + (q - rd.jofs);
                col_L[g] = rd.L;
            }
        }
    };
    auto gather = [&](int64_t blk, int var, T *xb) {
        const int64_t c0 = C.col0 + blk * COLS;
        const int ng = (int)(((C.col1 - c0) < COLS ? (C.col1 - c0) : COLS) / VEC);
        const T *H = (const T *)C.in + ((size_t)var * C.nvars + v) * C.bk * C.jDim;
        for (int e = threadIdx.x; e < bk * (COLS / VEC); e += blockDim.x) {
            const int zb = e / (COLS / VEC), g = e % (COLS / VEC);
            T *dst = xb + ((zb & 1) ? (size_t)(Ke + (zb >> 1)) * COLS : (size_t)(zb >> 1) * COLS) + g * VEC;
            if (g < ng) {
                cp_async<16>(dst, H + col_base[g] + (int64_t)zb * col_L[g]);
            } else {
#pragma unroll
                for (int q = 0; q < VEC; q++) dst[q] = T(0.0f);
            }
        }
    };
    meta(blockIdx.x);
    __syncthreads();
    gather(blockIdx.x, 0, xbuf);
    asm volatile("cp.async.commit_group;" ::: "memory");
    for (int64_t it = 0; it < nitem; it++) {
        const int64_t blk = blockIdx.x + (it / 5) * gridDim.x;
        const int var = (int)(it % 5);
        T *xb = xbuf + (size_t)(it & 1) * XS;
        T *xe = xb, *xo = xb + (size_t)Ke * COLS;
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        __syncthreads();  // item it's inputs (and, at first, the matrices) are in; item it−1 is done
        // s_p = Σ_i gu[p][i] b_i (the rank term of the Γ fold), appended to both input sets
        for (int t = threadIdx.x; t < COLS * nr; t += blockDim.x) {
            const int c = t % COLS, p = t / COLS;
            const int64_t g0 = (int64_t)p * bk;
            T se = T(0.0f), so = T(0.0f);
            for (int i2 = 0; 2 * i2 < bk; i2++) {
                se = se + ld_real<T>(cb.gu_t, g0 + 2 * i2) * xe[(size_t)i2 * COLS + c];
                if (2 * i2 + 1 < bk) so = so + ld_real<T>(cb.gu_t, g0 + 2 * i2 + 1) * xo[(size_t)i2 * COLS + c];
            }
            const T acc = se + so;
            xe[(size_t)(ke + p) * COLS + c] = acc;
            xo[(size_t)(ko + p) * COLS + c] = acc;
        }
        const bool more = it + 1 < nitem;
        const int64_t nblk_next = blockIdx.x + ((it + 1) / 5) * gridDim.x;
        if (more && nblk_next != blk) meta(nblk_next);
        __syncthreads();  // rank rows and the next block's metadata are visible
        if (more) gather(nblk_next, (int)((it + 1) % 5), xbuf + (size_t)((it + 1) & 1) * XS);
        asm volatile("cp.async.commit_group;" ::: "memory");

        const int64_t c0 = C.col0 + blk * COLS;
        const int ncol = (int)((C.col1 - c0) < COLS ? (C.col1 - c0) : COLS);
        const int nd = (var == 0) ? 3 : 1;
        for (int dd = 0; dd < nd; dd++) {
            const T *me = ms + (size_t)(2 * dd) * kcap * JP, *mo = me + (size_t)kcap * JP;
            const T *ie = (dd & 1) ? xo : xe, *io = (dd & 1) ? xe : xo;
            const int Kie = (dd & 1) ? Ko : Ke, Kio = (dd & 1) ? Ke : Ko;
            int slot;
            if (var == 0) slot = (dd == 0) ? 1 : (dd == 1 ? 6 : 7);
            else slot = (var == 1) ? 4 : (var == 2 ? 5 : (var == 3 ? 2 : 3));
            P *dst = (P *)C.out + ((size_t)(slot - 1) * C.nvars + v) * C.np + c0 * N;
            for (int t = threadIdx.x; t < JT * CT; t += blockDim.x) {
                const int jt = t % JT, ct = t / JT;
                const int j0 = jt * TJ, cc = ct * TC;
                if (cc >= ncol) continue;
                T E[TJ][TC], O[TJ][TC];
#pragma unroll
                for (int i = 0; i < TJ; i++)
#pragma unroll
                    for (int c = 0; c < TC; c++) { E[i][c] = T(0.0f); O[i][c] = T(0.0f); }
                for (int k = 0; k < Kie; k++) {
                    T w[TJ], b[TC];
                    load_row<T, TJ>(me + (size_t)k * JP + j0, w);
                    load_row<T, TC>(ie + (size_t)k * COLS + cc, b);
#pragma unroll
                    for (int i = 0; i < TJ; i++)
#pragma unroll
                        for (int c = 0; c < TC; c++) E[i][c] = E[i][c] + w[i] * b[c];
                }
                for (int k = 0; k < Kio; k++) {
                    T w[TJ], b[TC];
                    load_row<T, TJ>(mo + (size_t)k * JP + j0, w);
                    load_row<T, TC>(io + (size_t)k * COLS + cc, b);
#pragma unroll
                    for (int i = 0; i < TJ; i++)
#pragma unroll
                        for (int c = 0; c < TC; c++) O[i][c] = O[i][c] + w[i] * b[c];
                }
                // whole run below the middle: u[j0..j0+TJ) and its mirror as two runs
                const bool full = j0 + TJ <= N - (j0 + TJ) && j0 + TJ <= half;
#pragma unroll
                for (int c = 0; c < TC; c++) {
                    if (cc + c >= ncol) break;
                    P *u = dst + (size_t)(cc + c) * N;
                    if (full) {
                        P lo[TJ], hi[TJ];
#pragma unroll
                        for (int i = 0; i < TJ; i++) {
                            lo[i] = to_storage<P>(E[i][c] + O[i][c]);
                            hi[TJ - 1 - i] = to_storage<P>(E[i][c] - O[i][c]);
                        }
                        store_run<P, TJ>(u + j0, lo, vec_ok);
                        store_run<P, TJ>(u + (N - TJ - j0), hi, vec_ok);
                    } else {
#pragma unroll
                        for (int i = 0; i < TJ; i++) {
                            const int j = j0 + i;
                            if (j >= half) break;
                            u[j] = to_storage<P>(E[i][c] + O[i][c]);
                            if (N - 1 - j != j) u[N - 1 - j] = to_storage<P>(E[i][c] - O[i][c]);
                        }
                    }
                }
            }
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

template <typename T>
size_t cheb_inverse_p_smem(int N, int bk) {  // rank of the Γ fold ≤ 2
    const size_t kcap = (size_t)(bk + 1) / 2 + 2, jp = (size_t)cheb_pad4((N + 1) / 2);
    const size_t kk = (size_t)(bk + 1) / 2 + bk / 2 + 4;
    return (6 * kcap * jp + 2 * kk * cheb_inv_cols<T>()) * sizeof(T);
}

template <typename T>
size_t cheb_inverse_m_smem(int N, int bk) {  // rank of the Γ fold ≤ 2: two s rows per input set
    const size_t kcap = (size_t)(bk + 1) / 2 + 2, jp = (size_t)cheb_pad4((N + 1) / 2);
    return ((size_t)(bk + 4) * 64 + (size_t)64 * (N | 1) + 2 * kcap * jp) * sizeof(T);
}

// ====================================================================
// fused multi-grid launches: CTA blockIdx.x runs work[blockIdx.x], the launch
// record it names staged in shared memory (one 4-byte word per thread)
// ====================================================================
template <typename R>
__device__ __forceinline__ void load_record(R &dst, const R *src) {
    static_assert(sizeof(R) % 4 == 0, "launch records are whole 4-byte words");
    const int tid = threadIdx.x + threadIdx.y * blockDim.x, nt = blockDim.x * blockDim.y;
    for (int i = tid; i < (int)(sizeof(R) / 4); i += nt)
        reinterpret_cast<int *>(&dst)[i] = __ldg(reinterpret_cast<const int *>(src) + i);
    __syncthreads();
}
template <typename P, typename T>
__global__ void __launch_bounds__(256, kRingMinBlocks<T>) ring_forward_fused_kernel(const RingLaunch *recs,
                                                                                    const BatchWork *work) {
    __shared__ __align__(16) RingLaunch L;
    const BatchWork w = work[blockIdx.x];
    load_record(L, recs + w.rec);
    ring_forward_body<P, T>(L, w.bx, w.by);
}
template <typename P, typename T>
__global__ void __launch_bounds__(256, kRingMinBlocks<T>) ring_inverse_fused_kernel(const RingLaunch *recs,
                                                                                    const BatchWork *work) {
    __shared__ __align__(16) RingLaunch L;
    const BatchWork w = work[blockIdx.x];
    load_record(L, recs + w.rec);
    ring_inverse_body<P, T>(L, w.bx, w.by);
}
template <typename P, typename T>
__global__ void __launch_bounds__(256) sb_project_fused_kernel(const SbLaunch *recs, const BatchWork *work) {
    __shared__ __align__(16) SbLaunch S;
    const BatchWork w = work[blockIdx.x];
    load_record(S, recs + w.rec);
    sb_project_body<P, T>(S, w.bx, w.by, w.bz);
}
template <typename P, typename T>
__global__ void __launch_bounds__(128) sa_si_fused_kernel(const SaLaunch *recs, const BatchWork *work) {
    __shared__ __align__(16) SaLaunch A;
    const BatchWork w = work[blockIdx.x];
    load_record(A, recs + w.rec);
    sa_si_body<P, T>(A, w.bx, w.by);
}

// ====================================================================
// launchers
// ====================================================================
// SMs of the current device (cached) and a CTA count that keeps them busy
static int sm_count() {
    static int cached[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 152;
    if (!cached[dev]) {
        int n = 0;
        cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
        cached[dev] = n > 0 ? n : 152;
    }
    return cached[dev];
}
static int resident_ctas(size_t smem, int threads) {
    int per = std::min(2048 / threads, 32);
    if (smem > 0) per = std::min<int>(per, (int)((227 * 1024) / (smem + 2048)));
    return sm_count() * std::max(per, 1);
}

template <typename K>
static void set_smem(K kernel, size_t smem) {
    if (smem > 48 * 1024) cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}
// `per_item`: shared-memory bytes of one item of the bucket's largest ring; a
// CTA takes L.ib items (1 when unset)
template <typename P, typename T>
cudaError_t launch_ring_forward(const RingLaunch &L0, int nrings, int nitems, size_t per_item, int threads,
                                cudaStream_t st) {
    RingLaunch L = L0;
    L.ib = std::max(1, std::min(L.ib, kRingBatchMax));
    const size_t smem = per_item * L.ib;
    set_smem(ring_forward_kernel<P, T>, smem);
    if (nrings > 65535) return cudaErrorInvalidConfiguration;  // rings index gridDim.y
    ring_forward_kernel<P, T><<<dim3((nitems + L.ib - 1) / L.ib, nrings), threads, smem, st>>>(L);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_ring_inverse(const RingLaunch &L0, int nrings, int nitems, size_t per_item, int threads,
                                cudaStream_t st) {
    RingLaunch L = L0;
    L.ib = std::max(1, std::min(L.ib, kRingBatchMax));
    const size_t smem = per_item * L.ib;
    set_smem(ring_inverse_kernel<P, T>, smem);
    if (nrings > 65535) return cudaErrorInvalidConfiguration;  // rings index gridDim.y
    ring_inverse_kernel<P, T><<<dim3((nitems + L.ib - 1) / L.ib, nrings), threads, smem, st>>>(L);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_ring_forward_fused(const RingLaunch *recs, const BatchWork *work, int nwork, size_t smem,
                                      int threads, cudaStream_t st) {
    if (nwork <= 0) return cudaSuccess;
    set_smem(ring_forward_fused_kernel<P, T>, smem);
    ring_forward_fused_kernel<P, T><<<nwork, threads, smem, st>>>(recs, work);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_ring_inverse_fused(const RingLaunch *recs, const BatchWork *work, int nwork, size_t smem,
                                      int threads, cudaStream_t st) {
    if (nwork <= 0) return cudaSuccess;
    set_smem(ring_inverse_fused_kernel<P, T>, smem);
    ring_inverse_fused_kernel<P, T><<<nwork, threads, smem, st>>>(recs, work);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_sb_project_fused(const SbLaunch *recs, const BatchWork *work, int nwork, cudaStream_t st) {
    if (nwork <= 0) return cudaSuccess;
    sb_project_fused_kernel<P, T><<<nwork, dim3(32, 8), 0, st>>>(recs, work);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_sa_si_fused(const SaLaunch *recs, const BatchWork *work, int nwork, size_t smem, cudaStream_t st) {
    if (nwork <= 0) return cudaSuccess;
    set_smem(sa_si_fused_kernel<P, T>, smem);
    sa_si_fused_kernel<P, T><<<nwork, 128, smem, st>>>(recs, work);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_sb_project(const SbLaunch &S, int nitems, cudaStream_t st) {
    dim3 grid((S.nslots_z + 31) / 32, (S.b + kSbOut - 1) / kSbOut, nitems);
    sb_project_kernel<P, T><<<grid, dim3(32, 8), 0, st>>>(S);
    return cudaGetLastError();
}
template <typename P, typename T>
cudaError_t launch_sa_si(const SaLaunch &A, int nitems, size_t smem, cudaStream_t st) {
    set_smem(sa_si_kernel<P, T>, smem);
    dim3 grid((A.nslots_z + 31) / 32, nitems);
    sa_si_kernel<P, T><<<grid, 128, smem, st>>>(A);
    return cudaGetLastError();
}
// the register-tiled kernel; `smem` (the one-MAC-per-load kernel's size) is unused
template <typename P, typename T>
cudaError_t launch_cheb_forward(const ChebLaunch &C, size_t smem, cudaStream_t st, int N) {
    (void)smem;
    const size_t sm = cheb_forward_tiled_smem<T>(N, C.bk);
    set_smem(cheb_forward_tiled_kernel<P, T>, sm);
    const int64_t nblk = (C.col1 - C.col0 + 63) / 64;
    if (nblk <= 0) return cudaSuccess;
    const int64_t want = std::max<int64_t>(1, (int64_t)resident_ctas(sm, 128) / std::max(C.nvars, 1));
    dim3 grid((unsigned)std::min(nblk, want), C.nvars);
    cheb_forward_tiled_kernel<P, T><<<grid, 128, sm, st>>>(C);
    return cudaGetLastError();
}
// the register-tiled kernel; `smem` (the 64-column kernel's size) is unused.
// N and bk are the grid's (every variable shares them).
template <typename P, typename T>
cudaError_t launch_cheb_inverse(const ChebLaunch &C, size_t smem, cudaStream_t st, int N) {
    (void)smem;
    if (C.col1 <= C.col0) return cudaSuccess;
    const size_t sp = cheb_inverse_p_smem<T>(N, C.bk);
    if (sp <= (size_t)227 * 1024) {  // the three matrices stay resident: persistent CTAs
        set_smem(cheb_inverse_p_kernel<P, T>, sp);
        constexpr int cols = cheb_inv_cols<T>();
        const int64_t nblk = (C.col1 - C.col0 + cols - 1) / cols;
        const int64_t want = std::max<int64_t>(1, (int64_t)resident_ctas(sp, 128) / std::max(C.nvars, 1));
        cheb_inverse_p_kernel<P, T><<<dim3((unsigned)std::min(nblk, want), C.nvars), 128, sp, st>>>(C);
        return cudaGetLastError();
    }
    // long columns: one matrix at a time, one CTA per (block, variable, variant)
    const size_t sm = cheb_inverse_m_smem<T>(N, C.bk);
    set_smem(cheb_inverse_m_kernel<P, T>, sm);
    if (C.col1 <= C.col0) return cudaSuccess;
    dim3 grid((unsigned)((C.col1 - C.col0 + 63) / 64), C.nvars, 5);
    cheb_inverse_m_kernel<P, T><<<grid, 128, sm, st>>>(C);
    return cudaGetLastError();
}

// ====================================================================
// RL chain coupling: SA of 32 primary slots per CTA (FP64), the three
// interface coefficients, times the 3×3 coupling matrix
// (COUPLING_MATRIX_1X / _2X, src/multipatch.jl:21-33).
// ====================================================================
template <typename P>
__global__ void __launch_bounds__(32) chain_couple_kernel(ChainLaunch C) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int item = blockIdx.y, v = item / C.bk, zb = item - v * C.bk;  // RLZ: every Chebyshev level
    const SplineDev &sp = C.spl[v];
    const int b = C.b_p, ld = C.ld, n = sp.Min;
    double *X = reinterpret_cast<double *>(smem_raw);
    double *Ls = X + 32 * ld;
    double *Di = Ls + 4 * n;
    const int q0 = blockIdx.x * 32;
    const int nsl = min(32, C.nq - q0);
    const P *spec = (const P *)C.spec + (size_t)v * C.nspec_p + ((size_t)zb * C.zblk_p + q0) * b;
    for (int e = threadIdx.x; e < nsl * b; e += blockDim.x) X[(e / b) * ld + (e % b)] = (double)spec[e];
    for (int e = threadIdx.x; e < 4 * n; e += blockDim.x) Ls[e] = sp.L4[e];
    for (int e = threadIdx.x; e < n; e += blockDim.x) Di[e] = sp.dinv[e];
    __syncthreads();
    if (threadIdx.x < nsl) {
        double *x = X + threadIdx.x * ld;
        // an R3X primary solves with its spline object's background, as
        // SAtransform!(spline) does: k0 / real / imag objects by slot parity
        const int q = q0 + threadIdx.x;
        const double *ah = (sp.r3x && C.pstate) ? C.pstate + ((size_t)v * 3 + (q == 0 ? 0 : ((q & 1) ? 1 : 2))) * b
                                                : nullptr;
        if (ah)  // b̃ = b − PQ·ahat (full P+Q band)
            for (int i = 0; i < b; i++) {
                double acc = 0.0;
                for (int j = max(0, i - 3); j <= min(b - 1, i + 3); j++) acc += sp.PQb[i * 7 + (j - i + 3)] * ah[j];
                x[i] -= acc;
            }
        gamma_fold(sp, x, b, n);
        band_solve(Ls, Di, x, n, sp.periodic ? sp.tail : nullptr);
        gamma_unfold(sp, x, b, n);
        if (ah)
            for (int i = 0; i < b; i++) x[i] += ah[i];
        const double e0 = x[C.node[0]], e1 = x[C.node[1]], e2 = x[C.node[2]];
        double *out = C.coupled + ((size_t)item * C.nq + q0 + threadIdx.x) * 3;
        for (int r = 0; r < 3; r++) out[r] = C.C[r * 3] * e0 + C.C[r * 3 + 1] * e1 + C.C[r * 3 + 2] * e2;
    }
}

// registry[z_b, q] = (spline-object ahat with this interface's side replaced by
// the coupled values of that slot): _write_interface_ahat! + _set_wavenumber_ahat!
// copy the whole shared ahat vector, src/multipatch.jl:433-476 (RL), 522-569 (RLZ,
// registry block z_b·(1+2K_s) + q)
__global__ void chain_assemble_kernel(ChainLaunch C) {
    const int64_t total = (int64_t)C.nvars * C.bk * C.nq * C.b_s;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % C.b_s);
        const int q = (int)((e / C.b_s) % C.nq);
        const int item = (int)(e / ((int64_t)C.b_s * C.nq));
        const int v = item / C.bk, zb = item - v * C.bk;
        const int obj = (q == 0) ? 0 : ((q & 1) ? 1 : 2);
        double val = C.state[((size_t)v * 3 + obj) * C.b_s + i];
        const double *cp = C.coupled + ((size_t)item * C.nq + q) * 3;
        if (C.side == 0 && i < 3) val = cp[i];
        if (C.side == 1 && i >= C.b_s - 3) val = cp[i - (C.b_s - 3)];
        C.reg[((size_t)v * C.nblocks_s + (size_t)zb * C.zblk_s + q) * C.b_s + i] = val;
    }
}
// after the loops over levels and wavenumbers each spline object keeps the
// values of its last slot (the last level's)
__global__ void chain_state_kernel(ChainLaunch C) {
    const int v = blockIdx.x, obj = threadIdx.x / 3, r = threadIdx.x % 3;
    if (v >= C.nvars || obj >= 3) return;
    int q_last = -1;
    if (obj == 0) q_last = 0;
    else if (C.nq >= 3) q_last = (obj == 1) ? C.nq - 2 : C.nq - 1;
    if (q_last < 0) return;
    double *st = C.state + ((size_t)v * 3 + obj) * C.b_s + (C.side == 0 ? 0 : C.b_s - 3);
    st[r] = C.coupled[(((size_t)v * C.bk + C.bk - 1) * C.nq + q_last) * 3 + r];
}

template <typename P>
cudaError_t launch_chain_couple(const ChainLaunch &C, size_t smem, cudaStream_t st) {
    set_smem(chain_couple_kernel<P>, smem);
    chain_couple_kernel<P><<<dim3((C.nq + 31) / 32, C.nvars * C.bk), 32, smem, st>>>(C);
    return cudaGetLastError();
}
cudaError_t launch_chain_assemble(const ChainLaunch &C, cudaStream_t st) {
    const int64_t total = (int64_t)C.nvars * C.bk * C.nq * C.b_s;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 4096);
    chain_assemble_kernel<<<blocks, 256, 0, st>>>(C);
    chain_state_kernel<<<C.nvars, 9, 0, st>>>(C);
    return cudaGetLastError();
}
template cudaError_t launch_chain_couple<double>(const ChainLaunch &, size_t, cudaStream_t);
template cudaError_t launch_chain_couple<float>(const ChainLaunch &, size_t, cudaStream_t);

// ====================================================================
// tile halo sum: patch spectral blocks += tile spectral blocks at the tile's
// spectralIndexL offset (sumSpectralTile!); set = 1 overwrites instead.
// ====================================================================
template <typename P>
__global__ void tile_sum_kernel(TileLaunch T) {
    const int64_t per_var = (int64_t)T.bk * T.blocks_t * T.b_t;
    const int64_t total = per_var * T.nvars;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total; e += (int64_t)gridDim.x * blockDim.x) {
        const int v = (int)(e / per_var);
        int64_t r = e % per_var;
        const int m = (int)(r % T.b_t);
        r /= T.b_t;
        const int blk = (int)(r % T.blocks_t);
        const int zb = (int)(r / T.blocks_t);
        const P tv = ((const P *)T.tile)[(size_t)v * T.nspec_t + ((size_t)zb * T.blocks_t + blk) * T.b_t + m];
        P *pp = (P *)T.patch + (size_t)v * T.nspec_p + ((size_t)zb * T.blocks_p + blk) * T.b_p + T.offset + m;
        *pp = T.set ? tv : (*pp + tv);
    }
}
template <typename P>
cudaError_t launch_tile_sum(const TileLaunch &T, cudaStream_t st) {
    const int64_t total = (int64_t)T.bk * T.blocks_t * T.b_t * T.nvars;
    const int blocks = (int)std::min<int64_t>((total + 255) / 256, 8192);
    tile_sum_kernel<P><<<blocks, 256, 0, st>>>(T);
    return cudaGetLastError();
}
template cudaError_t launch_tile_sum<double>(const TileLaunch &, cudaStream_t);
template cudaError_t launch_tile_sum<float>(const TileLaunch &, cudaStream_t);

#define SS_INSTANTIATE(P, T)                                                                                 \
    template cudaError_t launch_ring_forward_fused<P, T>(const RingLaunch *, const BatchWork *, int, size_t, int, \
                                                         cudaStream_t);                                          \
    template cudaError_t launch_ring_inverse_fused<P, T>(const RingLaunch *, const BatchWork *, int, size_t, int, \
                                                         cudaStream_t);                                          \
    template cudaError_t launch_sb_project_fused<P, T>(const SbLaunch *, const BatchWork *, int, cudaStream_t);   \
    template cudaError_t launch_sa_si_fused<P, T>(const SaLaunch *, const BatchWork *, int, size_t, cudaStream_t); \
    template cudaError_t launch_ring_forward<P, T>(const RingLaunch &, int, int, size_t, int, cudaStream_t); \
    template cudaError_t launch_ring_inverse<P, T>(const RingLaunch &, int, int, size_t, int, cudaStream_t); \
    template cudaError_t launch_sb_project<P, T>(const SbLaunch &, int, cudaStream_t);                      \
    template cudaError_t launch_sa_si<P, T>(const SaLaunch &, int, size_t, cudaStream_t);                   \
    template cudaError_t launch_cheb_forward<P, T>(const ChebLaunch &, size_t, cudaStream_t, int);               \
    template cudaError_t launch_cheb_inverse<P, T>(const ChebLaunch &, size_t, cudaStream_t, int);
SS_INSTANTIATE(double, double)
SS_INSTANTIATE(double, df64)
SS_INSTANTIATE(float, float)

}  // namespace ss
