// ss_kernels.cu — sm_103a kernels of the RL/RLZ transform path.
//
// Data flow of one variable (RL: b_kDim = 1, no column stages):
//   spectralTransform!  (src/transforms_cylindrical.jl:159-222, 530-618)
//     cheb_forward   physical slot 1 columns (kz) → C[r][zb][l]      (CBtransform!)
//     ring_forward   ring R2HC + 1/L + phase rotation → F rows       (FBtransform!)
//     sb_project     12-tap B-spline projection per slot → spectral  (SBtransform!)
//   gridTransform!     (src/transforms_cylindrical.jl:259-428, 659-853)
//     sa_si          Γ fold + banded LLᵀ solve (FP64 factor) + Γᵀ (+ahat),
//                    then f, ∂r, ∂rr at the mish points → G rows    (SAtransform!, SI*)
//     ring_inverse   phase rotation back + HC2R for f, ∂λ, ∂λλ, ∂r, ∂rr
//     cheb_inverse   CA (Γ fold) + DCT-I for each ring output; f column also ∂z, ∂zz
//
// Packed coefficient rows: ring r (ri = r + patchOffsetL) owns 1+2ri entries
// [DC, re1, im1, re2, im2, …] — the order of the reference's spectral slots.
#include <cuda_runtime.h>

#include <cstdio>

#include "ss_fft.cuh"
#include "ss_kernels.h"

namespace ss {

// ------------------------------------------------------------ constants
void fft_init_constants() {
    static bool done = false;
    if (done) return;
    double c[14][14] = {}, s[14][14] = {};
    for (int R = 2; R < 14; R++)
        for (int j = 0; j < R; j++) {
            double a = -2.0 * 3.14159265358979323846 * j / R;  // exp(-2πi j/R) = cos a + i sin a
            c[R][j] = cos(a);
            s[R][j] = -sin(a);  // sin(2π j/R)
        }
    cudaMemcpyToSymbol(c_rcos, c, sizeof c);
    cudaMemcpyToSymbol(c_rsin, s, sizeof s);
    done = true;
}

// ====================================================================
// ring_forward: one CTA per (ring, item); item = v*bk + zb
// ====================================================================
template <typename T>
__global__ void __launch_bounds__(256) ring_forward_kernel(RingLaunch L) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ring = L.ring_list[blockIdx.x];
    const int item = blockIdx.y;
    const int vv = L.rlz ? item / L.bk : item;
    const RingDesc rd = L.rings[(size_t)vv * L.ring_var_stride + ring];
    const FftPlan &pl = L.plans[rd.plan];
    const int buf = fft_buffer_len(pl);
    cpx<T> *A = reinterpret_cast<cpx<T> *>(smem_raw);
    cpx<T> *B = A + buf;
    const int Lr = rd.L, N = Lr / 2;

    const T *in;
    if (L.rlz) {
        const int v = item / L.bk, zb = item % L.bk;
        in = (const T *)L.in + (size_t)v * L.bk * L.jDim + (size_t)L.bk * rd.jofs + (size_t)zb * Lr;
    } else {
        in = (const T *)L.in + (size_t)item * L.in_item_stride + rd.jofs;
    }
    for (int n = threadIdx.x; n < N; n += blockDim.x) A[n] = {in[2 * n], in[2 * n + 1]};
    __syncthreads();
    cpx<T> *Z = dft<-1, T>(A, B, pl, L.pool);

    T *out = (T *)L.out + (size_t)item * L.frows + rd.fofs;
    const double2 *ph = L.phase + rd.phase;
    const T invL = T(1.0) / T(Lr);
    for (int k = threadIdx.x; k <= rd.ri; k += blockDim.x) {
        cpx<T> zk = Z[k];
        cpx<T> zn = c_conj(Z[(N - k) % N]);
        if (k == 0) {
            out[0] = (zk.x + zk.y) * invL;
            continue;
        }
        T bre = T(0), bim = T(0);
        if (k <= rd.kmax) {
            cpx<T> e = {T(0.5) * (zk.x + zn.x), T(0.5) * (zk.y + zn.y)};
            cpx<T> d = {T(0.5) * (zk.x - zn.x), T(0.5) * (zk.y - zn.y)};
            cpx<T> o = {d.y, -d.x};  // d / i
            cpx<T> X = c_add(e, c_mul(load_tw<T>(L.pool + rd.utw, k), o));
            T re = X.x * invL, im = X.y * invL;
            double2 cs = __ldg(ph + (k - 1));
            T c = (T)cs.x, s = (T)cs.y;
            bre = c * re + s * im;
            bim = -s * re + c * im;
        }
        out[2 * k - 1] = bre;
        out[2 * k] = bim;
    }
}

// ====================================================================
// ring_inverse: one CTA per (ring, item).  For d = 0 (value), 1 (∂r), 2 (∂rr)
// read the ring's coefficient row, undo the phase rotation (FAtransform!),
// and run HC2R for the variants: d=0 → f, ∂λ, ∂λλ; d=1 → ∂r; d=2 → ∂rr.
// ====================================================================
template <typename T>
__global__ void __launch_bounds__(256) ring_inverse_kernel(RingLaunch L) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ring = L.ring_list[blockIdx.x];
    const int item = blockIdx.y;
    const int v = L.rlz ? item / L.bk : item;
    const int zb = L.rlz ? item % L.bk : 0;
    const RingDesc rd = L.rings[(size_t)v * L.ring_var_stride + ring];
    const FftPlan &pl = L.plans[rd.plan];
    const int buf = fft_buffer_len(pl);
    cpx<T> *A = reinterpret_cast<cpx<T> *>(smem_raw);
    cpx<T> *B = A + buf;
    cpx<T> *Xs = B + buf;  // rotated spectrum X_k, k = 0..kmax
    const int Lr = rd.L, N = Lr / 2, kmax = rd.kmax;
    const double2 *ph = L.phase + rd.phase;

    for (int d = 0; d < 3; d++) {
        const T *g = (const T *)L.in + ((size_t)d * L.nitems + item) * L.frows + rd.fofs;
        // FAtransform!: a_re = c br - s bi, a_im = s br + c bi (phase_filter.jl:154-190)
        for (int k = threadIdx.x; k <= kmax; k += blockDim.x) {
            if (k == 0) {
                Xs[0] = {g[0], T(0)};
            } else {
                T br = g[2 * k - 1], bi = g[2 * k];
                double2 cs = __ldg(ph + (k - 1));
                T c = (T)cs.x, s = (T)cs.y;
                Xs[k] = {c * br - s * bi, s * br + c * bi};
            }
        }
        __syncthreads();
        const int nvar = (d == 0) ? 3 : 1;
        for (int dl = 0; dl < nvar; dl++) {
            // packed spectrum Zp_k = E_k + i O_k, k < N (HC2R of length L via length-N inverse DFT)
            for (int k = threadIdx.x; k < N; k += blockDim.x) {
                cpx<T> xa = {T(0), T(0)}, xb = {T(0), T(0)};
                if (k <= kmax) xa = Xs[k];
                if (N - k <= kmax && k > 0) xb = c_conj(Xs[N - k]);
                if (dl > 0) {
                    // FIxcoefficients: X_k → i k X_k (twice for ∂λλ)
                    T ka = T(k), kb = T(k) - T(N);  // signed wavenumber of index k+N is k+N-L = k-N
                    if (dl == 1) {
                        xa = {-ka * xa.y, ka * xa.x};
                        xb = {-kb * xb.y, kb * xb.x};
                    } else {
                        xa = {-ka * ka * xa.x, -ka * ka * xa.y};
                        xb = {-kb * kb * xb.x, -kb * kb * xb.y};
                    }
                }
                cpx<T> e = c_add(xa, xb);
                cpx<T> o = c_mul(c_sub(xa, xb), c_conj(load_tw<T>(L.pool + rd.utw, k)));
                A[k] = {e.x - o.y, e.y + o.x};
            }
            __syncthreads();
            cpx<T> *z = dft<1, T>(A, B, pl, L.pool);
            T *dst;
            int slot;  // 1-based physical slot (RL) / ring variant (RLZ)
            if (d == 0) slot = (dl == 0) ? 1 : (dl == 1 ? 4 : 5);
            else slot = (d == 1) ? 2 : 3;
            if (L.rlz) {
                // H[variant][v][r][zb][l], variant: 0 f, 1 ∂λ, 2 ∂λλ, 3 ∂r, 4 ∂rr
                int var = (d == 0) ? dl : (d == 1 ? 3 : 4);
                dst = (T *)L.out + ((size_t)var * L.nvars + v) * L.bk * L.jDim + (size_t)L.bk * rd.jofs +
                      (size_t)zb * Lr;
            } else {
                dst = (T *)L.out + ((size_t)(slot - 1) * L.nvars + v) * L.np + rd.jofs;
            }
            for (int n = threadIdx.x; n < N; n += blockDim.x) {
                cpx<T> w = z[n];
                dst[2 * n] = w.x;
                dst[2 * n + 1] = w.y;
            }
            __syncthreads();
        }
    }
}

// ====================================================================
// sb_project: spectral[(zb*(1+2K) + s)*b + mi] = Σ_taps w(mi,tap) F[row][s]
// block (32 slots, 8 rows of outputs); 64 outputs per CTA in mi
// ====================================================================
template <typename T>
__global__ void __launch_bounds__(256) sb_project_kernel(SbLaunch P) {
    __shared__ T tile[32][65];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int s0 = blockIdx.x * 32, m0 = blockIdx.y * 64;
    const int item = blockIdx.z;
    const int v = item / P.bk, zb = item % P.bk;
    const int s = s0 + tx;
    const SplineDev &sp = P.spl[v];
    const int taps = 4 * P.mubar;
    const T *F = (const T *)P.F + (size_t)item * P.frows;
    for (int q = 0; q < 8; q++) {
        const int mi = m0 + ty + 8 * q;
        T acc = T(0);
        if (mi < P.b && s < P.nslots_z) {
            const double *w = sp.sbw + (size_t)mi * taps;
            const int row0 = P.mubar * (mi - 3);
            for (int t = 0; t < taps; t++) {
                const int row = row0 + t;  // radial mish index (0-based ring r-1)
                if (row < 0 || row >= P.iDim) continue;
                const int ri = row + 1 + P.pOL;
                if (s >= 1 + 2 * ri) continue;  // wavenumber k > ri: reference zero-fills
                acc += (T)__ldg(w + t) * F[P.fofs[row] + s];
            }
        }
        tile[tx][ty + 8 * q] = acc;
    }
    __syncthreads();
    T *spec = (T *)P.spec + (size_t)v * P.nspec + (size_t)zb * P.nslots_z * P.b;
    const double *fw = P.fw ? P.fw + (size_t)v * (P.K + 1) : nullptr;
    const double *cw = P.cw ? P.cw + (size_t)v * P.bk : nullptr;
    const int tid = ty * 32 + tx;
    for (int e = tid; e < 32 * 64; e += 256) {
        const int sl = e / 64, ml = e % 64;
        const int ss = s0 + sl, mi = m0 + ml;
        if (ss < P.nslots_z && mi < P.b) {
            T val = tile[sl][ml];
            if (P.filtered) {
                double wgt = (fw ? fw[(ss + 1) / 2] : 1.0) * (cw ? cw[zb] : 1.0);
                if (wgt != 1.0) val = (wgt == 0.0) ? T(0) : val * (T)wgt;
            }
            spec[(size_t)ss * P.b + mi] = val;
        }
    }
}

// ====================================================================
// sa_si: per 32-slot tile: Γ b → L⁻ᵀL⁻¹ → Γᵀ (+ahat) in FP64 (SAtransform!,
// src/CubicBSpline.jl:1368-1396) then 4-tap SI/SIx/SIxx at the mish points.
// ====================================================================
template <typename T>
__global__ void __launch_bounds__(128) sa_si_kernel(SaLaunch P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int item = blockIdx.y;
    const int v = item / P.bk, zb = item % P.bk;
    const SplineDev &sp = P.spl[v];
    const int b = P.b, ld = P.ld, n = sp.Min;
    double *X = reinterpret_cast<double *>(smem_raw);  // 32 × ld
    double *Ls = X + 32 * ld;                          // 4n factor
    double *Di = Ls + 4 * n;                           // n reciprocals
    const int s0 = blockIdx.x * 32;
    const T *spec = (const T *)P.spec + (size_t)v * P.nspec + ((size_t)zb * P.nslots_z + s0) * b;
    const int nsl = min(32, P.nslots_z - s0);
    for (int e = threadIdx.x; e < nsl * b; e += blockDim.x) X[(e / b) * ld + (e % b)] = (double)spec[e];
    for (int e = threadIdx.x; e < 4 * n; e += blockDim.x) Ls[e] = sp.L4[e];
    for (int e = threadIdx.x; e < n; e += blockDim.x) Di[e] = sp.dinv[e];
    __syncthreads();

    if (threadIdx.x < nsl) {
        double *x = X + threadIdx.x * ld;
        const int Md = b, rL = sp.rankL;
        if (sp.r3x && P.ahat) {
            const double *ah = P.ahat + ((size_t)v * P.nblocks + (size_t)zb * P.nslots_z + s0 + threadIdx.x) * b;
            // b̃ = b − PQ·ahat (PQ = full P+Q, band 3); row i only changes b_i
            for (int i = 0; i < Md; i++) {
                double acc = 0.0;
                for (int j = max(0, i - 3); j <= min(Md - 1, i + 3); j++) acc += sp.PQb[i * 7 + (j - i + 3)] * ah[j];
                x[i] = x[i] - acc;
            }
        }
        // Γ b (src/CubicBSpline.jl:427-458)
        const double b0 = x[0], b1 = x[1], bM1 = x[Md - 1], bM2 = x[Md - 2];
        for (int i = 0; i < n; i++) x[i] = x[i + rL];
        if (sp.lk == BC_A1) { x[0] += sp.aL * b0; x[1] += sp.bL * b0; }
        else if (sp.lk == BC_A2) { x[0] += sp.aL * b0 + sp.bL * b1; }
        if (sp.rk == BC_A1) { x[n - 1] += sp.aR * bM1; x[n - 2] += sp.bR * bM1; }
        else if (sp.rk == BC_A2) { x[n - 1] += sp.aR * bM1 + sp.bR * bM2; }
        // forward L y = Γb, backward Lᵀ x = y (src/banded_cholesky.jl:202-231)
        double y1 = 0, y2 = 0, y3 = 0;  // y[i-1], y[i-2], y[i-3]
        for (int i = 0; i < n; i++) {
            double sacc = x[i];
            if (i >= 3) sacc -= Ls[(i - 3) * 4 + 3] * y3;
            if (i >= 2) sacc -= Ls[(i - 2) * 4 + 2] * y2;
            if (i >= 1) sacc -= Ls[(i - 1) * 4 + 1] * y1;
            double yi = sacc * Di[i];
            x[i] = yi;
            y3 = y2; y2 = y1; y1 = yi;
        }
        double x1 = 0, x2 = 0, x3 = 0;  // x[i+1], x[i+2], x[i+3]
        for (int i = n - 1; i >= 0; i--) {
            double sacc = x[i];
            if (i + 1 < n) sacc -= Ls[i * 4 + 1] * x1;
            if (i + 2 < n) sacc -= Ls[i * 4 + 2] * x2;
            if (i + 3 < n) sacc -= Ls[i * 4 + 3] * x3;
            double xi = sacc * Di[i];
            x[i] = xi;
            x3 = x2; x2 = x1; x1 = xi;
        }
        // Γᵀ x (src/CubicBSpline.jl:461-500)
        const double s0v = x[0], s1v = x[1], sM1 = x[n - 1], sM2 = x[n - 2];
        for (int i = n - 1; i >= 0; i--) x[i + rL] = x[i];
        for (int j = 0; j < rL; j++) x[j] = 0.0;
        for (int j = Md - sp.rankR; j < Md; j++) x[j] = 0.0;
        if (sp.lk == BC_A1) x[0] = sp.aL * s0v + sp.bL * s1v;
        else if (sp.lk == BC_A2) { x[0] = sp.aL * s0v; x[1] = sp.bL * s0v; }
        if (sp.rk == BC_A1) x[Md - 1] = sp.aR * sM1 + sp.bR * sM2;
        else if (sp.rk == BC_A2) { x[Md - 2] = sp.bR * sM1; x[Md - 1] = sp.aR * sM1; }
        if (sp.r3x && P.ahat) {
            const double *ah = P.ahat + ((size_t)v * P.nblocks + (size_t)zb * P.nslots_z + s0 + threadIdx.x) * b;
            for (int i = 0; i < Md; i++) x[i] += ah[i];
        }
    }
    __syncthreads();

    // SI at the iDim mish points for the slots each ring carries
    const int lane = threadIdx.x & 31, grp = threadIdx.x >> 5;
    const int s = s0 + lane;
    const double *xa = X + lane * ld;
    for (int r = grp; r < P.iDim; r += 4) {
        const int ri = r + 1 + P.pOL;
        if (lane >= nsl || s >= 1 + 2 * ri) continue;
        const int m0 = sp.si_m0[r];
        const double a0 = xa[m0], a1 = xa[m0 + 1], a2 = xa[m0 + 2], a3 = xa[m0 + 3];
        const size_t orow = P.fofs[r] + s;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            const double *w = sp.siw + ((size_t)d * P.iDim + r) * 4;
            double u = w[0] * a0 + w[1] * a1 + w[2] * a2 + w[3] * a3;
            ((T *)P.G)[((size_t)d * P.nitems + item) * P.frows + orow] = (T)u;
        }
    }
}

// ====================================================================
// cheb_forward: DCT-I of each kz-point column, scaled 1/(2(kz-1)), first bk modes
// (CBtransform!, src/Chebyshev.jl:417-426).  CTA = 64 consecutive columns.
// ====================================================================
template <typename T>
__global__ void __launch_bounds__(256) cheb_forward_kernel(ChebLaunch P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int v = blockIdx.y;
    const ChebDev &cb = P.cheb[v];
    const int N = cb.N, bk = cb.bk, half = cb.half;
    T *xs = reinterpret_cast<T *>(smem_raw);  // 64 × N
    T *fw = xs + 64 * N;                        // bk × half
    const int64_t c0 = (int64_t)blockIdx.x * 64;
    const int ncol = (int)((P.jDim - c0) < 64 ? (P.jDim - c0) : 64);
    const T *in = (const T *)P.in + (size_t)v * P.np + c0 * N;
    for (int e = threadIdx.x; e < ncol * N; e += blockDim.x) xs[e] = in[e];
    for (int e = threadIdx.x; e < bk * half; e += blockDim.x) fw[e] = (T)cb.fwd[e];
    __syncthreads();
    const int col = threadIdx.x & 63, kg = threadIdx.x >> 6;  // 4 groups of modes
    if (col < ncol) {
        const int64_t q = c0 + col;
        // ring of column q (binary search in ring start table)
        int lo = 0, hi = P.iDim - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (P.rings[mid].jofs <= q) lo = mid; else hi = mid - 1;
        }
        const RingDesc &rd = P.rings[lo];
        const int l = (int)(q - rd.jofs);
        T *out = (T *)P.out + (size_t)v * P.bk * P.jDim + (size_t)P.bk * rd.jofs + l;
        const T *x = xs + col * N;
        for (int k = kg; k < bk; k += 4) {
            const T *row = fw + k * half;
            T acc = T(0);
            const bool odd = k & 1;
            for (int j = 0; j < half; j++) {
                const int jj = N - 1 - j;
                T e = (jj == j) ? x[j] : (odd ? x[j] - x[jj] : x[j] + x[jj]);
                acc += row[j] * e;
            }
            out[(size_t)k * rd.L] = acc;
        }
    }
}

// ====================================================================
// cheb_inverse: CAtransform! (a = bfill + Γᵀ bfill, Γ = Σ u vᵀ) then
// CItransform! (DCT-I); variant 0 also CIx/CIxx (recurrence, src/Chebyshev.jl:636-646).
// CTA = 64 consecutive columns of one variable; grid.z = ring variant.
// ====================================================================
template <typename T>
__global__ void __launch_bounds__(256) cheb_inverse_kernel(ChebLaunch P) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int v = blockIdx.y, var = blockIdx.z;
    const ChebDev &cb = P.cheb[v];
    const int N = cb.N, bk = cb.bk, half = cb.half;
    const int ne = (N + 1) / 2, no = N / 2;
    T *as = reinterpret_cast<T *>(smem_raw);  // 64 × N coefficients
    T *us = as + 64 * N;                        // 64 × N outputs
    T *ie = us + 64 * N;                        // half × ne
    T *io = ie + half * ne;                     // half × no
    T *bs = io + half * (no > 0 ? no : 1);      // 64 × bk inputs
    const int64_t c0 = (int64_t)blockIdx.x * 64;
    const int ncol = (int)((P.jDim - c0) < 64 ? (P.jDim - c0) : 64);
    for (int e = threadIdx.x; e < half * ne; e += blockDim.x) ie[e] = (T)cb.inv_e[e];
    for (int e = threadIdx.x; e < half * no; e += blockDim.x) io[e] = (T)cb.inv_o[e];
    // gather the bk ring outputs of each column
    const T *H = (const T *)P.in + ((size_t)var * P.nvars + v) * P.bk * P.jDim;
    for (int e = threadIdx.x; e < ncol * bk; e += blockDim.x) {
        const int zb = e / ncol, col = e % ncol;
        const int64_t q = c0 + col;
        int lo = 0, hi = P.iDim - 1;
        while (lo < hi) {
            int mid = (lo + hi + 1) >> 1;
            if (P.rings[mid].jofs <= q) lo = mid; else hi = mid - 1;
        }
        const RingDesc &rd = P.rings[lo];
        bs[col * bk + zb] = H[(size_t)P.bk * rd.jofs + (size_t)zb * rd.L + (q - rd.jofs)];
    }
    __syncthreads();
    const int col = threadIdx.x & 63, jg = threadIdx.x >> 6;
    // CA: a_j = b_j (j < bk) + Σ_p (u_p·b) v_p[j]
    if (col < ncol) {
        const T *bb = bs + col * bk;
        T sp[2] = {T(0), T(0)};
        for (int p = 0; p < cb.nrank; p++) {
            T acc = T(0);
            for (int i = 0; i < bk; i++) acc += (T)cb.gu[p * bk + i] * bb[i];
            sp[p] = acc;
        }
        for (int j = jg; j < N; j += 4) {
            T aj = (j < bk) ? bb[j] : T(0);
            for (int p = 0; p < cb.nrank; p++) aj += (T)cb.gv[p * N + j] * sp[p];
            as[col * N + j] = aj;
        }
    }
    __syncthreads();
    const int nd = (var == 0) ? 3 : 1;
    for (int dd = 0; dd < nd; dd++) {
        if (dd > 0) {
            // CIxcoefficients in place (src/Chebyshev.jl:636-646):
            // ax[N-1] = 0, ax[i] = 2(i+1) a[i+1] + ax[i+2] for i = N-2..0, then ax /= dscale
            if (jg == 0 && col < ncol) {
                T *a = as + col * N;
                T a_next = a[N - 1];
                a[N - 1] = T(0);
                T ax1 = T(0), ax2 = T(0);  // ax[i+1], ax[i+2]
                for (int i = N - 2; i >= 0; i--) {
                    T axi = T(2.0 * (i + 1)) * a_next + ax2;
                    a_next = a[i];
                    a[i] = axi;
                    ax2 = ax1;
                    ax1 = axi;
                }
                const T sc = (T)cb.dscale;
                for (int j = 0; j < N; j++) a[j] = a[j] / sc;
            }
            __syncthreads();
        }
        if (col < ncol) {
            const T *a = as + col * N;
            T *u = us + col * N;
            for (int j = jg; j < half; j += 4) {
                T E = T(0), O = T(0);
                for (int k = 0; k < ne; k++) E += ie[j * ne + k] * a[2 * k];
                for (int k = 0; k < no; k++) O += io[j * no + k] * a[2 * k + 1];
                u[j] = E + O;
                if (N - 1 - j != j) u[N - 1 - j] = E - O;
            }
        }
        __syncthreads();
        // coalesced write of the tile: physical slot of (variant, derivative)
        int slot;
        if (var == 0) slot = (dd == 0) ? 1 : (dd == 1 ? 6 : 7);
        else slot = (var == 1) ? 4 : (var == 2 ? 5 : (var == 3 ? 2 : 3));
        T *dst = (T *)P.out + ((size_t)(slot - 1) * P.nvars + v) * P.np + c0 * N;
        for (int e = threadIdx.x; e < ncol * N; e += blockDim.x) dst[e] = us[e];
        __syncthreads();
    }
}

// ====================================================================
// launchers
// ====================================================================
template <typename T>
cudaError_t launch_ring_forward(const RingLaunch &L, int nrings, int nitems, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(ring_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    ring_forward_kernel<T><<<dim3(nrings, nitems), 256, smem, st>>>(L);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_ring_inverse(const RingLaunch &L, int nrings, int nitems, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(ring_inverse_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    ring_inverse_kernel<T><<<dim3(nrings, nitems), 256, smem, st>>>(L);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_sb_project(const SbLaunch &P, int nitems, cudaStream_t st) {
    dim3 grid((P.nslots_z + 31) / 32, (P.b + 63) / 64, nitems);
    sb_project_kernel<T><<<grid, dim3(32, 8), 0, st>>>(P);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_sa_si(const SaLaunch &P, int nitems, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(sa_si_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((P.nslots_z + 31) / 32, nitems);
    sa_si_kernel<T><<<grid, 128, smem, st>>>(P);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_cheb_forward(const ChebLaunch &P, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(cheb_forward_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((unsigned)((P.jDim + 63) / 64), P.nvars);
    cheb_forward_kernel<T><<<grid, 256, smem, st>>>(P);
    return cudaGetLastError();
}
template <typename T>
cudaError_t launch_cheb_inverse(const ChebLaunch &P, size_t smem, cudaStream_t st) {
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(cheb_inverse_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    dim3 grid((unsigned)((P.jDim + 63) / 64), P.nvars, 5);
    cheb_inverse_kernel<T><<<grid, 256, smem, st>>>(P);
    return cudaGetLastError();
}

#define SS_INSTANTIATE(T)                                                                                   \
    template cudaError_t launch_ring_forward<T>(const RingLaunch &, int, int, size_t, cudaStream_t);       \
    template cudaError_t launch_ring_inverse<T>(const RingLaunch &, int, int, size_t, cudaStream_t);       \
    template cudaError_t launch_sb_project<T>(const SbLaunch &, int, cudaStream_t);                        \
    template cudaError_t launch_sa_si<T>(const SaLaunch &, int, size_t, cudaStream_t);                     \
    template cudaError_t launch_cheb_forward<T>(const ChebLaunch &, size_t, cudaStream_t);                 \
    template cudaError_t launch_cheb_inverse<T>(const ChebLaunch &, size_t, cudaStream_t);
SS_INSTANTIATE(double)
SS_INSTANTIATE(float)

}  // namespace ss
