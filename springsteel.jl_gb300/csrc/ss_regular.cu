// ss_regular.cu — regularGridTransform on the device for RL and RLZ grids
// (src/transforms_cylindrical.jl:929-1020 RL, 1168-1287 RLZ): the spectral
// array evaluated on a tensor-product (r, λ[, z]) point set.
//
//   reg_sa        SAtransform! of every spectral slot (each Chebyshev mode, each
//                 wavenumber's cos / sin block), FP64, the grid's spline factor
//   reg_si        SI / SIx / SIxx of those coefficients at the r points
//   reg_fourier   the Fourier series at the λ points with the R2HC half-amplitude
//                 factor 2: f, ∂r f, ∂rr f (from SI, SIx, SIxx) and ∂λ f, ∂λλ f
//   reg_cheb      (RLZ) CAtransform! and the Chebyshev series at the z points, as
//                 per-variable matrices composed on the host: value for every
//                 variant, ∂z and ∂zz for the value variant
// Every stage computes in FP64 whatever the grid's precision; the result is a
// host array (n_r·n_λ[·n_z], nvars, 5|7), λ (then z) fastest, as the reference
// returns it.  The reference runs SAtransform! on the grid's spline objects,
// whose R3X background (ahat) is zero unless multipatch coupling set it; this
// path applies no ahat.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "ss_grid.h"
#include "ss_kernels.h"
#include "ss_spline_dev.cuh"
#include "ss_types.cuh"

using namespace ss;

#define CUDA_TRY(expr)                                                                      \
    do {                                                                                    \
        cudaError_t _e = (expr);                                                            \
        if (_e != cudaSuccess) {                                                            \
            set_error("%s failed: %s", #expr, cudaGetErrorString(_e));                      \
            return (_e == cudaErrorMemoryAllocation) ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;   \
        }                                                                                   \
    } while (0)

namespace {

// SAtransform! of `per` consecutive slots of one item per CTA (one thread each):
// Γ fold, banded LLᵀ solve with the FP64 factor, Γᵀ unfold → coef[item][slot][b]
template <typename P>
__global__ void reg_sa_kernel(const P *spec, const SplineDev *spl, double *coef, int64_t nspec, int b, int ld,
                              int nslots_z, int bk) {
    extern __shared__ __align__(16) double sm[];
    const int item = blockIdx.y, v = item / bk, zb = item % bk;
    const SplineDev &sp = spl[v];
    const int n = sp.Min, per = blockDim.x;
    double *X = sm;              // per × ld
    double *Ls = X + per * ld;   // 4n
    double *Di = Ls + 4 * n;     // n
    const int s0 = blockIdx.x * per, nsl = min(per, nslots_z - s0);
    const P *src = spec + (size_t)v * nspec + ((size_t)zb * nslots_z + s0) * b;
    for (int e = threadIdx.x; e < nsl * b; e += per) X[(e / b) * ld + e % b] = (double)src[e];
    for (int e = threadIdx.x; e < 4 * n; e += per) Ls[e] = sp.L4[e];
    for (int e = threadIdx.x; e < n; e += per) Di[e] = sp.dinv[e];
    __syncthreads();
    if (threadIdx.x < nsl) {
        double *x = X + threadIdx.x * ld;
        gamma_fold(sp, x, b, n);
        band_solve(Ls, Di, x, n, sp.periodic ? sp.tail : nullptr);
        gamma_unfold(sp, x, b, n);
    }
    __syncthreads();
    double *dst = coef + ((size_t)item * nslots_z + s0) * b;
    for (int e = threadIdx.x; e < nsl * b; e += per) dst[e] = X[(e / b) * ld + e % b];
}

// sr[d][item][r][slot] = Σ_tap w[d][r][tap] · coef[item][slot][m0[r] + tap]
__global__ void reg_si_kernel(const double *coef, const int *m0, const double *w, double *sr, int b,
                              int nslots_z, int n_r, int nitems) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y, item = blockIdx.z;
    if (s >= nslots_z) return;
    const double *a = coef + ((size_t)item * nslots_z + s) * b + m0[r];
    const double a0 = a[0], a1 = a[1], a2 = a[2], a3 = a[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const double *wd = w + ((size_t)d * n_r + r) * 4;
        sr[(((size_t)d * nitems + item) * n_r + r) * nslots_z + s] = wd[0] * a0 + wd[1] * a1 + wd[2] * a2 + wd[3] * a3;
    }
}

// The Fourier series at λ_j for one (item, r) per CTA row, j over threads:
//   f = a0 + Σ_k 2 (rc cos kλ + rs sin kλ), the same with the SIx / SIxx
//   coefficients for ∂r f / ∂rr f, ∂λ f = Σ_k 2k (−rc sin + rs cos),
//   ∂λλ f = −Σ_k 2k² (rc cos + rs sin)   (src/transforms_cylindrical.jl:985-1005)
// cos/sin(kλ_j) come from host tables tc/ts[(k−1)·n_λ + j].  RL writes the result
// slots straight into out (rows r·n_λ + j); RLZ writes fb[variant][v][r][j][zb].
__global__ void __launch_bounds__(128) reg_fourier_kernel(const double *sr, const double *tc, const double *ts,
                                                          double *dst, int nslots_z, int K, int n_r, int n_lam,
                                                          int nitems, int rlz, int bk, int nvars) {
    extern __shared__ __align__(16) double c[];  // [d][slot]
    const int r = blockIdx.y, item = blockIdx.z;
    for (int e = threadIdx.x; e < 3 * nslots_z; e += blockDim.x) {
        const int d = e / nslots_z, s = e - d * nslots_z;
        c[e] = sr[(((size_t)d * nitems + item) * n_r + r) * nslots_z + s];
    }
    __syncthreads();
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n_lam) return;
    const double *c1 = c + nslots_z, *c2 = c + 2 * nslots_z;
    double f = c[0], fr = c1[0], frr = c2[0], fl = 0.0, fll = 0.0;
    for (int k = 1; k <= K; k++) {
        const double ck = tc[(size_t)(k - 1) * n_lam + j], sk = ts[(size_t)(k - 1) * n_lam + j];
        const double rc = c[2 * k - 1], rs = c[2 * k];
        const double kk = (double)k;
        f += 2.0 * (rc * ck + rs * sk);
        fr += 2.0 * (c1[2 * k - 1] * ck + c1[2 * k] * sk);
        frr += 2.0 * (c2[2 * k - 1] * ck + c2[2 * k] * sk);
        fl += 2.0 * kk * (-rc * sk + rs * ck);
        fll -= 2.0 * (kk * kk) * (rc * ck + rs * sk);
    }
    const double vals[5] = {f, fr, frr, fl, fll};  // variants: f, ∂r, ∂rr, ∂λ, ∂λλ
    if (!rlz) {
        const size_t nrows = (size_t)n_r * n_lam, row = (size_t)r * n_lam + j;
#pragma unroll
        for (int q = 0; q < 5; q++) dst[((size_t)q * nvars + item) * nrows + row] = vals[q];
    } else {
        const int v = item / bk, zb = item - v * bk;
#pragma unroll
        for (int q = 0; q < 5; q++)
            dst[((((size_t)q * nvars + v) * n_r + r) * n_lam + j) * bk + zb] = vals[q];
    }
}

// Chebyshev series at z for every (r, λ) column of one variable and variant:
// out[row = col·n_z + z][v][slot] = Σ_zb M[z][zb] fb[col][zb], M = E·CA (value),
// and for the value variant also Dz·CA (∂z) and Dzz·CA (∂zz)
__global__ void reg_cheb_kernel(const double *fb, const double *mats, double *out, int64_t ncol, int n_z, int bk,
                                int nvars, int n_r) {
    extern __shared__ __align__(16) double M[];  // 3 × n_z × bk
    const int v = blockIdx.y, q = blockIdx.z;
    const int nm = (q == 0) ? 3 : 1;
    const double *mv = mats + (size_t)v * 3 * n_z * bk;
    for (int e = threadIdx.x; e < nm * n_z * bk; e += blockDim.x) M[e] = mv[e];
    __syncthreads();
    const int64_t nrows = ncol * n_z;
    const double *src = fb + ((size_t)q * nvars + v) * ncol * bk;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nrows; t += (int64_t)gridDim.x * blockDim.x) {
        const int64_t col = t / n_z;
        const int z = (int)(t - col * n_z);
        const double *bcol = src + col * bk;
        for (int m = 0; m < nm; m++) {
            const double *row = M + ((size_t)m * n_z + z) * bk;
            double acc = 0.0;
            for (int i = 0; i < bk; i++) acc += row[i] * bcol[i];
            const int slot = m == 0 ? q : 4 + m;  // variant q's slot; ∂z, ∂zz → slots 6, 7 (0-based 5, 6)
            out[((size_t)slot * nvars + v) * nrows + t] = acc;
        }
    }
    (void)n_r;
}

// Value of the spectral fields at arbitrary points: one warp per (point, variable).
// Per Chebyshev mode z_b the warp sums the Fourier series of the SI values at the
// point's radius (4-tap window m0, weights w):
//   f_zb = S_0 + 2 Σ_k (S_{2k−1} cos kλ + S_{2k} sin kλ),  S_q = Σ_tap w_tap a_q[m0 + tap]
// (src/interpolation.jl:1628-1656 RL, 1670-1718 RLZ).  mode 1 keeps the k = 0
// term only (the azimuthal mean), mode 2 writes NaN; taper t blends
// t·full + (1 − t)·mean (src/relocation.jl:252-258).  RL: one value per point.
// RLZ: CAtransform! of f_zb (the composed matrix CA, N × bk) and the Chebyshev
// series at z (_cheb_eval_single, src/interpolation.jl:1271-1285) — at the
// point's own z (zcol = nullptr) or at the n_z column levels zcol (relocation).
struct PointArgs {
    const double *coef;   // [item][slot][b] spline coefficients (FP64)
    const double *lam, *z, *w, *taper;  // per point; z RLZ only; w[p][4]
    const int *m0, *mode;
    const double *ca;     // RLZ: per variable N × bk
    const double *zcol;   // RLZ relocation: n_z column levels, else null
    void *out;            // P storage
    int64_t npts, ostride_v;  // rows between variables of out
    int b, nslots, K, bk, nvars, N, n_z, rlz, out_f32;
    double zmin, zmax;
    int first_var, nvar_eval;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(128) point_eval_kernel(PointArgs A) {
    extern __shared__ __align__(16) double fz[];  // per warp: bk values
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int64_t gw = (int64_t)blockIdx.x * (blockDim.x >> 5) + wib;
    const int64_t p = gw / A.nvar_eval;
    if (p >= A.npts) return;  // whole warps leave together (no block barrier below)
    const int v = A.first_var + (int)(gw - p * A.nvar_eval);
    double *f = fz + (size_t)wib * A.bk;
    const int mode = A.mode ? A.mode[p] : 0;
    auto store = [&](int64_t row, double val) {
        if (A.out_f32) ((float *)A.out)[(size_t)v * A.ostride_v + row] = (float)val;
        else ((double *)A.out)[(size_t)v * A.ostride_v + row] = val;
    };
    const int nout = A.rlz && A.zcol ? A.n_z : 1;
    const int64_t row0 = A.rlz && A.zcol ? p * A.n_z : p;
    if (mode == 2) {
        if (lane < nout) store(row0 + lane, __longlong_as_double(0x7ff8000000000000LL));
        for (int q = lane + 32; q < nout; q += 32) store(row0 + q, __longlong_as_double(0x7ff8000000000000LL));
        return;
    }
    const double lam = A.lam[p], t = A.taper ? A.taper[p] : 1.0;
    const double w0 = A.w[p * 4], w1 = A.w[p * 4 + 1], w2 = A.w[p * 4 + 2], w3 = A.w[p * 4 + 3];
    const int m0 = A.m0[p];
    for (int zb = 0; zb < A.bk; zb++) {
        const double *a = A.coef + ((size_t)(v * A.bk + zb) * A.nslots) * A.b + m0;
        auto si = [&](int q) {
            const double *c = a + (size_t)q * A.b;
            return w0 * c[0] + w1 * c[1] + w2 * c[2] + w3 * c[3];
        };
        double full = 0.0;
        if (mode == 0)
            for (int k = 1 + lane; k <= A.K; k += 32) {
                double sk, ck;
                sincos((double)k * lam, &sk, &ck);
                full += 2.0 * (si(2 * k - 1) * ck + si(2 * k) * sk);
            }
        full = warp_sum(full);
        const double mean = si(0);
        const double val = (mode == 1) ? mean : (t * (mean + full) + (1.0 - t) * mean);
        if (lane == 0) f[zb] = val;
    }
    __syncwarp();
    if (!A.rlz) {
        if (lane == 0) store(p, f[0]);
        return;
    }
    // CAtransform! then the Chebyshev series (clamped to [−1, 1]) at each level
    const double scale = -0.5 * (A.zmax - A.zmin), offset = 0.5 * (A.zmin + A.zmax);
    const double *ca = A.ca + (size_t)v * A.N * A.bk;
    for (int zi = 0; zi < nout; zi++) {
        const double z = A.zcol ? A.zcol[zi] : A.z[p];
        const double xi = fmin(fmax((z - offset) / scale, -1.0), 1.0);
        const double th = acos(xi);
        double acc = 0.0;
        for (int n = lane; n < A.N; n += 32) {
            double an = 0.0;
            for (int i = 0; i < A.bk; i++) an += ca[(size_t)n * A.bk + i] * f[i];
            const double e = (n == 0) ? 1.0 : (n == A.N - 1 ? cos((double)n * th) : 2.0 * cos((double)n * th));
            acc += e * an;
        }
        acc = warp_sum(acc);
        if (lane == 0) store(row0 + zi, acc);
    }
}

// E (value), Dz, Dzz of the DCT-I series at z (n_z × N, row-major) with the
// reference's clamps (_cheb_eval_pts!, _cheb_dz_pts!, _cheb_dzz_pts!,
// src/transforms_cylindrical.jl:1030-1094)
void cheb_point_matrices(int N, double zmin, double zmax, const double *z, int n_z, std::vector<double> &E,
                         std::vector<double> &Dz, std::vector<double> &Dzz) {
    const double scale = -0.5 * (zmax - zmin), offset = 0.5 * (zmin + zmax);
    E.assign(size_t(n_z) * N, 0.0);
    Dz.assign(size_t(n_z) * N, 0.0);
    Dzz.assign(size_t(n_z) * N, 0.0);
    for (int i = 0; i < n_z; i++) {
        const double xi0 = std::min(std::max((z[i] - offset) / scale, -1.0 + 1e-14), 1.0 - 1e-14);
        const double t0 = std::acos(xi0);
        const double xi = std::min(std::max((z[i] - offset) / scale, -1.0 + 1e-10), 1.0 - 1e-10);
        const double t = std::acos(xi), st = std::sin(t), ct = std::cos(t);
        for (int k = 0; k < N; k++) {
            const double m = (double)k;
            const double wgt = (k == 0) ? 0.0 : (k == N - 1 ? 1.0 : 2.0);
            E[size_t(i) * N + k] = (k == 0) ? 1.0 : (k == N - 1 ? std::cos(m * t0) : 2.0 * std::cos(m * t0));
            const double d1 = -wgt * m * std::sin(m * t);       // df/dt coefficient
            const double d2 = -wgt * m * m * std::cos(m * t);   // d²f/dt² coefficient
            Dz[size_t(i) * N + k] = d1 / (-scale * st);
            Dzz[size_t(i) * N + k] = (d2 * st - d1 * ct) / (scale * scale * st * st * st);
        }
    }
}

template <typename P>
int32_t regular(ss_grid *g, const double *r_pts, int n_r, const double *lam_pts, int n_lam, const double *z_pts,
                int n_z, double *out_host, cudaStream_t st) {
    const ss_dims &d = g->d;
    const int b = (int)d.b_iDim, K = (int)d.kDim_wn, ns = g->nslots_z, bk = (int)d.b_kDim;
    const int nv = (int)d.nvars, nitems = g->nitems;
    const int nz = g->rlz ? n_z : 1;
    const size_t nrows = size_t(n_r) * n_lam * nz;
    // host tables: SI weights at r, cos/sin(kλ), Chebyshev point matrices composed with CA
    std::vector<int> m0;
    std::vector<double> w;
    spline_point_weights(g->spl_host[0], r_pts, n_r, m0, w);  // every variable shares the radial knots
    std::vector<double> tc(size_t(K) * n_lam), ts(size_t(K) * n_lam);
    for (int k = 1; k <= K; k++)
        for (int j = 0; j < n_lam; j++) {
            const double a = (double)k * lam_pts[j];
            tc[size_t(k - 1) * n_lam + j] = std::cos(a);
            ts[size_t(k - 1) * n_lam + j] = std::sin(a);
        }
    std::vector<double> mats;
    if (g->rlz) {
        const int N = (int)d.kDim;
        std::vector<double> E, Dz, Dzz;
        cheb_point_matrices(N, g->p.kMin, g->p.kMax, z_pts, n_z, E, Dz, Dzz);
        mats.assign(size_t(nv) * 3 * n_z * bk, 0.0);
        for (int v = 0; v < nv; v++) {
            ChebHost ch;
            int32_t rc = build_cheb(N, bk, g->bcb[v], g->bct[v], g->p.kMin, g->p.kMax, ch);
            if (rc) return rc;
            // CA[n][i] = δ_ni + Σ_p v_p[n] u_p[i]  (a = bfill + Γᵀ bfill)
            std::vector<double> CA(size_t(N) * bk, 0.0);
            for (int n = 0; n < N; n++)
                for (int i = 0; i < bk; i++) {
                    double a = (n == i) ? 1.0 : 0.0;
                    for (int p = 0; p < ch.nrank; p++) a += ch.gv[size_t(p) * N + n] * ch.gu[size_t(p) * bk + i];
                    CA[size_t(n) * bk + i] = a;
                }
            const std::vector<double> *src[3] = {&E, &Dz, &Dzz};
            for (int m = 0; m < 3; m++)
                for (int z = 0; z < n_z; z++)
                    for (int i = 0; i < bk; i++) {
                        double acc = 0.0;
                        for (int n = 0; n < N; n++) acc += (*src[m])[size_t(z) * N + n] * CA[size_t(n) * bk + i];
                        mats[((size_t(v) * 3 + m) * n_z + z) * bk + i] = acc;
                    }
        }
    }
    // device buffers (freed before returning)
    std::vector<void *> bufs;
    auto dmalloc = [&](void **p, size_t bytes) -> cudaError_t {
        cudaError_t e = cudaMalloc(p, std::max<size_t>(bytes, 16));
        if (e == cudaSuccess) bufs.push_back(*p);
        return e;
    };
    auto release = [&]() {
        for (void *p : bufs) cudaFree(p);
        bufs.clear();
    };
    double *d_coef = nullptr, *d_w = nullptr, *d_tc = nullptr, *d_ts = nullptr, *d_sr = nullptr, *d_out = nullptr;
    double *d_fb = nullptr, *d_mats = nullptr;
    int *d_m0 = nullptr;
    cudaError_t e = cudaSuccess;
    const size_t out_elems = nrows * nv * d.nslots;
    if ((e = dmalloc((void **)&d_coef, size_t(nitems) * ns * b * 8)) != cudaSuccess ||
        (e = dmalloc((void **)&d_w, w.size() * 8)) != cudaSuccess ||
        (e = dmalloc((void **)&d_m0, m0.size() * 4)) != cudaSuccess ||
        (e = dmalloc((void **)&d_tc, tc.size() * 8)) != cudaSuccess ||
        (e = dmalloc((void **)&d_ts, ts.size() * 8)) != cudaSuccess ||
        (e = dmalloc((void **)&d_sr, size_t(3) * nitems * n_r * ns * 8)) != cudaSuccess ||
        (e = dmalloc((void **)&d_out, out_elems * 8)) != cudaSuccess ||
        (g->rlz && (e = dmalloc((void **)&d_fb, size_t(5) * nv * n_r * n_lam * bk * 8)) != cudaSuccess) ||
        (g->rlz && (e = dmalloc((void **)&d_mats, mats.size() * 8)) != cudaSuccess)) {
        release();
        set_error("regular grid buffers: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;
    }
    auto run = [&]() -> int32_t {
        CUDA_TRY(cudaMemcpyAsync(d_w, w.data(), w.size() * 8, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_m0, m0.data(), m0.size() * 4, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_tc, tc.data(), tc.size() * 8, cudaMemcpyHostToDevice, st));
        CUDA_TRY(cudaMemcpyAsync(d_ts, ts.data(), ts.size() * 8, cudaMemcpyHostToDevice, st));
        if (g->rlz) CUDA_TRY(cudaMemcpyAsync(d_mats, mats.data(), mats.size() * 8, cudaMemcpyHostToDevice, st));
        // SAtransform! of every slot
        int nmax = 0;
        for (auto &sh : g->spl_host) nmax = std::max(nmax, sh.Min);
        const int ld = (b % 2) ? b : b + 1;
        int optin = 0;
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, g->device);
        int per = 32;
        auto sa_smem = [&](int p) { return (size_t(p) * ld + size_t(5) * nmax) * 8; };
        while (per > 1 && sa_smem(per) > (size_t)optin) per /= 2;
        if (sa_smem(per) > (size_t)optin) {
            set_error("regularGridTransform: %d radial coefficients exceed shared memory", b);
            return SS_BAD_SHAPE;
        }
        CUDA_TRY(cudaFuncSetAttribute(reg_sa_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sa_smem(per)));
        reg_sa_kernel<P><<<dim3((ns + per - 1) / per, nitems), per, sa_smem(per), st>>>(
            (const P *)g->spec, g->d_spl, d_coef, d.n_spectral, b, ld, ns, bk);
        CUDA_TRY(cudaGetLastError());
        reg_si_kernel<<<dim3((ns + 127) / 128, n_r, nitems), 128, 0, st>>>(d_coef, d_m0, d_w, d_sr, b, ns, n_r,
                                                                            nitems);
        CUDA_TRY(cudaGetLastError());
        const size_t fsm = size_t(3) * ns * 8;
        if (fsm > (size_t)optin) {
            set_error("regularGridTransform: %d wavenumber slots exceed shared memory", ns);
            return SS_BAD_SHAPE;
        }
        CUDA_TRY(cudaFuncSetAttribute(reg_fourier_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)fsm));
        reg_fourier_kernel<<<dim3((n_lam + 127) / 128, n_r, nitems), 128, fsm, st>>>(
            d_sr, d_tc, d_ts, g->rlz ? d_fb : d_out, ns, K, n_r, n_lam, nitems, g->rlz, bk, nv);
        CUDA_TRY(cudaGetLastError());
        if (g->rlz) {
            const size_t msm = size_t(3) * n_z * bk * 8;
            if (msm > (size_t)optin) {
                set_error("regularGridTransform: %d z points exceed shared memory", n_z);
                return SS_BAD_SHAPE;
            }
            CUDA_TRY(cudaFuncSetAttribute(reg_cheb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)msm));
            const int64_t ncol = int64_t(n_r) * n_lam;
            const int64_t blocks = std::min<int64_t>((ncol * n_z + 255) / 256, 4096);
            reg_cheb_kernel<<<dim3((unsigned)blocks, nv, 5), 256, msm, st>>>(d_fb, d_mats, d_out, ncol, n_z, bk,
                                                                             nv, n_r);
            CUDA_TRY(cudaGetLastError());
        }
        CUDA_TRY(cudaMemcpyAsync(out_host, d_out, out_elems * 8, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        return SS_OK;
    };
    const int32_t rc = run();
    if (rc) cudaStreamSynchronize(st);
    release();
    return rc;
}

// Spline coefficients of every spectral block of `src` (FP64, [item][slot][b]) into a
// fresh device buffer (the caller frees it)
template <typename P>
int32_t block_coefficients(ss_grid *src, double **d_coef, cudaStream_t st) {
    const ss_dims &d = src->d;
    const int b = (int)d.b_iDim, ns = src->nslots_z, bk = (int)d.b_kDim;
    int nmax = 0;
    for (auto &sh : src->spl_host) nmax = std::max(nmax, sh.Min);
    const int ld = (b % 2) ? b : b + 1;
    int optin = 0;
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, src->device);
    int per = 32;
    auto sa_smem = [&](int q) { return (size_t(q) * ld + size_t(5) * nmax) * 8; };
    while (per > 1 && sa_smem(per) > (size_t)optin) per /= 2;
    if (sa_smem(per) > (size_t)optin) {
        set_error("%d radial coefficients exceed shared memory", b);
        return SS_BAD_SHAPE;
    }
    CUDA_TRY(cudaMalloc(d_coef, size_t(src->nitems) * ns * b * 8));
    CUDA_TRY(cudaFuncSetAttribute(reg_sa_kernel<P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sa_smem(per)));
    reg_sa_kernel<P><<<dim3((ns + per - 1) / per, src->nitems), per, sa_smem(per), st>>>(
        (const P *)src->spec, src->d_spl, *d_coef, d.n_spectral, b, ld, ns, bk);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

// The point kernel over host-described points: radii r (SI windows built here),
// angles, optional z, modes and taper weights; `out` is device memory
int32_t eval_points(ss_grid *g, const double *coef, const std::vector<double> &r, const std::vector<double> &lam,
                    const std::vector<double> &z, const std::vector<int> &mode, const std::vector<double> &taper,
                    const std::vector<double> &zcol, void *out, int64_t ostride_v, int out_f32, cudaStream_t st) {
    const ss_dims &d = g->d;
    const int64_t npts = (int64_t)r.size();
    if (npts == 0) return SS_OK;
    std::vector<int> m0;
    std::vector<double> w3;
    spline_point_weights(g->spl_host[0], r.data(), (int)npts, m0, w3);  // every variable shares the knots
    std::vector<double> w(size_t(npts) * 4);
    std::copy(w3.begin(), w3.begin() + w.size(), w.begin());  // d = 0: the value weights
    std::vector<double> ca;
    const int N = (int)d.kDim, bk = (int)d.b_kDim, nv = (int)d.nvars;
    if (g->rlz) {
        ca.assign(size_t(nv) * N * bk, 0.0);
        for (int v = 0; v < nv; v++) {
            ChebHost ch;
            int32_t rc = build_cheb(N, bk, g->bcb[v], g->bct[v], g->p.kMin, g->p.kMax, ch);
            if (rc) return rc;
            for (int n = 0; n < N; n++)  // CA[n][i] = δ_ni + Σ_p v_p[n] u_p[i]
                for (int i = 0; i < bk; i++) {
                    double a = (n == i) ? 1.0 : 0.0;
                    for (int q = 0; q < ch.nrank; q++) a += ch.gv[size_t(q) * N + n] * ch.gu[size_t(q) * bk + i];
                    ca[(size_t(v) * N + n) * bk + i] = a;
                }
        }
    }
    std::vector<void *> bufs;
    auto up = [&](const void *h, size_t bytes, void **dptr) -> cudaError_t {
        if (!bytes) { *dptr = nullptr; return cudaSuccess; }
        cudaError_t e = cudaMalloc(dptr, bytes);
        if (e != cudaSuccess) return e;
        bufs.push_back(*dptr);
        return cudaMemcpyAsync(*dptr, h, bytes, cudaMemcpyHostToDevice, st);
    };
    PointArgs A{};
    cudaError_t e = cudaSuccess;
    void *p_lam, *p_z, *p_w, *p_t, *p_m0, *p_mode, *p_ca, *p_zc;
    if ((e = up(lam.data(), lam.size() * 8, &p_lam)) || (e = up(z.data(), z.size() * 8, &p_z)) ||
        (e = up(w.data(), w.size() * 8, &p_w)) || (e = up(taper.data(), taper.size() * 8, &p_t)) ||
        (e = up(m0.data(), m0.size() * 4, &p_m0)) || (e = up(mode.data(), mode.size() * 4, &p_mode)) ||
        (e = up(ca.data(), ca.size() * 8, &p_ca)) || (e = up(zcol.data(), zcol.size() * 8, &p_zc))) {
        cudaStreamSynchronize(st);
        for (void *q : bufs) cudaFree(q);
        set_error("point evaluation buffers: %s", cudaGetErrorString(e));
        return e == cudaErrorMemoryAllocation ? SS_OUT_OF_MEMORY : SS_CUDA_ERROR;
    }
    A.coef = coef; A.lam = (const double *)p_lam; A.z = (const double *)p_z; A.w = (const double *)p_w;
    A.taper = (const double *)p_t; A.m0 = (const int *)p_m0; A.mode = (const int *)p_mode;
    A.ca = (const double *)p_ca; A.zcol = (const double *)p_zc; A.out = out;
    A.npts = npts; A.ostride_v = ostride_v; A.b = (int)d.b_iDim; A.nslots = g->nslots_z; A.K = (int)d.kDim_wn;
    A.bk = bk; A.nvars = nv; A.N = N; A.n_z = (int)zcol.size(); A.rlz = g->rlz; A.out_f32 = out_f32;
    A.zmin = g->p.kMin; A.zmax = g->p.kMax; A.first_var = 0; A.nvar_eval = nv;
    const int64_t warps = npts * nv;
    point_eval_kernel<<<(unsigned)((warps + 3) / 4), 128, size_t(4) * bk * 8, st>>>(A);
    e = cudaGetLastError();
    cudaError_t e2 = cudaStreamSynchronize(st);
    for (void *q : bufs) cudaFree(q);
    if (e != cudaSuccess || e2 != cudaSuccess) {
        set_error("point evaluation: %s", cudaGetErrorString(e != cudaSuccess ? e : e2));
        return SS_CUDA_ERROR;
    }
    return SS_OK;
}

template <typename P>
int32_t unstructured(ss_grid *g, const double *pts, int64_t npts, double *out, int oob, double fill,
                     cudaStream_t st) {
    const double rmin = g->p.iMin, rmax = g->p.iMax, zmin = g->p.kMin, zmax = g->p.kMax;
    std::vector<double> r(npts), lam(npts), z(g->rlz ? npts : 0), taper;
    std::vector<int> mode(npts, 0);
    int64_t n_oob = 0;
    for (int64_t i = 0; i < npts; i++) {
        r[i] = pts[i];
        lam[i] = pts[npts + i];
        bool in = r[i] >= rmin && r[i] <= rmax;  // _check_bounds_nd: Fourier λ is always in bounds
        if (g->rlz) {
            z[i] = pts[2 * npts + i];
            in = in && z[i] >= zmin && z[i] <= zmax;
        }
        if (!in) {
            mode[i] = 2;
            r[i] = std::min(std::max(r[i], rmin), rmax);
            n_oob++;
        }
    }
    if (oob == 1 && n_oob) {
        set_error("%lld points are outside the source domain", (long long)n_oob);
        return SS_BAD_ARG;
    }
    const int nv = (int)g->d.nvars;
    double *d_coef = nullptr, *d_out = nullptr;
    int32_t rc = block_coefficients<P>(g, &d_coef, st);
    if (rc) return rc;
    if (cudaMalloc((void **)&d_out, size_t(npts) * nv * 8) != cudaSuccess) {
        cudaGetLastError();
        cudaStreamSynchronize(st);
        cudaFree(d_coef);
        set_error("out of device memory");
        return SS_OUT_OF_MEMORY;
    }
    rc = eval_points(g, d_coef, r, lam, z, mode, taper, {}, d_out, npts, 0, st);
    if (!rc && cudaMemcpy(out, d_out, size_t(npts) * nv * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        set_error("point evaluation download: %s", cudaGetErrorString(cudaGetLastError()));
        rc = SS_CUDA_ERROR;
    }
    cudaFree(d_coef);
    cudaFree(d_out);
    if (!rc && oob == 2)
        for (int64_t i = 0; i < npts; i++)
            if (mode[i] == 2)
                for (int v = 0; v < nv; v++) out[size_t(v) * npts + i] = fill;
    return rc;
}

// relocate_grid / relocate_grid! fast path (src/relocation.jl:144-439): every
// gridpoint of the target evaluates the source at its shifted position
template <typename P>
int32_t relocate(ss_grid *t, ss_grid *s, double dx, double dy, int boundary, int taper_width, cudaStream_t st) {
    const ss_dims &d = s->d;
    const double rmin = s->p.iMin, rmax = s->p.iMax;
    const double DX = (rmax - rmin) / s->p.num_cells;
    const double r_start = taper_width > 0 ? rmax - taper_width * DX : rmax;
    const int64_t nring_pts = d.jDim;
    std::vector<double> r(nring_pts), lam(nring_pts), taper(nring_pts, 1.0), zcol;
    std::vector<int> mode(nring_pts, 0);
    const double twopi = 2 * 3.14159265358979323846;
    int64_t q = 0;
    for (int ri0 = 0; ri0 < (int)d.iDim; ri0++) {
        const int ri = ri0 + 1 + s->pOL, L = 4 + 4 * ri;
        const double ymin = 0.5 * (twopi / L) * (ri - 1), rm = s->spl_host[0].mish[ri0];
        for (int l = 0; l < L; l++, q++) {
            const double ln = ymin + twopi * l / L;
            const double xo = rm * std::cos(ln) + dx, yo = rm * std::sin(ln) + dy;
            const double ro = std::sqrt(xo * xo + yo * yo);
            lam[q] = std::atan2(yo, xo);
            const bool oob = ro > rmax || ro < rmin;
            r[q] = oob ? std::min(std::max(ro, rmin + 1e-10), rmax - 1e-10) : ro;
            if (oob) mode[q] = boundary == 0 ? 2 : (boundary == 2 ? 1 : 0);  // nan / nearest / azimuthal mean
            else if (taper_width > 0 && r[q] > r_start)
                taper[q] = 0.5 * (1.0 + std::cos(3.14159265358979323846 * (r[q] - r_start) / (rmax - r_start)));
        }
    }
    if (s->rlz) {
        ChebHost ch;
        int32_t rc = build_cheb((int)d.kDim, (int)d.b_kDim, s->bcb[0], s->bct[0], s->p.kMin, s->p.kMax, ch);
        if (rc) return rc;
        zcol = ch.mish;  // the column's Chebyshev points, zmin → zmax
    }
    double *d_coef = nullptr;
    int32_t rc = block_coefficients<P>(s, &d_coef, st);
    if (rc) return rc;
    rc = eval_points(s, d_coef, r, lam, {}, mode, taper, zcol, t->phys, d.n_physical, t->esz == 4, st);
    cudaFree(d_coef);
    if (rc) return rc;
    if ((rc = grid_forward(t, st))) return rc;  // spectralTransform!(target); gridTransform!(target)
    return grid_inverse(t, st);
}

}  // namespace

extern "C" int32_t ss_regular_grid_transform(ss_grid *g, const double *r_pts, int32_t n_r, const double *lam_pts,
                                             int32_t n_lam, const double *z_pts, int32_t n_z, double *out,
                                             void *stream) {
    if (!g || !r_pts || !lam_pts || !out || n_r < 1 || n_lam < 1) {
        set_error("regularGridTransform: null pointer or empty point set");
        return SS_BAD_ARG;
    }
    if (g->rlz && (!z_pts || n_z < 1)) {
        set_error("regularGridTransform: RLZ grids need z points");
        return SS_BAD_ARG;
    }
    CUDA_TRY(cudaSetDevice(g->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    if (g->esz == 4) return regular<float>(g, r_pts, n_r, lam_pts, n_lam, z_pts, n_z, out, st);
    return regular<double>(g, r_pts, n_r, lam_pts, n_lam, z_pts, n_z, out, st);
}

extern "C" int32_t ss_evaluate_unstructured(ss_grid *g, const double *pts, int64_t npts, double *out,
                                            int32_t out_of_bounds, double fill, void *stream) {
    if (!g || !pts || !out || npts < 0 || out_of_bounds < 0 || out_of_bounds > 2) {
        set_error("evaluate_unstructured: bad arguments");
        return SS_BAD_ARG;
    }
    if (npts == 0) return SS_OK;
    CUDA_TRY(cudaSetDevice(g->device));
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    if (g->esz == 4) return unstructured<float>(g, pts, npts, out, out_of_bounds, fill, st);
    return unstructured<double>(g, pts, npts, out, out_of_bounds, fill, st);
}

extern "C" int32_t ss_relocate_grid(ss_grid *target, ss_grid *source, double dx, double dy, int32_t boundary,
                                    int32_t taper_width, void *stream) {
    if (!target || !source || boundary < 0 || boundary > 2 || taper_width < 0) {
        set_error("relocate_grid: bad arguments");
        return SS_BAD_ARG;
    }
    if (target->rlz != source->rlz || target->d.n_physical != source->d.n_physical ||
        target->d.nvars != source->d.nvars || target->esz != source->esz || target->device != source->device ||
        target->d.n_spectral != source->d.n_spectral) {
        set_error("relocate_grid: target must be a grid with the source's parameters");
        return SS_BAD_SHAPE;
    }
    CUDA_TRY(cudaSetDevice(source->device));
    // queued on the target's stream (where the caller's later work on the target
    // goes), after the source's queued work has finished
    cudaStream_t st = stream ? (cudaStream_t)stream : target->stream;
    CUDA_TRY(cudaStreamSynchronize(source->stream));
    if (source->esz == 4) return relocate<float>(target, source, dx, dy, boundary, taper_width, st);
    return relocate<double>(target, source, dx, dy, boundary, taper_width, st);
}
