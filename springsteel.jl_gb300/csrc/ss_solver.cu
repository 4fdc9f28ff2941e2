// ss_solver.cu — elliptic solve on RL grids, one Fourier wavenumber at a time:
//   (∂rr + (1/r)∂r + (1/r²)∂λλ − k²(r)) u = f.
//
// The reference's solver assembles Kron products of 1-D basis matrices with the
// ring-1 Fourier basis only (src/solver.jl:339-363), which RL's variable rings
// violate, so it has no RL solve.  Here each wavenumber m gets the radial
// Galerkin operator built from the reference's own pieces — B-spline values
// and derivatives at the mish points (spline_*_matrix, src/CubicBSpline.jl:
// 1729-1816), tested with the SB weights (_build_sb_matrix, :1000-1030), Γ
// folded (src/solver.jl:721-756) with axis regularity (u'(0) = 0 for m = 0,
// u(0) = 0 for m ≥ 1) and u(R) = 0:
//     G_m = Γ_m [Σ_i w_{·,i} (Lφ_j)(r_i)] Γ_mᵀ,  G_m x = Γ_m b_m,  a = Γ_mᵀ x.
// b_m is the spectral B-vector of f (spectralTransform!); a feeds the SI and
// ring stages of gridTransform!.  Backends (src/solver_problem.jl:99-222):
// direct banded LU (FP64), restarted GMRES with the reference's :diag
// (Jacobi) preconditioner, and flexible GMRES whose preconditioner is
// z = D⁻¹(v + N(v)) with N the learned MLP (Jacobi plus a learned
// correction).  Systems the flexible solve leaves unconverged fall back to
// Jacobi GMRES from where it stopped, then to the direct solve.
//
// Device layout: one warp per radial system.  Lane l holds elements
// i = l + 32e (e < 8, so n ≤ 256) of every vector in registers; the banded
// operator (7 diagonals per row, one copy per wavenumber) and the Krylov
// bases V, Z (per system, rows of nmax doubles) live in global memory, which
// the 129 MB L2 keeps resident (1201 systems × 31 × 201 doubles ≈ 60 MB).
// Reductions are warp shuffles; no block barrier appears on the solve path.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ss_grid.h"
#include "ss_kernels.h"
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

// ---------------------------------------------------------------- host setup
// basis(sp, m, x, d) for d ≤ 2 (src/CubicBSpline.jl:585-628)
static double bval(const SplineHost &s, int m, double x, int d) {
    double b = 0.0, xm = s.xmin + (m * s.DX), delta = (x - xm) * s.DXrecip, z = std::fabs(delta);
    if (z < 2.0) {
        if (d == 0) {
            z = 2.0 - z; b = (z * z * z) * (1.0 / 6.0); z -= 1.0;
            if (z > 0) b -= (z * z * z) * (4.0 / 6.0);
        } else if (d == 1) {
            z = 2.0 - z; b = (z * z) * (1.0 / 6.0); z -= 1.0;
            if (z > 0) b -= (z * z) * (4.0 / 6.0);
            b *= ((delta > 0) ? -1.0 : 1.0) * 3.0 * s.DXrecip;
        } else {
            z = 2.0 - z; b = z; z -= 1.0;
            if (z > 0) b -= z * 4;
            b *= s.DXrecip * s.DXrecip;
        }
    }
    return b;
}
static double gam(const SplineHost &g, int i, int j) {  // 1-based Γ entry
    double val = (j == i + g.rankL) ? 1.0 : 0.0;
    if (g.lk == BC_A1) { if (j == 1) { if (i == 1) val += g.aL; if (i == 2) val += g.bL; } }
    else if (g.lk == BC_A2) { if (j == 1 && i == 1) val += g.aL; else if (j == 2 && i == 1) val += g.bL; }
    if (g.rk == BC_A1) { if (j == g.Mdim) { if (i == g.Min) val += g.aR; if (i == g.Min - 1) val += g.bR; } }
    else if (g.rk == BC_A2) { if (j == g.Mdim && i == g.Min) val += g.aR; else if (j == g.Mdim - 1 && i == g.Min) val += g.bR; }
    return val;
}

// dense G_m (n × n, row-major) of the template s for wavenumber m
static void assemble_operator(const SplineHost &s, int m, const std::vector<double> &k2, std::vector<double> &G) {
    const int b = s.bDim, n = s.Min;
    std::vector<double> Gf((size_t)b * b, 0.0);
    for (int mc = 0; mc < s.nc; mc++)
        for (int mu = 0; mu < s.mubar; mu++) {
            const int i = mu + s.mubar * mc;
            const double x = s.mish[i], m2 = double(m) * double(m);
            const double c1 = 1.0 / x, c0 = -(m2 / (x * x) + k2[i]);
            const long xm = (long)std::ceil((x - s.xmin - (2.0 * s.DX)) * s.DXrecip);
            for (long jj = xm; jj <= xm + 3; jj++) {
                if (jj < -1 || jj > s.nc + 1) continue;
                const double Lphi = bval(s, (int)jj, x, 2) + c1 * bval(s, (int)jj, x, 1) + c0 * bval(s, (int)jj, x, 0);
                for (int ti = std::max(mc - 1, -1); ti <= mc + 2; ti++) {
                    if (ti > s.nc + 1) continue;
                    const double w = s.DX * s.qw[mu] * bval(s, ti, x, 0);
                    Gf[(size_t)(ti + 1) * b + (jj + 1)] += w * Lphi;
                }
            }
        }
    G.assign((size_t)n * n, 0.0);
    for (int r = 1; r <= n; r++)
        for (int c = std::max(1, r - 6); c <= std::min(n, r + 6); c++) {
            double acc = 0.0;
            for (int a = std::max(1, r - 3); a <= std::min(b, r + 3 + s.rankL); a++) {
                const double ga = gam(s, r, a);
                if (ga == 0.0) continue;
                for (int bb = std::max(1, a - 3); bb <= std::min(b, a + 3); bb++) {
                    const double gb = gam(s, c, bb);
                    if (gb != 0.0) acc += ga * Gf[(size_t)(a - 1) * b + (bb - 1)] * gb;
                }
            }
            G[(size_t)(r - 1) * n + (c - 1)] = acc;
        }
}

struct GammaDev {
    int Md, Min, rankL, rankR, lk, rk, _p0, _p1;
    double aL, bL, aR, bR;
};

// band geometry the warp kernels are compiled for: 3 sub- and 3 superdiagonals
// (cubic B-splines), so U of the pivoted LU has 7 diagonals
constexpr int KL = 3, KU = 3, WG = KL + KU + 1, WU = KL + KU + 1;
constexpr int kPer = 8;               // vector elements per lane: n ≤ 256
constexpr int kMaxN = 32 * kPer;
constexpr int kSysPerBlock = 4;       // warps (systems) per CTA
constexpr int kMaxRestart = 100;

}  // namespace ss

struct ss_problem {
    ss_grid *g = nullptr;
    int K = 0, nsys = 0, nmax = 0, kl = 0, ku = 0;
    int n[2] = {0, 0};
    GammaDev gam[2];
    double *d_G = nullptr, *d_Lm = nullptr, *d_U = nullptr, *d_dinv = nullptr;
    int *d_piv = nullptr;
    GammaDev *d_gam = nullptr;
    double *d_rhs = nullptr, *d_x = nullptr, *d_res = nullptr, *d_cnorm = nullptr;
    int *d_iters = nullptr, *d_state = nullptr;
    // Krylov workspace (both GMRES variants)
    int ws_restart = 0;
    double *d_V = nullptr, *d_Z = nullptr, *d_H = nullptr, *d_gv = nullptr, *d_cs = nullptr, *d_sn = nullptr;
    int *d_cyc = nullptr;
    __nv_bfloat16 *d_mlp_in = nullptr;
    float *d_mlp_out = nullptr;
    ss_mlp *mlp = nullptr;
    int mpad = 0, mcut = 1 << 30;
    // gridpoints (r, λ) and blob parameters for training fields
    double *d_pts = nullptr, *d_blobs = nullptr;
    int64_t blobs_cap = 0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    std::vector<void *> allocs;
};

static int32_t palloc(ss_problem *p, void **ptr, size_t bytes) {
    if (cudaMalloc(ptr, bytes ? bytes : 16) != cudaSuccess) {
        cudaGetLastError();
        set_error("cudaMalloc(%zu) failed", bytes);
        return SS_OUT_OF_MEMORY;
    }
    p->allocs.push_back(*ptr);
    cudaMemset(*ptr, 0, bytes ? bytes : 16);
    return SS_OK;
}
template <typename V>
static int32_t pupload(ss_problem *p, V **dst, const std::vector<V> &v) {
    int32_t st = palloc(p, (void **)dst, v.size() * sizeof(V));
    if (st) return st;
    CUDA_TRY(cudaMemcpy(*dst, v.data(), v.size() * sizeof(V), cudaMemcpyHostToDevice));
    return SS_OK;
}

// ---------------------------------------------------------------- kernels
// spectral slot q: wavenumber (q + 1) / 2 ([k0 | k1 re | k1 im | ...]), template 0 (m = 0) or 1
__device__ __forceinline__ int slot_wavenumber(int q) { return (q + 1) / 2; }

struct SolveArgs {
    const double *spec;  // grid spectral: B-vectors in
    double *spec_out;    // coefficients a out
    const GammaDev *gam;
    const double *G, *Lm, *U, *dinv;  // G: [m][nmax][WG]; Lm: [m][nmax][KL]; U: [m][nmax][WU] (U[.][0] = 1/pivot)
    const int *piv;
    double *rhs, *x, *res, *cnorm;
    int *iters, *state;  // state: 0 active, 1 converged (or solved directly), 2 stopped inside a cycle
    double *V, *Z, *H, *gv, *cs, *sn;  // Krylov workspace per system
    int *cyc;
    __nv_bfloat16 *mlp_in;
    const float *mlp_out;
    int64_t nspec;
    int nsys, nslots, nvars, nmax, b, restart, max_iter, warm, masked, K, mcut, j;
    double tol;
};

__device__ __forceinline__ const GammaDev &gam_of(const SolveArgs &A, int m) { return A.gam[m == 0 ? 0 : 1]; }

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// per-warp shared scratch: one staged vector and the Gram–Schmidt coefficients
struct WarpSmem {
    double z[kSysPerBlock][kMaxN + 8];
    double h[kSysPerBlock][kMaxRestart + 1];
};

#define WARP_SYSTEM()                                                  \
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;         \
    const int sys = blockIdx.x * kSysPerBlock + wid;                   \
    if (sys >= A.nsys) return;                                         \
    const int q = sys % A.nslots, m = slot_wavenumber(q);              \
    const int n = gam_of(A, m).Min;

__device__ __forceinline__ void load_vec(double (&v)[kPer], const double *src, int n, int lane) {
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        v[e] = i < n ? src[i] : 0.0;
    }
}
__device__ __forceinline__ void store_vec(double *dst, const double (&v)[kPer], int n, int lane) {
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        if (i < n) dst[i] = v[e];
    }
}
__device__ __forceinline__ double dot_vec(const double (&a)[kPer], const double (&b)[kPer]) {
    double s = 0.0;
#pragma unroll
    for (int e = 0; e < kPer; e++) s += a[e] * b[e];
    return warp_sum(s);
}

// w = G_m z (radial_op_matvec): z staged in the warp's shared row, 7 diagonals per row
__device__ __forceinline__ void band_matvec_w(const double *G, const double (&z)[kPer], double (&w)[kPer], double *zs,
                                              int n, int lane) {
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        if (i < n) zs[i + KL] = z[e];
    }
    if (lane < KL) zs[lane] = 0.0;
    if (lane < KU) zs[n + KL + lane] = 0.0;
    __syncwarp();
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        double acc = 0.0;
        if (i < n) {
            const double *g = G + (size_t)i * WG;
#pragma unroll
            for (int t = 0; t < WG; t++) acc += g[t] * zs[i + t];
        }
        w[e] = acc;
    }
    __syncwarp();
}

// Orthogonalise w against V[0..jc) by modified Gram–Schmidt (the fewest FP64
// operations per step; FP64 runs at 1/64 of the FP32 rate on this part); the
// next row's load is issued before the current row's reduction.
__device__ __forceinline__ void mgs_w(const double *V, int ld, int jc, double (&w)[kPer], int n, int lane, double *hs) {
    double vk[kPer], vn[kPer];
    load_vec(vk, V, n, lane);
    for (int k = 0; k < jc; k++) {
        if (k + 1 < jc) load_vec(vn, V + (size_t)(k + 1) * ld, n, lane);
        const double h = dot_vec(w, vk);
#pragma unroll
        for (int e = 0; e < kPer; e++) w[e] -= h * vk[e];
        if (lane == 0) hs[k] = h;
#pragma unroll
        for (int e = 0; e < kPer; e++) vk[e] = vn[e];
    }
    __syncwarp();
}

// Givens update of column j of H and of g (lane 0)
__device__ __forceinline__ void givens_column(double *H, int R, int j, double *cs, double *sn, double *gv) {
    for (int k = 0; k < j; k++) {
        const double a = H[(size_t)k * R + j], bb = H[(size_t)(k + 1) * R + j];
        H[(size_t)k * R + j] = cs[k] * a + sn[k] * bb;
        H[(size_t)(k + 1) * R + j] = -sn[k] * a + cs[k] * bb;
    }
    const double a = H[(size_t)j * R + j], bb = H[(size_t)(j + 1) * R + j];
    const double rr = hypot(a, bb);
    cs[j] = rr > 0.0 ? a / rr : 1.0;
    sn[j] = rr > 0.0 ? bb / rr : 0.0;
    H[(size_t)j * R + j] = rr;
    H[(size_t)(j + 1) * R + j] = 0.0;
    gv[j + 1] = -sn[j] * gv[j];
    gv[j] = cs[j] * gv[j];
}

// y = H⁻¹ g over `steps` columns (lane 0), into ys
__device__ __forceinline__ void hessenberg_solve(const double *H, int R, const double *gv, int steps, double *ys) {
    for (int k = steps - 1; k >= 0; k--) {
        double s = gv[k];
        for (int l = k + 1; l < steps; l++) s -= H[(size_t)k * R + l] * ys[l];
        ys[k] = s / H[(size_t)k * R + k];
    }
}

// c = Γ_m b (src/CubicBSpline.jl:427-458), zero-padded to nmax; ‖c‖ per system
__global__ void __launch_bounds__(128) rhs_kernel(SolveArgs A) {
    WARP_SYSTEM();
    const GammaDev &g = gam_of(A, m);
    const int v = sys / A.nslots;
    const double *b = A.spec + (size_t)v * A.nspec + (size_t)q * A.b;
    double *r = A.rhs + (size_t)sys * A.nmax;
    const double b0 = b[0], b1 = b[1], bM1 = b[g.Md - 1], bM2 = b[g.Md - 2];
    double c[kPer];
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        double val = i < n ? b[i + g.rankL] : 0.0;
        if (i == 0) { if (g.lk == BC_A1) val += g.aL * b0; else if (g.lk == BC_A2) val += g.aL * b0 + g.bL * b1; }
        if (i == 1 && g.lk == BC_A1) val += g.bL * b0;
        if (i == n - 1) { if (g.rk == BC_A1) val += g.aR * bM1; else if (g.rk == BC_A2) val += g.aR * bM1 + g.bR * bM2; }
        if (i == n - 2 && g.rk == BC_A1) val += g.bR * bM1;
        c[e] = val;
        if (i < A.nmax) r[i] = val;
    }
    const double nrm = sqrt(dot_vec(c, c));
    if (lane == 0) A.cnorm[sys] = nrm;
}

// a = Γ_mᵀ x into the spectral array (src/CubicBSpline.jl:461-500)
__global__ void __launch_bounds__(128) unfold_kernel(SolveArgs A) {
    WARP_SYSTEM();
    const GammaDev &g = gam_of(A, m);
    const int v = sys / A.nslots;
    const double *x = A.x + (size_t)sys * A.nmax;
    double *a = A.spec_out + (size_t)v * A.nspec + (size_t)q * A.b;
    const int Md = g.Md, rL = g.rankL;
    const double x0 = x[0], x1 = x[1], xn1 = x[n - 1], xn2 = x[n - 2];
    for (int jx = lane; jx < Md; jx += 32) {
        double val = (jx >= rL && jx < rL + n) ? x[jx - rL] : 0.0;
        if (jx == 0) { if (g.lk == BC_A1) val = g.aL * x0 + g.bL * x1; else if (g.lk == BC_A2) val = g.aL * x0; }
        if (jx == 1 && g.lk == BC_A2) val = g.bL * x0;
        if (jx == Md - 1) { if (g.rk == BC_A1) val = g.aR * xn1 + g.bR * xn2; else if (g.rk == BC_A2) val = g.aR * xn1; }
        if (jx == Md - 2 && g.rk == BC_A2) val = g.bR * xn1;
        a[jx] = val;
    }
}

// direct solve: banded LU with partial pivoting (dgbtrs order).  The warp
// stages the right-hand side into shared memory; lane 0 runs both sweeps with
// the moving window of the band in registers.
__global__ void __launch_bounds__(128) direct_kernel(SolveArgs A) {
    __shared__ double xs[kSysPerBlock][kMaxN + 8];
    WARP_SYSTEM();
    if (A.masked && A.state[sys] == 1) return;
    double *xw = xs[wid];
    const double *r = A.rhs + (size_t)sys * A.nmax;
    for (int i = lane; i < n; i += 32) xw[i] = r[i];
    __syncwarp();
    if (lane == 0) {
        const double *Lm = A.Lm + (size_t)m * A.nmax * KL;
        const double *U = A.U + (size_t)m * A.nmax * WU;
        const int *piv = A.piv + (size_t)m * A.nmax;
        // forward: window w[0..KL] = x[k..k+KL]
        double w0 = xw[0], w1 = n > 1 ? xw[1] : 0.0, w2 = n > 2 ? xw[2] : 0.0, w3 = n > 3 ? xw[3] : 0.0;
        for (int k = 0; k < n; k++) {
            const int p = piv[k] - k;  // 0..KL
            if (p == 1) { const double t = w0; w0 = w1; w1 = t; }
            else if (p == 2) { const double t = w0; w0 = w2; w2 = t; }
            else if (p == 3) { const double t = w0; w0 = w3; w3 = t; }
            const double *l = Lm + (size_t)k * KL;
            w1 -= l[0] * w0;
            w2 -= l[1] * w0;
            w3 -= l[2] * w0;
            xw[k] = w0;
            w0 = w1; w1 = w2; w2 = w3;
            w3 = (k + 4 < n) ? xw[k + 4] : 0.0;
        }
        // backward: window y[1..6] = x[i+1..i+6]
        double y1 = 0.0, y2 = 0.0, y3 = 0.0, y4 = 0.0, y5 = 0.0, y6 = 0.0;
        for (int i = n - 1; i >= 0; i--) {
            const double *u = U + (size_t)i * WU;
            const double s = xw[i] - (u[1] * y1 + u[2] * y2) - (u[3] * y3 + u[4] * y4) - (u[5] * y5 + u[6] * y6);
            const double xi = s * u[0];
            xw[i] = xi;
            y6 = y5; y5 = y4; y4 = y3; y3 = y2; y2 = y1; y1 = xi;
        }
    }
    __syncwarp();
    double *x = A.x + (size_t)sys * A.nmax;
    for (int i = lane; i < n; i += 32) x[i] = xw[i];
    if (lane == 0) A.state[sys] = 1;
}

// true relative residual ‖c − G x‖ / ‖c‖
__global__ void __launch_bounds__(128) residual_kernel(SolveArgs A) {
    __shared__ double zs[kSysPerBlock][kMaxN + 8];
    WARP_SYSTEM();
    double x[kPer], w[kPer], c[kPer];
    load_vec(x, A.x + (size_t)sys * A.nmax, n, lane);
    load_vec(c, A.rhs + (size_t)sys * A.nmax, n, lane);
    band_matvec_w(A.G + (size_t)m * A.nmax * WG, x, w, zs[wid], n, lane);
#pragma unroll
    for (int e = 0; e < kPer; e++) w[e] = c[e] - w[e];
    const double rr = sqrt(dot_vec(w, w)) / (A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0);
    if (lane == 0) A.res[sys] = rr;
}

// block-wide sum (blockDim a multiple of 32, ≤ 1024)
__device__ double block_sum(double v, double *red) {
    v = warp_sum(v);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
    return s;
}

// w = G_m z with z and w in shared memory (block version)
__device__ __forceinline__ void band_matvec_b(const double *G, int n, const double *z, double *w) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double acc = 0.0;
#pragma unroll
        for (int t = 0; t < WG; t++) {
            const int j = i + t - KL;
            if (j >= 0 && j < n) acc += G[(size_t)i * WG + t] * z[j];
        }
        w[i] = acc;
    }
}

// restarted GMRES with right Jacobi preconditioning (the reference's :diag,
// src/solver_problem.jl:172-179).  One CTA per system with the Krylov basis in
// shared memory: FP64 throughput is 1/64 of FP32 on this part, so the slow
// low-wavenumber systems finish sooner when 128 threads share each iteration
// (modified Gram–Schmidt, the fewest FP64 operations per step).
__global__ void __launch_bounds__(128) gmres_kernel(SolveArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[32];
    const int sys = blockIdx.x;
    if (A.masked && A.state[sys] == 1) return;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min, R = A.restart;
    const double *G = A.G + (size_t)m * A.nmax * WG;
    const double *dv = A.dinv + (size_t)m * A.nmax;
    double *V = reinterpret_cast<double *>(smem_raw);   // (R+1) × n
    double *w = V + (size_t)(R + 1) * n;                 // n
    double *z = w + n;                                    // n
    double *H = z + n;                                    // (R+1) × R
    double *cs = H + (size_t)(R + 1) * R, *sn = cs + R, *gv = sn + R, *yv = gv + R + 1;
    double *x = A.x + (size_t)sys * A.nmax;
    const double *c = A.rhs + (size_t)sys * A.nmax;
    const double cn = A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0;
    if (!A.warm)
        for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = 0.0;
    __syncthreads();
    int it = 0;
    double rel = 1.0;
    while (it < A.max_iter) {
        band_matvec_b(G, n, x, w);
        __syncthreads();
        double part = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) { w[i] = c[i] - w[i]; part += w[i] * w[i]; }
        const double beta = sqrt(block_sum(part, red));
        rel = beta / cn;
        if (rel <= A.tol || beta == 0.0) break;
        for (int i = threadIdx.x; i < n; i += blockDim.x) V[i] = w[i] / beta;
        if (threadIdx.x == 0) { gv[0] = beta; for (int i = 1; i <= R; i++) gv[i] = 0.0; }
        __syncthreads();
        int j = 0;
        for (; j < R && it < A.max_iter; j++, it++) {
            for (int i = threadIdx.x; i < n; i += blockDim.x) z[i] = dv[i] * V[(size_t)j * n + i];
            __syncthreads();
            band_matvec_b(G, n, z, w);
            __syncthreads();
            for (int k = 0; k <= j; k++) {  // modified Gram–Schmidt
                double pk = 0.0;
                for (int i = threadIdx.x; i < n; i += blockDim.x) pk += w[i] * V[(size_t)k * n + i];
                const double hk = block_sum(pk, red);
                for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] -= hk * V[(size_t)k * n + i];
                if (threadIdx.x == 0) H[(size_t)k * R + j] = hk;
                __syncthreads();
            }
            double pn = 0.0;
            for (int i = threadIdx.x; i < n; i += blockDim.x) pn += w[i] * w[i];
            const double hn = sqrt(block_sum(pn, red));
            for (int i = threadIdx.x; i < n; i += blockDim.x) V[(size_t)(j + 1) * n + i] = hn > 0.0 ? w[i] / hn : 0.0;
            if (threadIdx.x == 0) {
                H[(size_t)(j + 1) * R + j] = hn;
                givens_column(H, R, j, cs, sn, gv);
            }
            __syncthreads();
            rel = fabs(gv[j + 1]) / cn;
            if (rel <= A.tol || hn == 0.0) { j++; it++; break; }
        }
        if (threadIdx.x == 0) hessenberg_solve(H, R, gv, j, yv);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {  // x += D⁻¹ V y
            double acc = 0.0;
            for (int k = 0; k < j; k++) acc += V[(size_t)k * n + i] * yv[k];
            x[i] += dv[i] * acc;
        }
        __syncthreads();
        if (rel <= A.tol) break;
    }
    band_matvec_b(G, n, x, w);  // true residual
    __syncthreads();
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { const double d = c[i] - w[i]; part += d * d; }
    const double rr = sqrt(block_sum(part, red)) / cn;
    if (threadIdx.x == 0) {
        A.res[sys] = rr;
        A.iters[sys] += it;
        if (rr <= A.tol) A.state[sys] = 1;
    }
}

static size_t gmres_smem(int R, int n) {
    return ((size_t)(R + 1) * n + 2 * (size_t)n + (size_t)(R + 1) * R + 4 * (size_t)R + 4) * 8;
}

// ---------------------------------------------------------------- flexible GMRES
// All systems advance in lockstep so the MLP runs as one batched tensor-core
// pass per Arnoldi step.  MLP input row of a system: v (first n entries),
// zeros, then the features m/K and log(1+m)/log(1+K) in the last two columns.
__device__ __forceinline__ void write_mlp_row_w(__nv_bfloat16 *row, const double (&v)[kPer], double scale, int n, int m,
                                                int K, int lane) {
    const float f0 = (float)m / (float)(K > 0 ? K : 1);
    const float f1 = (float)(log1p((double)m) / log1p((double)(K > 0 ? K : 1)));
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;  // covers 0..255
        float val = 0.f;
        if (i < n) val = (float)(v[e] * scale);
        else if (i == kMlpWidth - 2) val = f0;
        else if (i == kMlpWidth - 1) val = f1;
        row[i] = __float2bfloat16(val);
    }
}

// start of a cycle: r = c − G x; converged systems leave; else v0 = r / β
__global__ void __launch_bounds__(128) fg_begin_kernel(SolveArgs A) {
    __shared__ double zs[kSysPerBlock][kMaxN + 8];
    WARP_SYSTEM();
    const int R = A.restart;
    __nv_bfloat16 *row = A.mlp_in + (size_t)sys * kMlpWidth;
    double x[kPer], c[kPer], w[kPer];
    if (A.state[sys] == 1) {
#pragma unroll
        for (int e = 0; e < kPer; e++) w[e] = 0.0;
        write_mlp_row_w(row, w, 0.0, 0, m, A.K, lane);
        return;
    }
    load_vec(x, A.x + (size_t)sys * A.nmax, n, lane);
    load_vec(c, A.rhs + (size_t)sys * A.nmax, n, lane);
    band_matvec_w(A.G + (size_t)m * A.nmax * WG, x, w, zs[wid], n, lane);
#pragma unroll
    for (int e = 0; e < kPer; e++) w[e] = c[e] - w[e];
    const double beta = sqrt(dot_vec(w, w));
    const double cn = A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0;
    if (beta / cn <= A.tol || beta == 0.0) {
        if (lane == 0) { A.state[sys] = 1; A.res[sys] = beta / cn; }
#pragma unroll
        for (int e = 0; e < kPer; e++) w[e] = 0.0;
        write_mlp_row_w(row, w, 0.0, 0, m, A.K, lane);
        return;
    }
#pragma unroll
    for (int e = 0; e < kPer; e++) w[e] /= beta;
    store_vec(A.V + (size_t)sys * (R + 1) * A.nmax, w, n, lane);
    if (lane == 0) {
        double *gv = A.gv + (size_t)sys * (R + 1);
        gv[0] = beta;
        for (int i = 1; i <= R; i++) gv[i] = 0.0;
        A.state[sys] = 0;
        A.cyc[sys] = 0;
    }
    write_mlp_row_w(row, w, 1.0, n, m, A.K, lane);
}

// Arnoldi step j: z_j = D⁻¹(v_j + N(v_j)), w = G z_j, orthogonalise, Givens, next MLP input
__global__ void __launch_bounds__(128) fg_step_kernel(SolveArgs A) {
    __shared__ WarpSmem S;
    WARP_SYSTEM();
    if (A.state[sys] != 0) return;
    const int R = A.restart, j = A.j, ld = A.nmax;
    double *V = A.V + (size_t)sys * (R + 1) * ld;
    double *H = A.H + (size_t)sys * (R + 1) * R;
    double *gv = A.gv + (size_t)sys * (R + 1), *cs = A.cs + (size_t)sys * R, *sn = A.sn + (size_t)sys * R;
    double dv[kPer], v[kPer], z[kPer], w[kPer];
    load_vec(dv, A.dinv + (size_t)m * A.nmax, n, lane);
    load_vec(v, V + (size_t)j * ld, n, lane);
    const float *o = A.mlp_out + (size_t)sys * kMlpWidth;
    const bool learned = m <= A.mcut;
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        z[e] = i < n ? dv[e] * (v[e] + (learned ? (double)o[i] : 0.0)) : 0.0;
    }
    store_vec(A.Z + (size_t)sys * R * ld + (size_t)j * ld, z, n, lane);
    band_matvec_w(A.G + (size_t)m * A.nmax * WG, z, w, S.z[wid], n, lane);
    mgs_w(V, ld, j + 1, w, n, lane, S.h[wid]);
    const double hn = sqrt(dot_vec(w, w));
#pragma unroll
    for (int e = 0; e < kPer; e++) w[e] = hn > 0.0 ? w[e] / hn : 0.0;
    store_vec(V + (size_t)(j + 1) * ld, w, n, lane);
    double g1 = 0.0;
    if (lane == 0) {
        for (int k = 0; k <= j; k++) H[(size_t)k * R + j] = S.h[wid][k];
        H[(size_t)(j + 1) * R + j] = hn;
        givens_column(H, R, j, cs, sn, gv);
        A.iters[sys] += 1;
        A.cyc[sys] = j + 1;
        g1 = gv[j + 1];
    }
    g1 = __shfl_sync(0xffffffffu, g1, 0);
    const double cn = A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0;
    if (fabs(g1) / cn <= A.tol || hn == 0.0) {
        if (lane == 0) A.state[sys] = 2;  // converged estimate: stop this cycle
        return;
    }
    write_mlp_row_w(A.mlp_in + (size_t)sys * kMlpWidth, w, 1.0, n, m, A.K, lane);
}

// end of a cycle: x += Z y over the steps this system took
__global__ void __launch_bounds__(128) fg_end_kernel(SolveArgs A) {
    __shared__ double ys[kSysPerBlock][kMaxRestart + 1];
    WARP_SYSTEM();
    if (A.state[sys] == 1) return;
    const int R = A.restart, steps = A.cyc[sys], ld = A.nmax;
    const double *Z = A.Z + (size_t)sys * R * ld;
    if (lane == 0) hessenberg_solve(A.H + (size_t)sys * (R + 1) * R, R, A.gv + (size_t)sys * (R + 1), steps, ys[wid]);
    __syncwarp();
    double x[kPer];
    double *xg = A.x + (size_t)sys * ld;
    load_vec(x, xg, n, lane);
    for (int k = 0; k < steps; k++) {
        const double yk = ys[wid][k];
        const double *zk = Z + (size_t)k * ld;
#pragma unroll
        for (int e = 0; e < kPer; e++) {
            const int i = lane + 32 * e;
            if (i < n) x[e] += yk * zk[i];
        }
    }
    store_vec(xg, x, n, lane);
    if (lane == 0) A.state[sys] = 0;
}

// ---------------------------------------------------------------- training fields
// f(r, λ) = Σ A exp(−[(x − xc)² + (y − yc)²]/w²), x = r cos λ, y = r sin λ, in every variable
__global__ void blob_field_kernel(double *phys, int64_t np, int nvars, const double *pts, const double *blobs,
                                  int nb) {
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const double r = pts[i], lam = pts[np + i];
    const double x = r * cos(lam), y = r * sin(lam);
    double f = 0.0;
    for (int k = 0; k < nb; k++) {
        const double *bp = blobs + 4 * k;
        const double dx = x - bp[0], dy = y - bp[1];
        f += bp[3] * exp(-(dx * dx + dy * dy) / (bp[2] * bp[2]));
    }
    for (int v = 0; v < nvars; v++) phys[(size_t)v * np + i] = f;
}

// counter-based normal deviates (splitmix64 mixing + Box–Muller) for random right-hand sides
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double normal_dev(uint64_t seed, uint64_t idx) {
    const uint64_t a = mix64(seed ^ mix64(2 * idx)), b = mix64(seed ^ mix64(2 * idx + 1));
    const double u1 = ((a >> 11) + 1.0) * (1.0 / 9007199254740993.0);  // (0, 1]
    const double u2 = (b >> 11) * (1.0 / 9007199254740992.0);
    return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

// c = white noise smoothed `smooth` times by a (1, 2, 1)/4 filter, per system
__global__ void __launch_bounds__(128) rhs_random_kernel(SolveArgs A, uint64_t seed, int smooth) {
    __shared__ double ws[kSysPerBlock][kMaxN + 2];
    WARP_SYSTEM();
    double *w = ws[wid] + 1;
    for (int i = lane; i < n; i += 32) w[i] = normal_dev(seed, (uint64_t)sys * A.nmax + i);
    if (lane == 0) { w[-1] = 0.0; w[n] = 0.0; }
    __syncwarp();
    double c[kPer];
    for (int s = 0; s < smooth; s++) {
#pragma unroll
        for (int e = 0; e < kPer; e++) {
            const int i = lane + 32 * e;
            c[e] = i < n ? 0.25 * (w[i - 1] + 2.0 * w[i] + w[i + 1]) : 0.0;
        }
        __syncwarp();
        store_vec(w, c, n, lane);
        __syncwarp();
    }
    load_vec(c, w, n, lane);
    double *r = A.rhs + (size_t)sys * A.nmax;
    for (int i = lane; i < A.nmax; i += 32) r[i] = i < n ? w[i] : 0.0;
    const double nrm = sqrt(dot_vec(c, c));
    if (lane == 0) A.cnorm[sys] = nrm;
}

// training rows from the direct solution: input v = c/‖c‖, target D x/‖c‖ − v
__global__ void __launch_bounds__(128) training_rows_kernel(SolveArgs A, int64_t row0, __nv_bfloat16 *X,
                                                            __nv_bfloat16 *T, int32_t *nrow) {
    WARP_SYSTEM();
    if (m > A.mcut) return;
    // rows are packed per variable: the slots of wavenumbers ≤ mcut in slot order
    const int per_var = 1 + 2 * min(A.mcut, A.K);
    const int64_t row = row0 + (int64_t)(sys / A.nslots) * per_var + q;
    double c[kPer], x[kPer], dv[kPer];
    load_vec(c, A.rhs + (size_t)sys * A.nmax, n, lane);
    load_vec(x, A.x + (size_t)sys * A.nmax, n, lane);
    load_vec(dv, A.dinv + (size_t)m * A.nmax, n, lane);
    const double cn = A.cnorm[sys];
    const double s = cn > 0.0 ? 1.0 / cn : 0.0;
    write_mlp_row_w(X + row * kMlpWidth, c, s, n, m, A.K, lane);
#pragma unroll
    for (int e = 0; e < kPer; e++) {
        const int i = lane + 32 * e;
        const float t = i < n ? (float)((x[e] / dv[e] - c[e]) * s) : 0.f;
        T[row * kMlpWidth + i] = __float2bfloat16(t);
    }
    if (lane == 0) nrow[row] = n;
}

// ---------------------------------------------------------------- C ABI
extern "C" int32_t ss_problem_create(ss_grid *g, const double *k2, ss_problem **out) {
    if (!g || !k2 || !out) { set_error("null argument"); return SS_BAD_ARG; }
    *out = nullptr;
    if (g->rlz || g->esz != 8 || g->prec != SS_PREC_F64) {
        set_error("the elliptic solve runs on native-FP64 RL grids");
        return SS_BAD_ARG;
    }
    cudaSetDevice(g->device);
    const ss_grid_params &gp = g->p;
    const int iDim = (int)g->d.iDim;
    std::vector<double> kk(k2, k2 + iDim);
    // templates: m = 0 (u'(0) = 0, u(R) = 0) and m ≥ 1 (u(0) = 0, u(R) = 0)
    ss_spline_bc r1t0{SS_SBC_RANK1, 0, -4.0, -1.0}, r1t1{SS_SBC_RANK1, 0, 0.0, 1.0};
    SplineHost tpl[2];
    int32_t st = build_spline(gp.iMin, gp.iMax, gp.num_cells, gp.mubar, gp.quadrature, g->l_q[0], r1t1, r1t0, tpl[0]);
    if (!st) st = build_spline(gp.iMin, gp.iMax, gp.num_cells, gp.mubar, gp.quadrature, g->l_q[0], r1t0, r1t0, tpl[1]);
    if (st) return st;
    if (std::max(tpl[0].Min, tpl[1].Min) > kMaxN) {
        set_error("radial systems of %d unknowns exceed %d", std::max(tpl[0].Min, tpl[1].Min), kMaxN);
        return SS_BAD_SHAPE;
    }
    ss_problem *p = new ss_problem();
    p->g = g;
    for (int t = 0; t < 2; t++) {
        const SplineHost &s = tpl[t];
        GammaDev &gd = p->gam[t];
        std::memset(&gd, 0, sizeof gd);
        gd.Md = s.bDim; gd.Min = s.Min; gd.rankL = s.rankL; gd.rankR = s.rankR; gd.lk = s.lk; gd.rk = s.rk;
        gd.aL = s.aL; gd.bL = s.bL; gd.aR = s.aR; gd.bR = s.bR;
        p->n[t] = s.Min;
    }
    p->K = (int)g->d.kDim_wn;
    p->nmax = std::max(p->n[0], p->n[1]);
    p->nsys = (int)g->d.nvars * (1 + 2 * p->K);
    // operators, band widths, LU factors and Jacobi diagonals per wavenumber
    std::vector<std::vector<double>> Gs(p->K + 1);
    int kl = 0, ku = 0;
    for (int m = 0; m <= p->K; m++) {
        const SplineHost &s = tpl[m == 0 ? 0 : 1];
        assemble_operator(s, m, kk, Gs[m]);
        const int n = s.Min;
        for (int i = 0; i < n; i++)
            for (int j = std::max(0, i - 8); j < std::min(n, i + 9); j++)
                if (Gs[m][(size_t)i * n + j] != 0.0) { kl = std::max(kl, i - j); ku = std::max(ku, j - i); }
    }
    if (kl > KL || ku > KU) {
        delete p;
        set_error("radial operator bandwidth (%d, %d) exceeds (3, 3)", kl, ku);
        return SS_BAD_SHAPE;
    }
    p->kl = KL; p->ku = KU;
    const int nm = p->nmax, Kp = p->K + 1;
    std::vector<double> hG((size_t)Kp * nm * WG, 0.0), hL((size_t)Kp * nm * KL, 0.0), hU((size_t)Kp * nm * WU, 0.0),
        hD((size_t)Kp * nm, 1.0);
    std::vector<int> hP((size_t)Kp * nm, 0);
    for (int m = 0; m <= p->K; m++) {
        const int n = p->n[m == 0 ? 0 : 1];
        std::vector<double> &A = Gs[m];
        for (int i = 0; i < n; i++) {
            for (int t = 0; t < WG; t++) {
                const int j = i + t - KL;
                if (j >= 0 && j < n) hG[((size_t)m * nm + i) * WG + t] = A[(size_t)i * n + j];
            }
            const double d = A[(size_t)i * n + i];
            hD[(size_t)m * nm + i] = std::fabs(d) > 0.0 ? 1.0 / d : 1.0;
        }
        // banded LU with partial pivoting (dgbtf2 order); U gains KL superdiagonals
        for (int k = 0; k < n; k++) {
            int piv = k;
            double mx = std::fabs(A[(size_t)k * n + k]);
            for (int i = k + 1; i <= std::min(n - 1, k + KL); i++)
                if (std::fabs(A[(size_t)i * n + k]) > mx) { mx = std::fabs(A[(size_t)i * n + k]); piv = i; }
            if (mx == 0.0) { delete p; set_error("singular radial operator at wavenumber %d", m); return SS_NOT_SPD; }
            hP[(size_t)m * nm + k] = piv;
            const int jend = std::min(n - 1, k + KL + KU);
            if (piv != k)
                for (int j = k; j <= jend; j++) std::swap(A[(size_t)k * n + j], A[(size_t)piv * n + j]);
            for (int i = k + 1; i <= std::min(n - 1, k + KL); i++) {
                const double l = A[(size_t)i * n + k] / A[(size_t)k * n + k];
                hL[((size_t)m * nm + k) * KL + (i - k - 1)] = l;
                for (int j = k + 1; j <= jend; j++) A[(size_t)i * n + j] -= l * A[(size_t)k * n + j];
            }
            hU[((size_t)m * nm + k) * WU] = 1.0 / A[(size_t)k * n + k];  // the pivot, inverted
            for (int t = 1; t < WU && k + t < n; t++) hU[((size_t)m * nm + k) * WU + t] = A[(size_t)k * n + k + t];
        }
        std::vector<double>().swap(A);
    }
    if ((st = pupload(p, &p->d_G, hG)) || (st = pupload(p, &p->d_Lm, hL)) || (st = pupload(p, &p->d_U, hU)) ||
        (st = pupload(p, &p->d_dinv, hD)) || (st = pupload(p, &p->d_piv, hP))) {
        ss_problem_destroy(p);
        return st;
    }
    std::vector<GammaDev> gv(p->gam, p->gam + 2);
    if ((st = pupload(p, &p->d_gam, gv)) || (st = palloc(p, (void **)&p->d_rhs, (size_t)p->nsys * nm * 8)) ||
        (st = palloc(p, (void **)&p->d_x, (size_t)p->nsys * nm * 8)) ||
        (st = palloc(p, (void **)&p->d_res, (size_t)p->nsys * 8)) ||
        (st = palloc(p, (void **)&p->d_cnorm, (size_t)p->nsys * 8)) ||
        (st = palloc(p, (void **)&p->d_iters, (size_t)p->nsys * 4)) ||
        (st = palloc(p, (void **)&p->d_state, (size_t)p->nsys * 4))) {
        ss_problem_destroy(p);
        return st;
    }
    cudaEventCreate(&p->e0);
    cudaEventCreate(&p->e1);
    *out = p;
    return SS_OK;
}

extern "C" int32_t ss_problem_destroy(ss_problem *p) {
    if (!p) return SS_OK;
    cudaSetDevice(p->g->device);
    cudaDeviceSynchronize();
    for (void *a : p->allocs) cudaFree(a);
    if (p->e0) cudaEventDestroy(p->e0);
    if (p->e1) cudaEventDestroy(p->e1);
    delete p;
    return SS_OK;
}

extern "C" int32_t ss_problem_dims(const ss_problem *p, int32_t *nsys, int32_t *nmax, int32_t *K, int32_t *bandwidth) {
    if (!p) { set_error("null problem"); return SS_BAD_ARG; }
    if (nsys) *nsys = p->nsys;
    if (nmax) *nmax = p->nmax;
    if (K) *K = p->K;
    if (bandwidth) *bandwidth = WG;
    return SS_OK;
}

extern "C" int32_t ss_problem_set_mlp(ss_problem *p, ss_mlp *mlp, int32_t max_wavenumber) {
    if (!p) { set_error("null problem"); return SS_BAD_ARG; }
    if (mlp && p->nmax > kMlpWidth - 2) {
        set_error("radial systems of %d unknowns exceed the network width", p->nmax);
        return SS_BAD_SHAPE;
    }
    if (mlp && mlp->device != p->g->device) { set_error("network and grid on different devices"); return SS_BAD_ARG; }
    p->mlp = mlp;
    p->mcut = max_wavenumber < 0 ? (1 << 30) : max_wavenumber;
    return SS_OK;
}

// the operator G_m in band storage (row i: G[i][i + t − kl] at i·bandwidth + t; nmax rows)
extern "C" int32_t ss_problem_operator_band(const ss_problem *p, int32_t m, double *band, int32_t *n, int32_t *kl) {
    if (!p || m < 0 || m > p->K) { set_error("wavenumber out of range"); return SS_BAD_ARG; }
    cudaSetDevice(p->g->device);
    if (n) *n = p->n[m == 0 ? 0 : 1];
    if (kl) *kl = KL;
    if (band)
        CUDA_TRY(cudaMemcpy(band, p->d_G + (size_t)m * p->nmax * WG, (size_t)p->nmax * WG * 8, cudaMemcpyDeviceToHost));
    return SS_OK;
}

static SolveArgs solve_args(ss_problem *p, int restart, int max_iter, double tol) {
    ss_grid *g = p->g;
    SolveArgs A{};
    A.spec = (const double *)g->spec; A.spec_out = (double *)g->spec; A.gam = p->d_gam;
    A.G = p->d_G; A.Lm = p->d_Lm; A.U = p->d_U; A.dinv = p->d_dinv; A.piv = p->d_piv;
    A.rhs = p->d_rhs; A.x = p->d_x; A.res = p->d_res; A.cnorm = p->d_cnorm; A.iters = p->d_iters; A.state = p->d_state;
    A.V = p->d_V; A.Z = p->d_Z; A.H = p->d_H; A.gv = p->d_gv; A.cs = p->d_cs; A.sn = p->d_sn; A.cyc = p->d_cyc;
    A.mlp_in = p->d_mlp_in; A.mlp_out = p->d_mlp_out;
    A.nspec = g->d.n_spectral; A.nsys = p->nsys; A.nslots = 1 + 2 * p->K; A.nvars = (int)g->d.nvars;
    A.nmax = p->nmax; A.b = (int)g->d.b_iDim; A.K = p->K; A.mcut = p->mcut;
    A.restart = restart; A.max_iter = max_iter; A.tol = tol;
    return A;
}

static int32_t ensure_workspace(ss_problem *p, int R) {
    if (p->ws_restart >= R && p->d_V) return SS_OK;
    const size_t ns = p->nsys, nm = p->nmax;
    int32_t st;
    if ((st = palloc(p, (void **)&p->d_V, ns * (R + 1) * nm * 8)) || (st = palloc(p, (void **)&p->d_Z, ns * R * nm * 8)) ||
        (st = palloc(p, (void **)&p->d_H, ns * (R + 1) * R * 8)) || (st = palloc(p, (void **)&p->d_gv, ns * (R + 1) * 8)) ||
        (st = palloc(p, (void **)&p->d_cs, ns * R * 8)) || (st = palloc(p, (void **)&p->d_sn, ns * R * 8)))
        return st;
    if (!p->d_cyc) {
        p->mpad = (int)((ns + kMlpTileM - 1) / kMlpTileM * kMlpTileM);
        if ((st = palloc(p, (void **)&p->d_cyc, ns * 4)) ||
            (st = palloc(p, (void **)&p->d_mlp_in, (size_t)p->mpad * kMlpWidth * 2)) ||
            (st = palloc(p, (void **)&p->d_mlp_out, (size_t)p->mpad * kMlpWidth * 4)))
            return st;
    }
    p->ws_restart = R;
    return SS_OK;
}

static inline unsigned warp_blocks(int nsys) { return (unsigned)((nsys + kSysPerBlock - 1) / kSysPerBlock); }

static int32_t run_gmres(ss_problem *p, const SolveArgs &A, cudaStream_t st) {
    const size_t smem = gmres_smem(A.restart, p->nmax);
    if (smem > 200 * 1024) { set_error("restart %d too long for shared memory", A.restart); return SS_BAD_ARG; }
    if (smem > 48 * 1024) CUDA_TRY(cudaFuncSetAttribute(gmres_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gmres_kernel<<<p->nsys, 128, smem, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

// the chosen backend on the right-hand sides already in d_rhs (no transforms)
static int32_t solve_systems(ss_problem *p, int method, SolveArgs A, cudaStream_t st, int *fallback) {
    const int ns = p->nsys;
    const unsigned nb = warp_blocks(ns);
    int32_t r;
    *fallback = 0;
    CUDA_TRY(cudaMemsetAsync(p->d_iters, 0, (size_t)ns * 4, st));
    CUDA_TRY(cudaMemsetAsync(p->d_state, 0, (size_t)ns * 4, st));
    if (method == SS_SOLVER_DIRECT) {
        A.masked = 0;
        direct_kernel<<<nb, 128, 0, st>>>(A);
        CUDA_TRY(cudaGetLastError());
        residual_kernel<<<nb, 128, 0, st>>>(A);
        CUDA_TRY(cudaGetLastError());
        return SS_OK;
    }
    if (method == SS_SOLVER_GMRES_JACOBI) {
        A.warm = 0; A.masked = 0;
        return run_gmres(p, A, st);
    }
    // flexible GMRES with the learned preconditioner, cycles in lockstep
    if ((r = mlp_reserve(p->mlp, p->mpad))) return r;
    CUDA_TRY(cudaMemsetAsync(p->d_x, 0, (size_t)ns * p->nmax * 8, st));
    fg_begin_kernel<<<nb, 128, 0, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    int done_iters = 0;
    std::vector<int> hstate(ns);
    while (done_iters < A.max_iter) {
        const int steps = std::min(A.restart, A.max_iter - done_iters);
        for (int j = 0; j < steps; j++) {
            A.j = j;
            if ((r = mlp_forward(p->mlp, p->d_mlp_in, p->d_mlp_out, p->mpad, st))) return r;
            fg_step_kernel<<<nb, 128, 0, st>>>(A);
            CUDA_TRY(cudaGetLastError());
        }
        fg_end_kernel<<<nb, 128, 0, st>>>(A);
        CUDA_TRY(cudaGetLastError());
        done_iters += steps;
        fg_begin_kernel<<<nb, 128, 0, st>>>(A);  // true residual: converged systems leave, others restart
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(hstate.data(), p->d_state, (size_t)ns * 4, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        bool all = true;
        for (int v : hstate) all = all && (v == 1);
        if (all) break;
    }
    int err = 0;
    CUDA_TRY(cudaMemcpy(&err, p->mlp->err, sizeof(int), cudaMemcpyDeviceToHost));
    if (err) { cudaMemset(p->mlp->err, 0, sizeof(int)); set_error("tensor-core GEMM wait gave up"); return SS_DEVICE_TIMEOUT; }
    int left = 0;
    for (int v : hstate) left += (v != 1);
    if (left) {  // fall back: Jacobi GMRES from the current iterate, then the direct solve
        *fallback = left;
        A.warm = 1; A.masked = 1;
        if ((r = run_gmres(p, A, st))) return r;
        direct_kernel<<<nb, 128, 0, st>>>(A);
        CUDA_TRY(cudaGetLastError());
    }
    residual_kernel<<<nb, 128, 0, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

extern "C" int32_t ss_solve(ss_problem *p, int32_t method, double tol, int32_t max_iter, int32_t restart,
                            ss_solve_stats *stats, void *stream) {
    if (!p) { set_error("null problem"); return SS_BAD_ARG; }
    if (method < SS_SOLVER_DIRECT || method > SS_SOLVER_FGMRES_MLP) { set_error("unknown solver"); return SS_BAD_ARG; }
    if (!(tol > 0.0)) { set_error("tolerance must be positive"); return SS_BAD_ARG; }
    if (restart < 1) restart = 30;
    if (restart > kMaxRestart) { set_error("restart must be <= %d", kMaxRestart); return SS_BAD_ARG; }
    if (max_iter < 1) max_iter = 2000;
    if (method == SS_SOLVER_FGMRES_MLP && !p->mlp) { set_error("no MLP preconditioner attached"); return SS_BAD_ARG; }
    ss_grid *g = p->g;
    cudaSetDevice(g->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    int32_t r;
    if (method != SS_SOLVER_DIRECT && (r = ensure_workspace(p, restart))) return r;
    if ((r = grid_forward(g, st))) return r;  // f (physical slot 1) → spectral B-vectors
    SolveArgs A = solve_args(p, restart, max_iter, tol);
    CUDA_TRY(cudaEventRecord(p->e0, st));
    rhs_kernel<<<warp_blocks(p->nsys), 128, 0, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    int fallback = 0;
    if ((r = solve_systems(p, method, A, st, &fallback))) return r;
    unfold_kernel<<<warp_blocks(p->nsys), 128, 0, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaEventRecord(p->e1, st));
    if ((r = grid_inverse_coeffs(g, st))) return r;  // a → u and its derivatives in the physical slots
    if (stats) {
        CUDA_TRY(cudaStreamSynchronize(st));
        float ms = 0.f;
        CUDA_TRY(cudaEventElapsedTime(&ms, p->e0, p->e1));
        const int ns = p->nsys;
        std::vector<int> it(ns);
        std::vector<double> res(ns);
        CUDA_TRY(cudaMemcpy(it.data(), p->d_iters, (size_t)ns * 4, cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(res.data(), p->d_res, (size_t)ns * 8, cudaMemcpyDeviceToHost));
        std::memset(stats, 0, sizeof *stats);
        stats->method = method;
        stats->systems = ns;
        stats->fallback_systems = fallback;
        double sum = 0.0, mx = 0.0;
        for (int i = 0; i < ns; i++) {
            stats->max_iterations = std::max(stats->max_iterations, it[i]);
            sum += it[i];
            mx = std::max(mx, res[i]);
            if (res[i] <= tol) stats->converged++;
        }
        stats->mean_iterations = sum / ns;
        stats->max_rel_residual = mx;
        stats->ms = ms;
    }
    return SS_OK;
}

// right-hand sides c and solutions x of the last solve (nsys × nmax, row-major)
extern "C" int32_t ss_problem_export(const ss_problem *p, double *rhs, double *x, double *res, int32_t *iters) {
    if (!p) { set_error("null problem"); return SS_BAD_ARG; }
    cudaSetDevice(p->g->device);
    CUDA_TRY(cudaDeviceSynchronize());
    const size_t n = (size_t)p->nsys * p->nmax;
    if (rhs) CUDA_TRY(cudaMemcpy(rhs, p->d_rhs, n * 8, cudaMemcpyDeviceToHost));
    if (x) CUDA_TRY(cudaMemcpy(x, p->d_x, n * 8, cudaMemcpyDeviceToHost));
    if (res) CUDA_TRY(cudaMemcpy(res, p->d_res, (size_t)p->nsys * 8, cudaMemcpyDeviceToHost));
    if (iters) CUDA_TRY(cudaMemcpy(iters, p->d_iters, (size_t)p->nsys * 4, cudaMemcpyDeviceToHost));
    return SS_OK;
}

static int32_t check_training_args(ss_problem *p, ss_mlp *mlp) {
    if (p->nmax > kMlpWidth - 2) { set_error("radial systems exceed the network width"); return SS_BAD_SHAPE; }
    if (mlp->device != p->g->device) { set_error("network and grid on different devices"); return SS_BAD_ARG; }
    return SS_OK;
}

// Training pairs from the direct solve: for each field (blobs[offsets[f] ..
// offsets[f+1]) as (xc, yc, w, A) quadruples) the field is evaluated on the
// device at the gridpoints `pts` (n_physical × 2: r then λ), transformed,
// solved directly, and each radial system of wavenumber ≤ max_wavenumber is
// appended to the network's resident training set.
extern "C" int32_t ss_problem_collect_training(ss_problem *p, ss_mlp *mlp, const double *pts, const double *blobs,
                                               const int32_t *offsets, int32_t nfields, int32_t max_wavenumber) {
    if (!p || !mlp || !blobs || !offsets || nfields < 0) { set_error("bad argument"); return SS_BAD_ARG; }
    int32_t r;
    if ((r = check_training_args(p, mlp))) return r;
    for (int f = 0; f < nfields; f++)
        if (offsets[f + 1] < offsets[f] || offsets[f] < 0) { set_error("blob offsets decrease"); return SS_BAD_ARG; }
    ss_grid *g = p->g;
    cudaSetDevice(g->device);
    cudaStream_t st = g->stream;
    const int64_t np = g->d.n_physical;
    if (pts) {
        if (!p->d_pts && (r = palloc(p, (void **)&p->d_pts, (size_t)np * 16))) return r;
        CUDA_TRY(cudaMemcpy(p->d_pts, pts, (size_t)np * 16, cudaMemcpyHostToDevice));
    }
    if (!p->d_pts) { set_error("gridpoints not given"); return SS_BAD_ARG; }
    const int64_t nblob = offsets[nfields];
    if (nblob > p->blobs_cap) {
        if ((r = palloc(p, (void **)&p->d_blobs, (size_t)nblob * 32))) return r;
        p->blobs_cap = nblob;
    }
    if (nblob) CUDA_TRY(cudaMemcpy(p->d_blobs, blobs, (size_t)nblob * 32, cudaMemcpyHostToDevice));
    const int mcut = max_wavenumber < 0 ? p->K : std::min(max_wavenumber, p->K);
    const int per_field = (int)g->d.nvars * (1 + 2 * mcut);
    if ((r = mlp_dataset_reserve(mlp, mlp->ds_rows + (int64_t)nfields * per_field))) return r;
    SolveArgs A = solve_args(p, 1, 1, 1.0);
    A.masked = 0;
    A.mcut = mcut;
    const unsigned nb = warp_blocks(p->nsys);
    for (int f = 0; f < nfields; f++) {
        const int cnt = offsets[f + 1] - offsets[f];
        blob_field_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>((double *)g->phys, np, (int)g->d.nvars, p->d_pts,
                                                                         p->d_blobs + 4 * (size_t)offsets[f], cnt);
        CUDA_TRY(cudaGetLastError());
        if ((r = grid_forward(g, st))) return r;
        rhs_kernel<<<nb, 128, 0, st>>>(A);
        direct_kernel<<<nb, 128, 0, st>>>(A);
        training_rows_kernel<<<nb, 128, 0, st>>>(A, mlp->ds_rows, mlp->ds_X, mlp->ds_T, mlp->ds_n);
        CUDA_TRY(cudaGetLastError());
        mlp->ds_rows += per_field;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return SS_OK;
}

// Training pairs on random right-hand sides: `nsets` sets of one white-noise
// vector per radial system (smoothed `smooth` times by (1, 2, 1)/4), each
// solved directly; they widen the inputs beyond forcing-shaped vectors toward
// the Arnoldi vectors the flexible solve hands the network.
extern "C" int32_t ss_problem_collect_random(ss_problem *p, ss_mlp *mlp, int32_t nsets, uint64_t seed, int32_t smooth,
                                             int32_t max_wavenumber) {
    if (!p || !mlp || nsets < 0 || smooth < 0) { set_error("bad argument"); return SS_BAD_ARG; }
    int32_t r;
    if ((r = check_training_args(p, mlp))) return r;
    ss_grid *g = p->g;
    cudaSetDevice(g->device);
    cudaStream_t st = g->stream;
    const int mcut = max_wavenumber < 0 ? p->K : std::min(max_wavenumber, p->K);
    const int per_set = (int)g->d.nvars * (1 + 2 * mcut);
    if ((r = mlp_dataset_reserve(mlp, mlp->ds_rows + (int64_t)nsets * per_set))) return r;
    SolveArgs A = solve_args(p, 1, 1, 1.0);
    A.masked = 0;
    A.mcut = mcut;
    const unsigned nb = warp_blocks(p->nsys);
    for (int s = 0; s < nsets; s++) {
        rhs_random_kernel<<<nb, 128, 0, st>>>(A, seed * 0x100000001B3ull + (uint64_t)s, smooth);
        direct_kernel<<<nb, 128, 0, st>>>(A);
        training_rows_kernel<<<nb, 128, 0, st>>>(A, mlp->ds_rows, mlp->ds_X, mlp->ds_T, mlp->ds_n);
        CUDA_TRY(cudaGetLastError());
        mlp->ds_rows += per_set;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return SS_OK;
}
