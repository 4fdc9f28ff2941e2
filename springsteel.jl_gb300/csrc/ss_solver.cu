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

}  // namespace ss

struct ss_problem {
    ss_grid *g = nullptr;
    int K = 0, nsys = 0, nmax = 0, kl = 0, ku = 0, wG = 0, wU = 0;
    int n[2] = {0, 0};
    GammaDev gam[2];
    double *d_G = nullptr, *d_Lm = nullptr, *d_U = nullptr, *d_dinv = nullptr;
    int *d_piv = nullptr;
    GammaDev *d_gam = nullptr;
    double *d_rhs = nullptr, *d_x = nullptr, *d_res = nullptr, *d_cnorm = nullptr;
    int *d_iters = nullptr, *d_state = nullptr;
    // flexible GMRES workspace
    int fg_restart = 0;
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
    const double *G, *Lm, *U, *dinv;
    const int *piv;
    double *rhs, *x, *res, *cnorm;
    int *iters, *state;  // state: 0 active, 1 converged (or solved directly), 2 stopped inside a cycle
    int64_t nspec;
    int nslots, nvars, nmax, kl, ku, wG, wU, b, restart, max_iter, warm, masked;
    double tol;
};

__device__ __forceinline__ const GammaDev &gam_of(const SolveArgs &A, int m) { return A.gam[m == 0 ? 0 : 1]; }

// c = Γ_m b (src/CubicBSpline.jl:427-458), zero-padded to nmax; ‖c‖ per system
__global__ void rhs_kernel(SolveArgs A) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= A.nslots * A.nvars) return;
    const int v = sys / A.nslots, q = sys % A.nslots, m = slot_wavenumber(q);
    const GammaDev &g = gam_of(A, m);
    const double *b = A.spec + (size_t)v * A.nspec + (size_t)q * A.b;
    double *r = A.rhs + (size_t)sys * A.nmax;
    const double b0 = b[0], b1 = b[1], bM1 = b[g.Md - 1], bM2 = b[g.Md - 2];
    double nrm = 0.0;
    for (int i = 0; i < g.Min; i++) r[i] = b[i + g.rankL];
    if (g.lk == BC_A1) { r[0] += g.aL * b0; r[1] += g.bL * b0; }
    else if (g.lk == BC_A2) r[0] += g.aL * b0 + g.bL * b1;
    if (g.rk == BC_A1) { r[g.Min - 1] += g.aR * bM1; r[g.Min - 2] += g.bR * bM1; }
    else if (g.rk == BC_A2) r[g.Min - 1] += g.aR * bM1 + g.bR * bM2;
    for (int i = 0; i < g.Min; i++) nrm += r[i] * r[i];
    for (int i = g.Min; i < A.nmax; i++) r[i] = 0.0;
    A.cnorm[sys] = sqrt(nrm);
}

// a = Γ_mᵀ x into the spectral array (src/CubicBSpline.jl:461-500)
__global__ void unfold_kernel(SolveArgs A) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= A.nslots * A.nvars) return;
    const int v = sys / A.nslots, q = sys % A.nslots, m = slot_wavenumber(q);
    const GammaDev &g = gam_of(A, m);
    const double *x = A.x + (size_t)sys * A.nmax;
    double *a = A.spec_out + (size_t)v * A.nspec + (size_t)q * A.b;
    const int Md = g.Md, n = g.Min, rL = g.rankL;
    for (int j = 0; j < rL; j++) a[j] = 0.0;
    for (int j = Md - g.rankR; j < Md; j++) a[j] = 0.0;
    for (int i = 0; i < n; i++) a[i + rL] = x[i];
    if (g.lk == BC_A1) a[0] = g.aL * x[0] + g.bL * x[1];
    else if (g.lk == BC_A2) { a[0] = g.aL * x[0]; a[1] = g.bL * x[0]; }
    if (g.rk == BC_A1) a[Md - 1] = g.aR * x[n - 1] + g.bR * x[n - 2];
    else if (g.rk == BC_A2) { a[Md - 2] = g.bR * x[n - 1]; a[Md - 1] = g.aR * x[n - 1]; }
}

// direct solve: banded LU with partial pivoting (dgbtrs order), one thread per system
__global__ void direct_kernel(SolveArgs A) {
    const int sys = blockIdx.x * blockDim.x + threadIdx.x;
    if (sys >= A.nslots * A.nvars) return;
    if (A.masked && A.state[sys] == 1) return;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min;
    const double *Lm = A.Lm + (size_t)m * A.nmax * A.kl;
    const double *U = A.U + (size_t)m * A.nmax * A.wU;
    const int *piv = A.piv + (size_t)m * A.nmax;
    double *x = A.x + (size_t)sys * A.nmax;
    const double *r = A.rhs + (size_t)sys * A.nmax;
    for (int i = 0; i < n; i++) x[i] = r[i];
    for (int k = 0; k < n; k++) {
        const int p = piv[k];
        if (p != k) { double t = x[k]; x[k] = x[p]; x[p] = t; }
        const double xk = x[k];
        for (int t = 0; t < A.kl && k + 1 + t < n; t++) x[k + 1 + t] -= Lm[(size_t)k * A.kl + t] * xk;
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = x[i];
        for (int t = 1; t < A.wU && i + t < n; t++) s -= U[(size_t)i * A.wU + t] * x[i + t];
        x[i] = s / U[(size_t)i * A.wU];
    }
    A.state[sys] = 1;
}

// block-wide sum (blockDim a multiple of 32, ≤ 1024)
__device__ double block_sum(double v, double *red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
    return s;
}

// w = G_m z (radial_op_matvec; band rows: G[i][i + t − kl] at i·wG + t)
__device__ __forceinline__ void band_matvec(const double *G, int wG, int kl, int n, const double *z, double *w) {
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double acc = 0.0;
        for (int t = 0; t < wG; t++) {
            const int j = i + t - kl;
            if (j >= 0 && j < n) acc += G[(size_t)i * wG + t] * z[j];
        }
        w[i] = acc;
    }
}

// Givens update of column j of H and of g (thread 0)
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

// restarted GMRES with right Jacobi preconditioning (the reference's :diag,
// src/solver_problem.jl:172-179): one CTA per system, Krylov basis in shared memory
__global__ void gmres_kernel(SolveArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[32];
    const int sys = blockIdx.x;
    if (A.masked && A.state[sys] == 1) return;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min, R = A.restart;
    const double *G = A.G + (size_t)m * A.nmax * A.wG;
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
        band_matvec(G, A.wG, A.kl, n, x, w);
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
            band_matvec(G, A.wG, A.kl, n, z, w);
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
            if (rel <= A.tol) { j++; it++; break; }
        }
        if (threadIdx.x == 0)  // y = H⁻¹ g
            for (int k = j - 1; k >= 0; k--) {
                double s = gv[k];
                for (int l = k + 1; l < j; l++) s -= H[(size_t)k * R + l] * yv[l];
                yv[k] = s / H[(size_t)k * R + k];
            }
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {  // x += D⁻¹ V y
            double acc = 0.0;
            for (int k = 0; k < j; k++) acc += V[(size_t)k * n + i] * yv[k];
            x[i] += dv[i] * acc;
        }
        __syncthreads();
        if (rel <= A.tol) break;
    }
    band_matvec(G, A.wG, A.kl, n, x, w);  // true residual
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

// true relative residual ‖c − G x‖ / ‖c‖ (one CTA per system)
__global__ void residual_kernel(SolveArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[32];
    const int sys = blockIdx.x;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min;
    double *w = reinterpret_cast<double *>(smem_raw);
    band_matvec(A.G + (size_t)m * A.nmax * A.wG, A.wG, A.kl, n, A.x + (size_t)sys * A.nmax, w);
    __syncthreads();
    const double *c = A.rhs + (size_t)sys * A.nmax;
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { const double d = c[i] - w[i]; part += d * d; }
    const double rr = sqrt(block_sum(part, red)) / (A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0);
    if (threadIdx.x == 0) A.res[sys] = rr;
}

// ---------------------------------------------------------------- flexible GMRES
// All systems advance in lockstep so the MLP runs as one batched tensor-core
// pass per Arnoldi step.  MLP input row of a system: v (first n entries),
// zeros, then the features m/K and log(1+m)/log(1+K) in the last two columns.
struct FgArgs {
    SolveArgs S;
    double *V, *Z, *H, *gv, *cs, *sn;
    int *cyc;                // Arnoldi steps taken in the current cycle
    __nv_bfloat16 *mlp_in;   // [mpad][256]
    const float *mlp_out;    // [mpad][256]
    int j, K, mcut;
};

__device__ __forceinline__ void write_mlp_row(__nv_bfloat16 *row, const double *v, double scale, int n, int m, int K) {
    for (int i = threadIdx.x; i < kMlpWidth; i += blockDim.x) {
        float val = 0.f;
        if (i < n) val = (float)(v[i] * scale);
        else if (i == kMlpWidth - 2) val = (float)m / (float)(K > 0 ? K : 1);
        else if (i == kMlpWidth - 1) val = (float)(log1p((double)m) / log1p((double)(K > 0 ? K : 1)));
        row[i] = __float2bfloat16(val);
    }
}

// start of a cycle: r = c − G x; converged systems leave; else v0 = r / β
__global__ void fg_begin_kernel(FgArgs F) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[32];
    const SolveArgs &A = F.S;
    const int sys = blockIdx.x;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min, R = A.restart;
    __nv_bfloat16 *row = F.mlp_in + (size_t)sys * kMlpWidth;
    if (A.state[sys] == 1) { write_mlp_row(row, nullptr, 0.0, 0, m, F.K); return; }
    double *w = reinterpret_cast<double *>(smem_raw);
    const double *c = A.rhs + (size_t)sys * A.nmax;
    double *x = A.x + (size_t)sys * A.nmax;
    double *V = F.V + (size_t)sys * (R + 1) * A.nmax;
    band_matvec(A.G + (size_t)m * A.nmax * A.wG, A.wG, A.kl, n, x, w);
    __syncthreads();
    double part = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) { w[i] = c[i] - w[i]; part += w[i] * w[i]; }
    const double beta = sqrt(block_sum(part, red));
    const double cn = A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0;
    if (beta / cn <= A.tol || beta == 0.0) {
        if (threadIdx.x == 0) { A.state[sys] = 1; A.res[sys] = beta / cn; }
        write_mlp_row(row, nullptr, 0.0, 0, m, F.K);
        return;
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) V[i] = w[i] / beta;
    if (threadIdx.x == 0) {
        double *gv = F.gv + (size_t)sys * (R + 1);
        gv[0] = beta;
        for (int i = 1; i <= R; i++) gv[i] = 0.0;
        A.state[sys] = 0;
        F.cyc[sys] = 0;
    }
    write_mlp_row(row, w, 1.0 / beta, n, m, F.K);
}

// Arnoldi step j: z_j = D⁻¹(v_j + N(v_j)), w = G z_j, orthogonalise, Givens, next MLP input
__global__ void fg_step_kernel(FgArgs F) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ double red[32];
    const SolveArgs &A = F.S;
    const int sys = blockIdx.x;
    if (A.state[sys] != 0) return;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min, R = A.restart, j = F.j;
    const double *dv = A.dinv + (size_t)m * A.nmax;
    double *V = F.V + (size_t)sys * (R + 1) * A.nmax;
    double *Z = F.Z + (size_t)sys * R * A.nmax;
    double *H = F.H + (size_t)sys * (R + 1) * R;
    double *gv = F.gv + (size_t)sys * (R + 1), *cs = F.cs + (size_t)sys * R, *sn = F.sn + (size_t)sys * R;
    double *w = reinterpret_cast<double *>(smem_raw);
    double *z = Z + (size_t)j * A.nmax;
    const double *vj = V + (size_t)j * A.nmax;
    const float *o = F.mlp_out + (size_t)sys * kMlpWidth;
    const bool learned = m <= F.mcut;
    for (int i = threadIdx.x; i < n; i += blockDim.x) z[i] = dv[i] * (vj[i] + (learned ? (double)o[i] : 0.0));
    __syncthreads();
    band_matvec(A.G + (size_t)m * A.nmax * A.wG, A.wG, A.kl, n, z, w);
    __syncthreads();
    for (int k = 0; k <= j; k++) {
        double pk = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) pk += w[i] * V[(size_t)k * A.nmax + i];
        const double hk = block_sum(pk, red);
        for (int i = threadIdx.x; i < n; i += blockDim.x) w[i] -= hk * V[(size_t)k * A.nmax + i];
        if (threadIdx.x == 0) H[(size_t)k * R + j] = hk;
        __syncthreads();
    }
    double pn = 0.0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) pn += w[i] * w[i];
    const double hn = sqrt(block_sum(pn, red));
    double *vn = V + (size_t)(j + 1) * A.nmax;
    for (int i = threadIdx.x; i < n; i += blockDim.x) vn[i] = hn > 0.0 ? w[i] / hn : 0.0;
    if (threadIdx.x == 0) {
        H[(size_t)(j + 1) * R + j] = hn;
        givens_column(H, R, j, cs, sn, gv);
        A.iters[sys] += 1;
        F.cyc[sys] = j + 1;
    }
    __syncthreads();
    const double cn = A.cnorm[sys] > 0.0 ? A.cnorm[sys] : 1.0;
    if (fabs(gv[j + 1]) / cn <= A.tol || hn == 0.0) {
        if (threadIdx.x == 0) A.state[sys] = 2;  // converged estimate: stop this cycle
        return;
    }
    write_mlp_row(F.mlp_in + (size_t)sys * kMlpWidth, vn, 1.0, n, m, F.K);
}

// end of a cycle: x += Z y over the steps this system took
__global__ void fg_end_kernel(FgArgs F) {
    const SolveArgs &A = F.S;
    const int sys = blockIdx.x;
    if (A.state[sys] == 1) return;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    const int n = gam_of(A, m).Min, R = A.restart, steps = F.cyc[sys];
    const double *Z = F.Z + (size_t)sys * R * A.nmax;
    const double *H = F.H + (size_t)sys * (R + 1) * R;
    const double *gv = F.gv + (size_t)sys * (R + 1);
    __shared__ double yv[128];
    if (threadIdx.x == 0)
        for (int k = steps - 1; k >= 0; k--) {
            double s = gv[k];
            for (int l = k + 1; l < steps; l++) s -= H[(size_t)k * R + l] * yv[l];
            yv[k] = s / H[(size_t)k * R + k];
        }
    __syncthreads();
    double *x = A.x + (size_t)sys * A.nmax;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double acc = 0.0;
        for (int k = 0; k < steps; k++) acc += Z[(size_t)k * A.nmax + i] * yv[k];
        x[i] += acc;
    }
    if (threadIdx.x == 0) A.state[sys] = 0;
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

// training rows from the direct solution: input v = c/‖c‖, target D x/‖c‖ − v
__global__ void training_rows_kernel(SolveArgs A, int K, int mcut, int64_t row0, __nv_bfloat16 *X,
                                     __nv_bfloat16 *T, int32_t *nrow) {
    const int sys = blockIdx.x;
    const int q = sys % A.nslots, m = slot_wavenumber(q);
    if (m > mcut) return;
    // rows are packed per variable: the slots of wavenumbers ≤ mcut in slot order
    const int per_var = 1 + 2 * min(mcut, K);
    const int64_t row = row0 + (int64_t)(sys / A.nslots) * per_var + q;
    const int n = gam_of(A, m).Min;
    const double *c = A.rhs + (size_t)sys * A.nmax, *x = A.x + (size_t)sys * A.nmax;
    const double *dv = A.dinv + (size_t)m * A.nmax;
    const double cn = A.cnorm[sys];
    const double s = cn > 0.0 ? 1.0 / cn : 0.0;
    write_mlp_row(X + row * kMlpWidth, c, s, n, m, K);
    for (int i = threadIdx.x; i < kMlpWidth; i += blockDim.x) {
        float t = 0.f;
        if (i < n) t = (float)((x[i] / dv[i] - c[i]) * s);
        T[row * kMlpWidth + i] = __float2bfloat16(t);
    }
    if (threadIdx.x == 0) nrow[row] = n;
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
    ss_problem *p = new ss_problem();
    p->g = g;
    const ss_grid_params &gp = g->p;
    const int iDim = (int)g->d.iDim;
    std::vector<double> kk(k2, k2 + iDim);
    // templates: m = 0 (u'(0) = 0, u(R) = 0) and m ≥ 1 (u(0) = 0, u(R) = 0)
    ss_spline_bc r1t0{SS_SBC_RANK1, 0, -4.0, -1.0}, r1t1{SS_SBC_RANK1, 0, 0.0, 1.0};
    SplineHost tpl[2];
    int32_t st = build_spline(gp.iMin, gp.iMax, gp.num_cells, gp.mubar, gp.quadrature, g->l_q[0], r1t1, r1t0, tpl[0]);
    if (!st) st = build_spline(gp.iMin, gp.iMax, gp.num_cells, gp.mubar, gp.quadrature, g->l_q[0], r1t0, r1t0, tpl[1]);
    if (st) { delete p; return st; }
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
    p->kl = std::max(kl, 1); p->ku = ku; p->wG = p->kl + ku + 1; p->wU = p->kl + ku + 1;
    kl = p->kl;
    const int nm = p->nmax, Kp = p->K + 1;
    std::vector<double> hG((size_t)Kp * nm * p->wG, 0.0), hL((size_t)Kp * nm * kl, 0.0),
        hU((size_t)Kp * nm * p->wU, 0.0), hD((size_t)Kp * nm, 1.0);
    std::vector<int> hP((size_t)Kp * nm, 0);
    for (int m = 0; m <= p->K; m++) {
        const int n = p->n[m == 0 ? 0 : 1];
        std::vector<double> &A = Gs[m];
        for (int i = 0; i < n; i++) {
            for (int t = 0; t < p->wG; t++) {
                const int j = i + t - kl;
                if (j >= 0 && j < n) hG[((size_t)m * nm + i) * p->wG + t] = A[(size_t)i * n + j];
            }
            const double d = A[(size_t)i * n + i];
            hD[(size_t)m * nm + i] = std::fabs(d) > 0.0 ? 1.0 / d : 1.0;
        }
        // banded LU with partial pivoting (dgbtf2 order); U gains kl superdiagonals
        for (int k = 0; k < n; k++) {
            int piv = k;
            double mx = std::fabs(A[(size_t)k * n + k]);
            for (int i = k + 1; i <= std::min(n - 1, k + kl); i++)
                if (std::fabs(A[(size_t)i * n + k]) > mx) { mx = std::fabs(A[(size_t)i * n + k]); piv = i; }
            if (mx == 0.0) { delete p; set_error("singular radial operator at wavenumber %d", m); return SS_NOT_SPD; }
            hP[(size_t)m * nm + k] = piv;
            const int jend = std::min(n - 1, k + kl + ku);
            if (piv != k)
                for (int j = k; j <= jend; j++) std::swap(A[(size_t)k * n + j], A[(size_t)piv * n + j]);
            for (int i = k + 1; i <= std::min(n - 1, k + kl); i++) {
                const double l = A[(size_t)i * n + k] / A[(size_t)k * n + k];
                hL[((size_t)m * nm + k) * kl + (i - k - 1)] = l;
                for (int j = k + 1; j <= jend; j++) A[(size_t)i * n + j] -= l * A[(size_t)k * n + j];
            }
            for (int t = 0; t < p->wU && k + t < n; t++) hU[((size_t)m * nm + k) * p->wU + t] = A[(size_t)k * n + k + t];
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
    if (bandwidth) *bandwidth = p->wG;
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
    if (kl) *kl = p->kl;
    if (band)
        CUDA_TRY(cudaMemcpy(band, p->d_G + (size_t)m * p->nmax * p->wG, (size_t)p->nmax * p->wG * 8,
                            cudaMemcpyDeviceToHost));
    return SS_OK;
}

static SolveArgs solve_args(ss_problem *p, int restart, int max_iter, double tol) {
    ss_grid *g = p->g;
    SolveArgs A{};
    A.spec = (const double *)g->spec; A.spec_out = (double *)g->spec; A.gam = p->d_gam;
    A.G = p->d_G; A.Lm = p->d_Lm; A.U = p->d_U; A.dinv = p->d_dinv; A.piv = p->d_piv;
    A.rhs = p->d_rhs; A.x = p->d_x; A.res = p->d_res; A.cnorm = p->d_cnorm; A.iters = p->d_iters; A.state = p->d_state;
    A.nspec = g->d.n_spectral; A.nslots = 1 + 2 * p->K; A.nvars = (int)g->d.nvars; A.nmax = p->nmax;
    A.kl = p->kl; A.ku = p->ku; A.wG = p->wG; A.wU = p->wU; A.b = (int)g->d.b_iDim;
    A.restart = restart; A.max_iter = max_iter; A.tol = tol;
    return A;
}

static int32_t ensure_fg(ss_problem *p, int R) {
    if (p->fg_restart >= R && p->d_V) return SS_OK;
    const size_t ns = p->nsys, nm = p->nmax;
    int32_t st;
    if ((st = palloc(p, (void **)&p->d_V, ns * (R + 1) * nm * 8)) || (st = palloc(p, (void **)&p->d_Z, ns * R * nm * 8)) ||
        (st = palloc(p, (void **)&p->d_H, ns * (R + 1) * R * 8)) || (st = palloc(p, (void **)&p->d_gv, ns * (R + 1) * 8)) ||
        (st = palloc(p, (void **)&p->d_cs, ns * R * 8)) || (st = palloc(p, (void **)&p->d_sn, ns * R * 8)) ||
        (st = palloc(p, (void **)&p->d_cyc, ns * 4)))
        return st;
    p->mpad = (int)((ns + kMlpTileM - 1) / kMlpTileM * kMlpTileM);
    if (!p->d_mlp_in &&
        ((st = palloc(p, (void **)&p->d_mlp_in, (size_t)p->mpad * kMlpWidth * 2)) ||
         (st = palloc(p, (void **)&p->d_mlp_out, (size_t)p->mpad * kMlpWidth * 4))))
        return st;
    p->fg_restart = R;
    return SS_OK;
}

static size_t gmres_smem(int R, int n) {
    return ((size_t)(R + 1) * n + 2 * (size_t)n + (size_t)(R + 1) * R + 4 * (size_t)R + 4) * 8;
}

static int32_t run_gmres(ss_problem *p, SolveArgs A, cudaStream_t st) {
    const size_t smem = gmres_smem(A.restart, p->nmax);
    if (smem > 200 * 1024) { set_error("restart too long for shared memory"); return SS_BAD_ARG; }
    if (smem > 48 * 1024) CUDA_TRY(cudaFuncSetAttribute(gmres_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    gmres_kernel<<<p->nsys, 128, smem, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

// the chosen backend on the right-hand sides already in d_rhs (no transforms)
static int32_t solve_systems(ss_problem *p, int method, SolveArgs A, cudaStream_t st, int *fallback) {
    const int ns = p->nsys;
    int32_t r;
    *fallback = 0;
    CUDA_TRY(cudaMemsetAsync(p->d_iters, 0, (size_t)ns * 4, st));
    CUDA_TRY(cudaMemsetAsync(p->d_state, 0, (size_t)ns * 4, st));
    const size_t wsm = (size_t)p->nmax * 8;
    if (method == SS_SOLVER_DIRECT) {
        A.masked = 0;
        direct_kernel<<<(ns + 63) / 64, 64, 0, st>>>(A);
        CUDA_TRY(cudaGetLastError());
        residual_kernel<<<ns, 128, wsm, st>>>(A);
        CUDA_TRY(cudaGetLastError());
        return SS_OK;
    }
    if (method == SS_SOLVER_GMRES_JACOBI) {
        A.warm = 0; A.masked = 0;
        return run_gmres(p, A, st);
    }
    // flexible GMRES with the learned preconditioner, cycles in lockstep
    if ((r = ensure_fg(p, A.restart))) return r;
    if ((r = mlp_reserve(p->mlp, p->mpad))) return r;
    CUDA_TRY(cudaMemsetAsync(p->d_x, 0, (size_t)ns * p->nmax * 8, st));
    FgArgs F{};
    F.S = A; F.V = p->d_V; F.Z = p->d_Z; F.H = p->d_H; F.gv = p->d_gv; F.cs = p->d_cs; F.sn = p->d_sn;
    F.cyc = p->d_cyc; F.mlp_in = p->d_mlp_in; F.mlp_out = p->d_mlp_out; F.K = p->K; F.mcut = p->mcut;
    fg_begin_kernel<<<ns, 128, wsm, st>>>(F);
    CUDA_TRY(cudaGetLastError());
    int done_iters = 0;
    std::vector<int> hstate(ns);
    while (done_iters < A.max_iter) {
        const int steps = std::min(A.restart, A.max_iter - done_iters);
        for (int j = 0; j < steps; j++) {
            F.j = j;
            if ((r = mlp_forward(p->mlp, p->d_mlp_in, p->d_mlp_out, p->mpad, st))) return r;
            fg_step_kernel<<<ns, 128, wsm, st>>>(F);
            CUDA_TRY(cudaGetLastError());
        }
        fg_end_kernel<<<ns, 128, 0, st>>>(F);
        CUDA_TRY(cudaGetLastError());
        done_iters += steps;
        fg_begin_kernel<<<ns, 128, wsm, st>>>(F);  // true residual: converged systems leave, others restart
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
        direct_kernel<<<(ns + 63) / 64, 64, 0, st>>>(A);
        CUDA_TRY(cudaGetLastError());
    }
    residual_kernel<<<ns, 128, wsm, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    return SS_OK;
}

extern "C" int32_t ss_solve(ss_problem *p, int32_t method, double tol, int32_t max_iter, int32_t restart,
                            ss_solve_stats *stats, void *stream) {
    if (!p) { set_error("null problem"); return SS_BAD_ARG; }
    if (method < SS_SOLVER_DIRECT || method > SS_SOLVER_FGMRES_MLP) { set_error("unknown solver"); return SS_BAD_ARG; }
    if (!(tol > 0.0)) { set_error("tolerance must be positive"); return SS_BAD_ARG; }
    if (restart < 1) restart = 30;
    if (restart > 100) { set_error("restart must be <= 100"); return SS_BAD_ARG; }
    if (max_iter < 1) max_iter = 2000;
    if (method == SS_SOLVER_FGMRES_MLP && !p->mlp) { set_error("no MLP preconditioner attached"); return SS_BAD_ARG; }
    ss_grid *g = p->g;
    cudaSetDevice(g->device);
    cudaStream_t st = stream ? (cudaStream_t)stream : g->stream;
    int32_t r = grid_forward(g, st);  // f (physical slot 1) → spectral B-vectors
    if (r) return r;
    SolveArgs A = solve_args(p, restart, max_iter, tol);
    CUDA_TRY(cudaEventRecord(p->e0, st));
    rhs_kernel<<<(p->nsys + 127) / 128, 128, 0, st>>>(A);
    CUDA_TRY(cudaGetLastError());
    int fallback = 0;
    if ((r = solve_systems(p, method, A, st, &fallback))) return r;
    unfold_kernel<<<(p->nsys + 127) / 128, 128, 0, st>>>(A);
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

// Training pairs from the direct solve: for each field (blobs[offsets[f] ..
// offsets[f+1]) as (xc, yc, w, A) quadruples) the field is evaluated on the
// device at the gridpoints `pts` (n_physical × 2: r then λ), transformed,
// solved directly, and each radial system of wavenumber ≤ max_wavenumber is
// appended to the network's resident training set.
extern "C" int32_t ss_problem_collect_training(ss_problem *p, ss_mlp *mlp, const double *pts, const double *blobs,
                                               const int32_t *offsets, int32_t nfields, int32_t max_wavenumber) {
    if (!p || !mlp || !blobs || !offsets || nfields < 0) { set_error("bad argument"); return SS_BAD_ARG; }
    if (p->nmax > kMlpWidth - 2) { set_error("radial systems exceed the network width"); return SS_BAD_SHAPE; }
    if (mlp->device != p->g->device) { set_error("network and grid on different devices"); return SS_BAD_ARG; }
    for (int f = 0; f < nfields; f++)
        if (offsets[f + 1] < offsets[f] || offsets[f] < 0) { set_error("blob offsets decrease"); return SS_BAD_ARG; }
    ss_grid *g = p->g;
    cudaSetDevice(g->device);
    cudaStream_t st = g->stream;
    const int64_t np = g->d.n_physical;
    int32_t r;
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
    for (int f = 0; f < nfields; f++) {
        const int nb = offsets[f + 1] - offsets[f];
        blob_field_kernel<<<(unsigned)((np + 255) / 256), 256, 0, st>>>((double *)g->phys, np, (int)g->d.nvars, p->d_pts,
                                                                         p->d_blobs + 4 * (size_t)offsets[f], nb);
        CUDA_TRY(cudaGetLastError());
        if ((r = grid_forward(g, st))) return r;
        rhs_kernel<<<(p->nsys + 127) / 128, 128, 0, st>>>(A);
        direct_kernel<<<(p->nsys + 63) / 64, 64, 0, st>>>(A);
        training_rows_kernel<<<p->nsys, 128, 0, st>>>(A, p->K, mcut, mlp->ds_rows, mlp->ds_X, mlp->ds_T, mlp->ds_n);
        CUDA_TRY(cudaGetLastError());
        mlp->ds_rows += per_field;
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return SS_OK;
}
