// ss_setup.cpp — one-time FP64 host setup of a grid's device tables.
//
// This is the createGrid side of the library (src/factory.jl:646-740): the
// spline template (quadrature, Γ fold, P+Q and its banded Cholesky factor,
// src/CubicBSpline.jl:172-200, 321-424, 733-783; src/banded_cholesky.jl:99-197),
// the SB/SI weights (the entries of the reference's _sb_matrix,
// src/CubicBSpline.jl:1000-1030, and of SItransform's 4-tap window,
// :1554-1567), the Chebyshev tables (src/Chebyshev.jl:329-378, 991-1177) and
// the FFT plans/twiddles.  Nothing here runs per transform.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "ss_internal.h"

namespace ss {

static const double kPi = 3.14159265358979323846264338327950288;

// -------------------------------------------------------------- B-spline
static int quad_rule(int mb, int quad, std::vector<double> &qp, std::vector<double> &qw) {
    qp.assign(mb, 0.0);
    qw.assign(mb, 0.0);
    if (mb < 1) { set_error("mubar must be >= 1, got %d", mb); return SS_BAD_ARG; }
    if (quad == SS_QUAD_GAUSS) {
        double nd[5] = {0}, w[5] = {0};
        switch (mb) {
        case 1: nd[0] = 0.0; w[0] = 2.0; break;
        case 2: nd[0] = -1.0 / std::sqrt(3.0); nd[1] = 1.0 / std::sqrt(3.0); w[0] = w[1] = 1.0; break;
        case 3:
            nd[0] = -std::sqrt(3.0 / 5.0); nd[1] = 0.0; nd[2] = std::sqrt(3.0 / 5.0);
            w[0] = 5.0 / 9.0; w[1] = 8.0 / 9.0; w[2] = 5.0 / 9.0;
            break;
        case 4: {
            double a = std::sqrt(3.0 / 7.0 + 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
            double b = std::sqrt(3.0 / 7.0 - 2.0 / 7.0 * std::sqrt(6.0 / 5.0));
            nd[0] = -a; nd[1] = -b; nd[2] = b; nd[3] = a;
            w[0] = w[3] = (18.0 - std::sqrt(30.0)) / 36.0;
            w[1] = w[2] = (18.0 + std::sqrt(30.0)) / 36.0;
            break;
        }
        case 5: {
            double a = std::sqrt(5.0 + 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
            double b = std::sqrt(5.0 - 2.0 * std::sqrt(10.0 / 7.0)) / 3.0;
            nd[0] = -a; nd[1] = -b; nd[2] = 0.0; nd[3] = b; nd[4] = a;
            w[0] = w[4] = (322.0 - 13.0 * std::sqrt(70.0)) / 900.0;
            w[1] = w[3] = (322.0 + 13.0 * std::sqrt(70.0)) / 900.0;
            w[2] = 128.0 / 225.0;
            break;
        }
        default: set_error("Gauss-Legendre quadrature supports mubar 1-5, got %d", mb); return SS_BAD_ARG;
        }
        for (int k = 0; k < mb; k++) { qp[k] = (nd[k] + 1.0) / 2.0; qw[k] = w[k] / 2.0; }
        return SS_OK;
    }
    if (quad == SS_QUAD_REGULAR) {
        for (int k = 1; k <= mb; k++) { qp[k - 1] = double(2 * k - 1) / double(2 * mb); qw[k - 1] = 1.0 / mb; }
        return SS_OK;
    }
    set_error("unknown quadrature %d", quad);
    return SS_BAD_ARG;
}

// φ_m^(d)(x), Ooyama (2002) cubic B-spline (same piecewise form as basis(),
// src/CubicBSpline.jl:585-628)
static double bspline(const SplineHost &s, int m, double x, int d) {
    double b = 0.0;
    double xm = s.xmin + (m * s.DX);
    double delta = (x - xm) * s.DXrecip;
    double z = std::fabs(delta);
    if (z < 2.0) {
        if (d == 0) {
            z = 2.0 - z; b = (z * z * z) * (1.0 / 6.0); z -= 1.0;
            if (z > 0) b -= (z * z * z) * (4.0 / 6.0);
        } else if (d == 1) {
            z = 2.0 - z; b = (z * z) * (1.0 / 6.0); z -= 1.0;
            if (z > 0) b -= (z * z) * (4.0 / 6.0);
            b *= ((delta > 0) ? -1.0 : 1.0) * 3.0 * s.DXrecip;
        } else if (d == 2) {
            z = 2.0 - z; b = z; z -= 1.0;
            if (z > 0) b -= z * 4;
            b *= s.DXrecip * s.DXrecip;
        } else {
            if (z > 1.0) b = 1.0;
            else if (z < 1.0) b = -3.0;
            b *= ((delta > 0) ? -1.0 : 1.0) * s.DXrecip * s.DXrecip * s.DXrecip;
        }
    }
    return b;
}

// Γ entry (1-based), the structured BC fold of src/CubicBSpline.jl:336-376
static double gamma_at(const SplineHost &g, int i, int j) {
    double val = (j == i + g.rankL) ? 1.0 : 0.0;
    if (g.lk == BC_A1) {
        if (j == 1) { if (i == 1) val += g.aL; if (i == 2) val += g.bL; }
    } else if (g.lk == BC_A2) {
        if (j == 1 && i == 1) val += g.aL;
        else if (j == 2 && i == 1) val += g.bL;
    }
    else if (g.lk == BC_PER && j == 1 && i == g.Min) val += 1.0;
    if (g.rk == BC_A1) {
        if (j == g.Mdim) { if (i == g.Min) val += g.aR; if (i == g.Min - 1) val += g.bR; }
    } else if (g.rk == BC_A2) {
        if (j == g.Mdim && i == g.Min) val += g.aR;
        else if (j == g.Mdim - 1 && i == g.Min) val += g.bR;
    } else if (g.rk == BC_PER) {  // wrap-around rows (src/CubicBSpline.jl:366-369)
        if (j == g.Mdim - 1 && i == 1) val += 1.0;
        if (j == g.Mdim && i == 2) val += 1.0;
    }
    return val;
}

static int side_bc(const ss_spline_bc &bc, int right, int &rank, int &kind, double &a, double &b, int &r3x) {
    switch (bc.kind) {
    case SS_SBC_R0: rank = 0; kind = BC_R0; a = b = 0.0; return SS_OK;
    case SS_SBC_RANK1: rank = 1; kind = BC_A1; a = bc.alpha; b = bc.beta; return SS_OK;
    case SS_SBC_RANK2: rank = 2; kind = BC_A2; a = bc.alpha; b = bc.beta; return SS_OK;
    case SS_SBC_R3: rank = 3; kind = BC_R3; a = b = 0.0; return SS_OK;
    case SS_SBC_R3X: rank = 3; kind = BC_R3; a = b = 0.0; r3x = 1; return SS_OK;
    case SS_SBC_PERIODIC:  // GammaBC: rankL 1 / rankR 2 (src/CubicBSpline.jl:395-397, 414-416)
        rank = right ? 2 : 1; kind = BC_PER; a = b = 0.0; return SS_OK;
    default: set_error("unrecognised spline BC kind %d", bc.kind); return SS_UNSUPPORTED_BC;
    }
}

static int32_t finish_weights(SplineHost &s);

// PERIODIC: the wrap-around rows of Γ couple the first and the last interior
// coefficients, so Γ(P+Q)Γᵀ is banded plus corner entries and the reference
// factors it densely (cholesky_dense_factor, src/banded_cholesky.jl:70, 250-260,
// chosen by calcPQfactor, src/CubicBSpline.jl:777-781).  The corners sit in the
// last three rows (and columns), so the dense LLᵀ factor is banded except for
// its last three rows; it is kept as the (4, n) band plus those rows (`tail`),
// and the corners of A beyond the band for the binary32 refinement residual.
static int32_t periodic_factor(SplineHost &s, const std::vector<double> &P, const std::vector<double> &Q) {
    const int n = s.Min, Md = s.Mdim;
    if (n < 4) { set_error("PERIODIC spline BC needs at least 4 interior coefficients"); return SS_BAD_SHAPE; }
    std::vector<std::vector<std::pair<int, double>>> rows(n + 1);  // Γ row i (1-based): (column, value)
    for (int i = 1; i <= n; i++)
        for (int a : {i + s.rankL, 1, 2, Md - 1, Md}) {
            bool seen = false;
            for (auto &e : rows[i]) seen |= e.first == a;
            const double ga = (a >= 1 && a <= Md && !seen) ? gamma_at(s, i, a) : 0.0;
            if (ga != 0.0) rows[i].push_back({a, ga});
        }
    std::vector<double> A(size_t(n) * n, 0.0);  // column-major, A[i + j n]
    for (int i = 1; i <= n; i++)
        for (int j = 1; j <= n; j++) {
            double acc = 0.0;
            for (auto &ea : rows[i])
                for (auto &eb : rows[j]) {
                    const int d = eb.first - ea.first;
                    if (d < -3 || d > 3) continue;
                    const size_t k = size_t(ea.first - 1) * 7 + (d + 3);
                    acc += ea.second * (P[k] + Q[k]) * eb.second;
                }
            A[size_t(i - 1) + size_t(j - 1) * n] = acc;
        }
    s.Aopen.assign(size_t(n) * 4, 0.0);
    s.acorner.assign(9, 0.0);
    const int r0 = n - 3;
    for (int j = 0; j < n; j++)
        for (int d = 0; d < 4 && j + d < n; d++) s.Aopen[size_t(j) * 4 + d] = A[size_t(j + d) + size_t(j) * n];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            if (r0 + r - c > 3) s.acorner[r * 3 + c] = A[size_t(r0 + r) + size_t(c) * n];
    // dense LLᵀ, lower triangle in place (potrf's factor)
    for (int j = 0; j < n; j++) {
        double d = A[size_t(j) + size_t(j) * n];
        for (int k = 0; k < j; k++) d -= A[size_t(j) + size_t(k) * n] * A[size_t(j) + size_t(k) * n];
        if (d <= 0.0) { set_error("P+Q not positive definite (PosDefException at %d)", j + 1); return SS_NOT_SPD; }
        const double ljj = std::sqrt(d);
        A[size_t(j) + size_t(j) * n] = ljj;
        for (int i = j + 1; i < n; i++) {
            double t = A[size_t(i) + size_t(j) * n];
            for (int k = 0; k < j; k++) t -= A[size_t(i) + size_t(k) * n] * A[size_t(j) + size_t(k) * n];
            A[size_t(i) + size_t(j) * n] = t / ljj;
        }
    }
    for (int i = 0; i < r0; i++)  // rows above the tail keep the band: no fill-in below j = i − 3
        for (int j = 0; j < i - 3; j++)
            if (A[size_t(i) + size_t(j) * n] != 0.0) { set_error("periodic factor fills outside its band"); return SS_BAD_ARG; }
    s.L4.assign(size_t(n) * 4, 0.0);
    for (int j = 0; j < n; j++)
        for (int d = 0; d < 4 && j + d < n; d++) s.L4[size_t(j) * 4 + d] = A[size_t(j + d) + size_t(j) * n];
    s.tail.assign(size_t(3) * n, 0.0);
    for (int r = 0; r < 3; r++)
        for (int j = 0; j <= r0 + r; j++) s.tail[size_t(r) * n + j] = A[size_t(r0 + r) + size_t(j) * n];
    return SS_OK;
}

int32_t build_spline(double xmin, double xmax, int nc, int mubar, int quad, double l_q,
                     const ss_spline_bc &bcl, const ss_spline_bc &bcr, SplineHost &s) {
    if (nc < 1) { set_error("num_cells must be >= 1"); return SS_BAD_SHAPE; }
    if (!(xmax > xmin)) { set_error("iMax must exceed iMin"); return SS_BAD_ARG; }
    s.xmin = xmin; s.xmax = xmax; s.nc = nc; s.mubar = mubar; s.l_q = l_q;
    s.DX = (xmax - xmin) / nc;
    s.DXrecip = 1.0 / s.DX;
    s.bDim = nc + 3;
    s.mishDim = nc * mubar;
    int st = quad_rule(mubar, quad, s.qp, s.qw);
    if (st) return st;
    s.r3x = 0;
    st = side_bc(bcl, 0, s.rankL, s.lk, s.aL, s.bL, s.r3x);
    if (st) return st;
    st = side_bc(bcr, 1, s.rankR, s.rk, s.aR, s.bR, s.r3x);
    if (st) return st;
    s.Mdim = s.bDim;
    s.Min = s.Mdim - s.rankL - s.rankR;
    if (s.Min < 2) { set_error("too few interior coefficients (%d) for the banded solve", s.Min); return SS_BAD_SHAPE; }
    s.mish.resize(s.mishDim);
    for (int mc = 0; mc < nc; mc++)
        for (int mu = 0; mu < mubar; mu++) s.mish[mu + mubar * mc] = xmin + mc * s.DX + s.qp[mu] * s.DX;

    // P and Q on the ±3 band (calcPQfactor, src/CubicBSpline.jl:733-783)
    const int Md = s.Mdim;
    const double eps_q = std::pow((l_q * s.DX) / (2 * kPi), 6);
    std::vector<double> P(Md * 7, 0.0), Q(Md * 7, 0.0);
    for (int mi1 = 1; mi1 <= Md; mi1++)
        for (int mi2 = std::max(1, mi1 - 3); mi2 <= std::min(Md, mi1 + 3); mi2++) {
            int m1 = mi1 - 2, m2 = mi2 - 2;
            for (int mc = 0; mc < nc; mc++) {
                if (mc < m1 - 2 || mc > m1 + 1 || mc < m2 - 2 || mc > m2 + 1) continue;
                for (int mu = 0; mu < mubar; mu++) {
                    double x = xmin + mc * s.DX + s.qp[mu] * s.DX;
                    double pm1 = bspline(s, m1, x, 0), qm1 = bspline(s, m1, x, 3);
                    double pm2 = bspline(s, m2, x, 0), qm2 = bspline(s, m2, x, 3);
                    P[(mi1 - 1) * 7 + (mi2 - mi1 + 3)] += s.DX * s.qw[mu] * pm1 * pm2;
                    Q[(mi1 - 1) * 7 + (mi2 - mi1 + 3)] += s.DX * s.qw[mu] * eps_q * qm1 * qm2;
                }
            }
        }
    s.PQb.assign(Md * 7, 0.0);
    for (int i = 0; i < Md * 7; i++) s.PQb[i] = P[i] + Q[i];

    const int n = s.Min;
    s.periodic = (s.lk == BC_PER || s.rk == BC_PER);
    if (s.periodic) {
        const int32_t st = periodic_factor(s, P, Q);
        return st ? st : finish_weights(s);
    }
    // open form Γ P Γᵀ + Γ Q Γᵀ on the band, then the banded LLᵀ factor
    std::vector<double> A(size_t(n) * 4, 0.0);  // A[j*4+d] = Aopen[j+d][j]
    for (int j = 1; j <= n; j++)
        for (int i = j; i <= std::min(n, j + 6); i++) {
            double aP = 0.0, aQ = 0.0;
            for (int a = std::max(1, i - 3); a <= std::min(Md, i + 3 + s.rankL); a++) {
                double ga = gamma_at(s, i, a);
                if (ga == 0.0) continue;
                for (int b = std::max(1, a - 3); b <= std::min(Md, a + 3); b++) {
                    double gb = gamma_at(s, j, b);
                    if (gb == 0.0) continue;
                    aP += ga * P[(a - 1) * 7 + (b - a + 3)] * gb;
                    aQ += ga * Q[(a - 1) * 7 + (b - a + 3)] * gb;
                }
            }
            double v = aP + aQ;
            if (i - j > 3) {
                if (v != 0.0) { set_error("open-form P+Q exceeds half-bandwidth 3"); return SS_BAD_ARG; }
            } else {
                A[size_t(j - 1) * 4 + (i - j)] = v;
            }
        }
    s.Aopen = A;
    // _band_factor3! (src/banded_cholesky.jl:166-197)
    for (int j = 0; j < n; j++) {
        double d = A[j * 4];
        for (int k = std::max(0, j - 3); k < j; k++) { double l = A[k * 4 + (j - k)]; d -= l * l; }
        if (d <= 0.0) { set_error("P+Q not positive definite (PosDefException at %d)", j + 1); return SS_NOT_SPD; }
        double ljj = std::sqrt(d);
        A[j * 4] = ljj;
        double inv = 1.0 / ljj;
        for (int i = j + 1; i <= std::min(n - 1, j + 3); i++) {
            double t = A[j * 4 + (i - j)];
            for (int k = std::max(0, i - 3); k < j; k++) t -= A[k * 4 + (i - k)] * A[k * 4 + (j - k)];
            A[j * 4 + (i - j)] = t * inv;
        }
    }
    s.L4 = A;
    return finish_weights(s);
}

// SB weights and SI weights of a spline (shared by the banded and periodic setups)
static int32_t finish_weights(SplineHost &s) {
    const int Md = s.Mdim, nc = s.nc, mubar = s.mubar;
    const double xmin = s.xmin;
    // SB weights: row mi (0-based), tap t = c*mubar + mu over cells mc = mi-3+c
    const int taps = 4 * mubar;
    s.sbw.assign(size_t(Md) * taps, 0.0);
    for (int mi = 0; mi < Md; mi++) {
        int m = mi - 1;
        for (int c = 0; c < 4; c++) {
            int mc = m - 2 + c;
            if (mc < 0 || mc > nc - 1) continue;
            for (int mu = 0; mu < mubar; mu++) {
                double x = xmin + mc * s.DX + s.qp[mu] * s.DX;
                s.sbw[size_t(mi) * taps + c * mubar + mu] = s.DX * s.qw[mu] * bspline(s, m, x, 0);
            }
        }
    }
    // SI weights at the mish points (SItransform(sp, a, points, u, d))
    s.siw.assign(size_t(3) * s.mishDim * 4, 0.0);
    s.si_m0.assign(s.mishDim, 0);
    for (int i = 0; i < s.mishDim; i++) {
        double x = s.mish[i];
        long xm = (long)std::ceil((x - xmin - (2.0 * s.DX)) * s.DXrecip);
        int m0 = int(xm) + 1;  // coefficient index of m = xm
        int base = std::min(std::max(m0, 0), Md - 4);
        s.si_m0[i] = base;
        for (int q = 0; q < 4; q++) {
            long m = xm + q;
            if (m < -1 || m > nc + 1) continue;
            int idx = int(m + 1) - base;
            if (idx < 0 || idx > 3) { set_error("SI window out of range"); return SS_BAD_ARG; }
            for (int d = 0; d < 3; d++) s.siw[(size_t(d) * s.mishDim + i) * 4 + idx] = bspline(s, int(m), x, d);
        }
    }
    return SS_OK;
}

// -------------------------------------------------------------- Chebyshev
static double cospi_frac(long num, long den) {  // cos(π num/den) with exact reduction
    long per = 2 * den;
    num %= per;
    if (num < 0) num += per;
    bool flip = num > den;  // cos(π(2d - n)/d) = cos(πn/d)
    long nn = flip ? per - num : num;
    return std::cos(kPi * (double)nn / (double)den);
}

int32_t build_cheb(int N, int bk, int bcb, int bct, double zmin, double zmax, ChebHost &c) {
    if (N < 2) { set_error("kDim must be >= 2"); return SS_BAD_SHAPE; }
    if (bk < 1 || bk > N) { set_error("b_kDim out of range"); return SS_BAD_SHAPE; }
    c.N = N; c.bk = bk;
    c.half = (N + 1) / 2;
    c.dscale = -0.5 * (zmax - zmin);
    c.mish.resize(N);
    {
        double scale = -0.5 * (zmax - zmin), offset = 0.5 * (zmin + zmax);
        for (int n = 1; n <= N; n++) c.mish[n - 1] = std::cos((n - 1) * kPi / (N - 1)) * scale + offset;
    }
    // forward: b[k] = filt_k * (1/(2(N-1))) * REDFT00(x)[k], folded over j ↔ N-1-j
    const double scale = 1.0 / (2 * (N - 1));
    c.fwd.assign(size_t(bk) * c.half, 0.0);
    for (int k = 0; k < bk; k++) {
        double filt = (bk < N) ? 1.0 : std::exp(-36.0 * std::pow(double(k + 1) / N, 36));
        for (int j = 0; j < c.half; j++) {
            int jj = N - 1 - j;
            double w = (j == 0) ? 1.0 : 2.0;  // endpoint weight 1, interior 2
            double cs = cospi_frac((long)j * k, N - 1);
            if (jj == j) w = 2.0;              // middle point of odd N: counted once
            c.fwd[size_t(k) * c.half + j] = filt * scale * w * cs;
        }
    }
    // inverse REDFT00 folded over outputs j ↔ N-1-j; split into even / odd k
    const int ne = (N + 1) / 2, no = N / 2;
    c.inv_e.assign(size_t(c.half) * ne, 0.0);
    c.inv_o.assign(size_t(c.half) * (no > 0 ? no : 1), 0.0);
    for (int j = 0; j < c.half; j++) {
        for (int k = 0; k < N; k++) {
            double w = (k == 0 || k == N - 1) ? 1.0 : 2.0;
            double v = w * cospi_frac((long)j * k, N - 1);
            if (k % 2 == 0) c.inv_e[size_t(j) * ne + k / 2] = v;
            else c.inv_o[size_t(j) * no + k / 2] = v;
        }
    }
    // Γ (calcGammaBC, src/Chebyshev.jl:991-1177) as Σ_p u_p v_pᵀ, rank ≤ 2
    std::vector<double> cv(N, 1.0);
    cv[0] = 2.0; cv[N - 1] = 2.0;
    auto sgn = [](long e) { return (e % 2 == 0) ? 1.0 : -1.0; };
    std::vector<std::vector<double>> U, V;
    // R1T0 bottom vector gl (rank 1, v = ones)
    auto add_gl = [&]() {
        std::vector<double> u(N), v(N, 1.0);
        for (int i = 0; i < N; i++) u[i] = ((i == 0 || i == N - 1) ? 1.0 : 2.0) * (-0.5 / (N - 1));
        U.push_back(u); V.push_back(v);
    };
    // R1T0 top: D[i,j] = -(-1)^i (-1)^j/(N-1), rows 0 and N-1 halved
    auto add_top_dirichlet = [&]() {
        std::vector<double> u(N), v(N);
        for (int i = 0; i < N; i++) u[i] = -1.0 * sgn(i) / (N - 1) * ((i == 0 || i == N - 1) ? 0.5 : 1.0);
        for (int j = 0; j < N; j++) v[j] = sgn(j);
        U.push_back(u); V.push_back(v);
    };
    // R1T1 bottom: B[i,j] = n²/(sf c_j (N-1))
    auto add_bot_neumann = [&]() {
        double sf = 0.0;
        for (int i = 0; i < N; i++) sf += -(double(i) * i) / (cv[i] * (N - 1));
        std::vector<double> u(N), v(N);
        for (int i = 0; i < N; i++) u[i] = double(i) * i / sf;
        for (int j = 0; j < N; j++) v[j] = 1.0 / (cv[j] * (N - 1));
        U.push_back(u); V.push_back(v);
    };
    // R1T1 top: T[i,j] = (-1)^(j+1) (-1)^(n+1) n²/(sf c_j (N-1))  (1-based j)
    auto add_top_neumann = [&]() {
        double sf = 0.0;
        for (int i = 0; i < N; i++) sf += -(double(i) * i) * sgn(i) * sgn(i + 1) / (cv[i] * (N - 1));
        std::vector<double> u(N), v(N);
        for (int i = 0; i < N; i++) u[i] = sgn(i + 1) * double(i) * i / sf;
        for (int j = 0; j < N; j++) v[j] = sgn(j + 2) / (cv[j] * (N - 1));
        U.push_back(u); V.push_back(v);
    };
    if (bcb == SS_CBC_R0 && bct == SS_CBC_R0) {
    } else if (bcb == SS_CBC_R1T0 && bct == SS_CBC_R0) { add_gl();
    } else if (bcb == SS_CBC_R1T1 && bct == SS_CBC_R0) { add_bot_neumann();
    } else if (bcb == SS_CBC_R0 && bct == SS_CBC_R1T0) { add_top_dirichlet();
    } else if (bcb == SS_CBC_R0 && bct == SS_CBC_R1T1) { add_top_neumann();
    } else if (bcb == SS_CBC_R1T0 && bct == SS_CBC_R1T0) { add_top_dirichlet(); add_gl();
    } else if (bcb == SS_CBC_R1T1 && bct == SS_CBC_R1T1) { add_bot_neumann(); add_top_neumann();
    } else if (bcb == SS_CBC_R1T0 && bct == SS_CBC_R1T1) { add_gl(); add_top_neumann();
    } else if (bcb == SS_CBC_R1T1 && bct == SS_CBC_R1T0) { add_bot_neumann(); add_top_dirichlet();
    } else {
        set_error("Chebyshev boundary condition combination not implemented (BCB=%d, BCT=%d)", bcb, bct);
        return SS_UNSUPPORTED_BC;
    }
    c.nrank = (int)U.size();
    c.gu.assign(size_t(c.nrank) * bk, 0.0);
    c.gv.assign(size_t(c.nrank) * N, 0.0);
    for (int p = 0; p < c.nrank; p++) {
        for (int i = 0; i < bk; i++) c.gu[size_t(p) * bk + i] = U[p][i];
        for (int j = 0; j < N; j++) c.gv[size_t(p) * N + j] = V[p][j];
    }
    return SS_OK;
}

// -------------------------------------------------------------- FFT plans
static std::complex<double> unit_root(long t, long n, int sign);
int64_t TwiddlePool::push_table(int n, int sign, int len) {
    int64_t off = size();
    for (int t = 0; t < len; t++) {
        std::complex<double> w = unit_root(t, n, sign);
        v.push_back(w.real());
        v.push_back(w.imag());
    }
    return off;
}
int64_t TwiddlePool::push(const std::vector<double> &ci) {
    int64_t off = size();
    v.insert(v.end(), ci.begin(), ci.end());
    return off;
}

// Radix sequence of an n-point DFT: odd primes 17..kMaxPrimeRadix first (as the
// first pass they need no input twiddles), then 4s and 2, 3, 5, 7, 11, 13.
// smooth_only (Bluestein lengths) admits 2, 3, 5, 7 only.  False when a prime
// factor is not covered (the caller then uses Bluestein).
static bool factor_radices(int n, int *rad, int &nrad, bool smooth_only, int max_prime = kMaxPrimeRadix) {
    nrad = 0;
    if (!smooth_only)
        for (int f = 17; f <= std::min(max_prime, kMaxPrimeRadix) && n > 1; f += 2) {
            bool prime = true;
            for (int d = 3; d * d <= f; d += 2)
                if (f % d == 0) { prime = false; break; }
            if (!prime) continue;
            while (n % f == 0) {
                if (nrad >= kMaxRadices) return false;
                rad[nrad++] = f;
                n /= f;
            }
        }
    while (n % 4 == 0 && n > 1) {
        if (nrad >= kMaxRadices) return false;
        rad[nrad++] = 4;
        n /= 4;
    }
    const int primes[] = {2, 3, 5, 7, 11, 13};
    for (int f : primes) {
        if (smooth_only && f > 7) break;
        while (n % f == 0) {
            if (nrad >= kMaxRadices) return false;
            rad[nrad++] = f;
            n /= f;
        }
    }
    return n == 1;
}

// exp(sign 2πi t/n) for 0 <= t < n, reduced by conjugate symmetry to t <= n/2
static std::complex<double> unit_root(long t, long n, int sign) {
    t %= n;
    if (t < 0) t += n;
    bool flip = 2 * t > n;
    long tt = flip ? n - t : t;
    double a = 2.0 * kPi * (double)tt / (double)n;
    double c = std::cos(a), sn = std::sin(a);
    if (flip) sn = -sn;
    return std::complex<double>(c, sign * sn);
}

// host Stockham (double) used only to precompute Bluestein filters; tw[t] = W_N^t
static void host_stockham(std::vector<std::complex<double>> &x, const int *rad, int nrad,
                          const std::vector<std::complex<double>> &tw) {
    const int N = (int)x.size();
    std::vector<std::complex<double>> y(N);
    int Ns = 1;
    for (int s = 0; s < nrad; s++) {
        int R = rad[s];
        for (int j = 0; j < N / R; j++) {
            int k = j % Ns;
            std::complex<double> v[16], o[16];
            for (int r = 0; r < R; r++) {
                v[r] = x[j + r * (N / R)];
                if (r > 0 && k > 0) v[r] *= tw[(size_t)k * r * (N / (Ns * R))];
            }
            for (int q = 0; q < R; q++) {
                std::complex<double> acc = 0;
                for (int r = 0; r < R; r++) acc += v[r] * tw[(size_t)((r * q) % R) * (N / R)];
                o[q] = acc;
            }
            int idxD = (j / Ns) * Ns * R + k;
            for (int r = 0; r < R; r++) y[idxD + r * Ns] = o[r];
        }
        x.swap(y);
        Ns *= R;
    }
}


static long mod_pow(long b, long e, long m) {
    long r = 1;
    b %= m;
    while (e > 0) {
        if (e & 1) r = r * b % m;
        b = b * b % m;
        e >>= 1;
    }
    return r;
}

// smallest primitive root of the prime p
static int primitive_root(int p) {
    std::vector<int> qs;
    int m = p - 1;
    for (int d = 2; d * d <= m; d++)
        if (m % d == 0) {
            qs.push_back(d);
            while (m % d == 0) m /= d;
        }
    if (m > 1) qs.push_back(m);
    for (int g = 2; g < p; g++) {
        bool ok = true;
        for (int q : qs)
            if (mod_pow(g, (p - 1) / q, p) == 1) { ok = false; break; }
        if (ok) return g;
    }
    return 1;
}

// Rader plan: N = p·m with p the largest prime factor, above max_prime; m and
// p − 1 covered by direct radices.  The p-point DFTs become cyclic convolutions of length p − 1
// (Rader, 1968): X_{g^{−b}} = x_0 + Σ_a x_{g^a} W_p^{g^{a−b}}.
static int largest_prime_factor(int n) {
    int P = 1;
    for (int d = 2; d * d <= n; d++)
        while (n % d == 0) { P = std::max(P, d); n /= d; }
    return n > 1 ? std::max(P, n) : P;
}

static bool rader_plan(int N, int max_prime, int pad_prime, FftPlan &p, TwiddlePool &pool) {
    const int P = largest_prime_factor(N);
    if (P <= max_prime || P > 4096) return false;
    int nr = 0;
    // the cofactor and the inner length take direct passes up to the hard limit;
    // an inner length with a prime factor above pad_prime becomes a smooth
    // M ≥ 2(P − 1) − 1 (radices 2, 3, 5, 7) carrying the zero-padded convolution
    if (!factor_radices(N / P, p.rad + 1, nr, false, kMaxPrimeRadix)) return false;
    const int P1 = P - 1;
    int M = P1;
    if (largest_prime_factor(P1) > pad_prime || !factor_radices(P1, p.rrad, p.rnrad, false, kMaxPrimeRadix)) {
        M = 2 * P1 - 1;
        while (!factor_radices(M, p.rrad, p.rnrad, true)) M++;
    }
    p.rad[0] = P;
    p.nrad = 1 + nr;
    p.rp = P;
    p.rM = M;
    p.rg = primitive_root(P);
    p.rtw = pool.push_table(M, -1, M);
    // h_d = W_P^{g^{−d}} (d < P − 1); padded, h'_{M−q} = h_{P−1−q} (1 ≤ q < P − 1)
    // and zero between, so that the length-M cyclic convolution of the
    // zero-padded u with h' equals u ⊛ h on its first P − 1 entries.
    // H = DFT_M(h')/M (forward sign)
    std::vector<std::complex<double>> h(M, 0.0), root(M);
    const long ginv = mod_pow(p.rg, P - 2, P);
    long e = 1;
    for (int d = 0; d < P1; d++) {
        h[d] = unit_root(e, P, -1);
        e = e * ginv % P;
    }
    if (M > P1)
        for (int q = 1; q < P1; q++) h[M - q] = h[P1 - q];
    for (int t = 0; t < M; t++) root[t] = unit_root(t, M, -1);
    bool small_radices = true;  // host_stockham takes radices up to 16
    for (int i = 0; i < p.rnrad; i++) small_radices = small_radices && p.rrad[i] <= 16;
    std::vector<std::complex<double>> Hc(M);
    if (small_radices) {
        Hc = h;
        host_stockham(Hc, p.rrad, p.rnrad, root);
    } else {
        for (int k = 0; k < M; k++) {
            std::complex<double> acc = 0.0;
            for (int d = 0; d < M; d++) acc += h[d] * root[(size_t)d * k % M];
            Hc[k] = acc;
        }
    }
    std::vector<double> H(2 * (size_t)M);
    for (int k = 0; k < M; k++) {
        H[2 * k] = Hc[k].real() / M;
        H[2 * k + 1] = Hc[k].imag() / M;
    }
    p.rH = pool.push(H);
    // index permutations of the gather (g^a) and the scatter (g^{−b})
    std::vector<double> perm(2 * (size_t)P1);
    long ga = 1, gb = 1;
    for (int a = 0; a < P1; a++) {
        perm[2 * a] = (double)ga;
        perm[2 * a + 1] = (double)gb;
        ga = ga * p.rg % P;
        gb = gb * ginv % P;
    }
    p.rperm = pool.push(perm);
    return true;
}

int PlanSet::plan_for(int N, TwiddlePool &pool) {
    if ((int)plan_of_N.size() <= N) plan_of_N.resize(N + 1, -1);
    if (plan_of_N[N] >= 0) return plan_of_N[N];
    FftPlan p;
    std::memset(&p, 0, sizeof p);
    p.N = N;
    if (factor_radices(N, p.rad, p.nrad, false, max_prime)) {
        p.blu = 0;
        p.tw = pool.push_table(N, -1, N);
    } else if (rader && rader_plan(N, max_prime, pad_prime, p, pool)) {
        p.blu = 0;
        p.tw = pool.push_table(N, -1, N);
    } else {
        std::memset(&p, 0, sizeof p);
        p.N = N;
        p.blu = 1;
        int M = 2 * N - 1;
        for (;; M++)
            if (factor_radices(M, p.mrad, p.mnrad, true)) break;
        p.M = M;
        p.nrad = 0;
        if ((int)mtw_of_M.size() <= M) mtw_of_M.resize(M + 1, -1);
        if (mtw_of_M[M] < 0) mtw_of_M[M] = pool.push_table(M, -1, M);
        p.mtw = mtw_of_M[M];
        std::vector<double> ch(2 * N);
        std::vector<std::complex<double>> c(N);
        for (long k = 0; k < N; k++) {
            long t = (k * k) % (2L * N);  // exp(-πi t/N) = W_{2N}^t
            c[k] = unit_root(t, 2L * N, -1);
            ch[2 * k] = c[k].real();
            ch[2 * k + 1] = c[k].imag();
        }
        p.chirp = pool.push(ch);
        std::vector<std::complex<double>> f(M, 0.0);
        f[0] = std::conj(c[0]);
        for (int k = 1; k < N; k++) { f[k] = std::conj(c[k]); f[M - k] = std::conj(c[k]); }
        std::vector<std::complex<double>> twm(M);
        for (int t = 0; t < M; t++) twm[t] = unit_root(t, M, -1);
        host_stockham(f, p.mrad, p.mnrad, twm);
        std::vector<double> fi(2 * M);
        for (int k = 0; k < M; k++) { fi[2 * k] = f[k].real() / M; fi[2 * k + 1] = f[k].imag() / M; }
        p.filt = pool.push(fi);
    }
    if (p.blu) {
        pass_tables(p.M, p.mrad, p.mnrad, 0, 1, p.mpt, pool);
        pass_tables(0, nullptr, 0, 0, 1, p.pt, pool);
        pass_tables(0, nullptr, 0, 0, 1, p.rpt, pool);
    } else if (p.rp) {
        pass_tables(N, p.rad, p.nrad, 1, p.rp, p.pt, pool);
        pass_tables(p.rM, p.rrad, p.rnrad, 0, 1, p.rpt, pool);
        pass_tables(0, nullptr, 0, 0, 1, p.mpt, pool);
    } else {
        pass_tables(N, p.rad, p.nrad, 0, 1, p.pt, pool);
        pass_tables(0, nullptr, 0, 0, 1, p.rpt, pool);
        pass_tables(0, nullptr, 0, 0, 1, p.mpt, pool);
    }
    for (int i = 0; i < kMaxRadices; i++) {
        const bool direct = i < p.nrad && p.rad[i] > 13 && !(p.rp && i == 0);
        p.pm[i] = direct ? prime_matrix(p.rad[i], pool) : -1;
        p.rpm[i] = (p.rp && i < p.rnrad && p.rrad[i] > 13) ? prime_matrix(p.rrad[i], pool) : -1;
    }
    plans.push_back(p);
    plan_of_N[N] = (int)plans.size() - 1;
    max_smem_cplx = std::max(max_smem_cplx, fft_buffer_len(p));
    return plan_of_N[N];
}

// DFT matrix of a direct radix-R prime pass (layout at prime_matrix_width),
// shared by every plan of the set.  Its offset is even, so that a binary32 row
// segment of two entries is one aligned 16-byte load.
int64_t PlanSet::prime_matrix(int R, TwiddlePool &pool) {
    if ((int)pm_of_R.size() <= R) pm_of_R.resize(R + 1, -1);
    if (pm_of_R[R] >= 0) return pm_of_R[R];
    if (pool.size() % 2) pool.v.insert(pool.v.end(), {0.0, 0.0});
    const int H = (R - 1) / 2, W = prime_matrix_width(R);
    std::vector<double> m(size_t(2) * H * W);
    for (int q = 1; q <= H; q++)
        for (int s = 0; s < W; s++) {
            const std::complex<double> w = unit_root((long)q * s, R, -1);
            m[2 * ((size_t)(q - 1) * W + s)] = w.real();
            m[2 * ((size_t)(q - 1) * W + s) + 1] = w.imag();
        }
    pm_of_R[R] = pool.push(m);
    return pm_of_R[R];
}

// Twiddle rows of one radix-R pass of an n-point DFT after Ns points are
// combined (layout at pass_row_width); shared by the plans that have it.
int64_t PlanSet::pass_table(int n, int Ns, int R, TwiddlePool &pool) {
    const std::array<int, 3> key{n, Ns, R};
    auto it = pt_of.find(key);
    if (it != pt_of.end()) return it->second;
    if (pool.size() % 2) pool.v.insert(pool.v.end(), {0.0, 0.0});
    const int W = pass_row_width(R);
    const long tstride = n / ((long)Ns * R);
    std::vector<double> t(size_t(2) * Ns * W);
    for (int k = 0; k < Ns; k++)
        for (int r = 1; r <= W; r++) {
            const std::complex<double> w = r < R ? unit_root((long)r * k * tstride, n, -1) : std::complex<double>(1.0, 0.0);
            t[2 * ((size_t)k * W + r - 1)] = w.real();
            t[2 * ((size_t)k * W + r - 1) + 1] = w.imag();
        }
    const int64_t off = pool.push(t);
    pt_of[key] = off;
    return off;
}

// Per-pass twiddle rows of the radix passes s0..nrad−1 of an n-point plan
// whose first Ns0 points are already combined; −1 for prime passes and for
// passes with Ns = 1 (no input twiddles).
void PlanSet::pass_tables(int n, const int *rad, int nrad, int s0, int Ns0, int64_t *pt, TwiddlePool &pool) {
    for (int i = 0; i < kMaxRadices; i++) pt[i] = -1;
    int Ns = Ns0;
    for (int s = s0; s < nrad; s++) {
        const int R = rad[s];
        if (R <= 13 && Ns > 1) pt[s] = pass_table(n, Ns, R, pool);
        Ns *= R;
    }
}

int64_t PlanSet::unpack_for(int L, TwiddlePool &pool) {
    if ((int)utw_of_L.size() <= L) utw_of_L.resize(L + 1, -1);
    if (utw_of_L[L] < 0) utw_of_L[L] = pool.push_table(L, -1, L / 2);
    return utw_of_L[L];
}

}  // namespace ss

namespace ss {
// SI / SIx / SIxx weights at arbitrary radii (SItransform(sp, a, points, u, d),
// src/CubicBSpline.jl:1554-1567, 1650-1654, 1695-1699): the 4-coefficient window
// m0[i] of point x[i] and the basis values w[(d·n + i)·4 + tap]
int32_t spline_point_weights(const SplineHost &s, const double *x, int n, std::vector<int> &m0,
                             std::vector<double> &w) {
    const int Md = s.bDim, nc = s.nc;
    m0.assign(n, 0);
    w.assign(size_t(3) * n * 4, 0.0);
    for (int i = 0; i < n; i++) {
        const long xm = (long)std::ceil((x[i] - s.xmin - (2.0 * s.DX)) * s.DXrecip);
        const int base = std::min(std::max(int(xm) + 1, 0), Md - 4);
        m0[i] = base;
        for (int q = 0; q < 4; q++) {
            const long m = xm + q;
            if (m < -1 || m > nc + 1) continue;
            const int idx = int(m + 1) - base;
            if (idx < 0 || idx > 3) continue;  // a point outside [xmin, xmax]: the terms the window cannot hold
            for (int d = 0; d < 3; d++) w[(size_t(d) * n + i) * 4 + idx] = bspline(s, int(m), x[i], d);
        }
    }
    return SS_OK;
}
}  // namespace ss
