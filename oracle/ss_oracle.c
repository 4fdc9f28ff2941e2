/*
 * ss_oracle.c — FP64 CPU restatement of the Springsteel.jl RL/RLZ transform
 * hot path.  TEST INFRASTRUCTURE ONLY (the checker and the timed CPU
 * baseline); the GPU library never links or calls it.
 *
 * Each function cites the reference file:line it restates.  FFTW (FFTW.jl,
 * compat "1", version unpinned: the reference ships no Manifest) is the
 * third-party library behind FBtransform!/FItransform!/CBtransform!/
 * CItransform!; its R2HC, HC2R and REDFT00 kinds are restated from their
 * published definitions (FFTW manual, "What FFTW Really Computes") by a
 * self-written mixed-radix + Bluestein DFT below.
 */
#include "ss_oracle.h"

#include <complex.h>
#include <math.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double _Complex cplx;

static _Thread_local char g_err[512] = "";
static void set_err(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof g_err, fmt, ap);
    va_end(ap);
}
const char *or_last_error(void) { return g_err; }

static int g_threads = 1;
void or_set_threads(int n) { g_threads = n < 1 ? 1 : n; }

static const double PI = 3.14159265358979323846264338327950288;

/* ======================================================================
 * DFT engine (restates FFTW's transform definitions, not its code)
 * ====================================================================== */

typedef struct fft_plan {
    int n;
    int nfac;
    int fac[64];
    cplx *tw;          /* exp(-2πi t/n), t = 0..n-1 */
    int blu;           /* Bluestein for n with a prime factor > 13 */
    int m;             /* power-of-two convolution length */
    cplx *chirp;       /* exp(-πi k²/n) */
    cplx *bfft;        /* FFT_m of the conjugate chirp filter */
    struct fft_plan *sub;
} fft_plan;

static cplx twiddle(long t, long n) {
    /* exp(-2πi t/n) with t reduced modulo n first */
    t %= n;
    if (t < 0) t += n;
    double ang = -2.0 * PI * (double)t / (double)n;
    return cos(ang) + I * sin(ang);
}

static fft_plan *fft_plan_create(int n);

static void fft_plan_destroy(fft_plan *p) {
    if (!p) return;
    free(p->tw);
    free(p->chirp);
    free(p->bfft);
    fft_plan_destroy(p->sub);
    free(p);
}

static void fft_exec(const fft_plan *p, cplx *x, cplx *work);

static fft_plan *fft_plan_create(int n) {
    fft_plan *p = (fft_plan *)calloc(1, sizeof *p);
    p->n = n;
    int rem = n;
    int bigprime = 0;
    /* prefer radix 4 then small primes */
    while (rem % 4 == 0) { p->fac[p->nfac++] = 4; rem /= 4; }
    for (int f = 2; f <= 13 && rem > 1; f++) {
        while (rem % f == 0) { p->fac[p->nfac++] = f; rem /= f; }
    }
    if (rem > 1) bigprime = 1;
    if (!bigprime) {
        p->tw = (cplx *)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
        for (int t = 0; t < n; t++) p->tw[t] = twiddle(t, n);
        return p;
    }
    /* Bluestein: X_k = c_k Σ_j (x_j c_j) conj(c_{k-j}), c_k = exp(-πi k²/n) */
    p->blu = 1;
    int m = 1;
    while (m < 2 * n - 1) m <<= 1;
    p->m = m;
    p->chirp = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    for (long k = 0; k < n; k++) {
        long t = (k * k) % (2L * n); /* exact reduction of k² mod 2n */
        double ang = -PI * (double)t / (double)n;
        p->chirp[k] = cos(ang) + I * sin(ang);
    }
    p->sub = fft_plan_create(m);
    p->bfft = (cplx *)calloc((size_t)m, sizeof(cplx));
    p->bfft[0] = conj(p->chirp[0]);
    for (int k = 1; k < n; k++) {
        p->bfft[k] = conj(p->chirp[k]);
        p->bfft[m - k] = conj(p->chirp[k]);
    }
    cplx *w = (cplx *)malloc(sizeof(cplx) * (size_t)m);
    fft_exec(p->sub, p->bfft, w);
    free(w);
    return p;
}

/* recursive decimation-in-time mixed radix, out-of-place into `out` */
static void fft_rec(const fft_plan *p, int fi, const cplx *in, int stride, cplx *out, int n) {
    if (n == 1) { out[0] = in[0]; return; }
    int r = p->fac[fi];
    int m = n / r;
    for (int q = 0; q < r; q++) fft_rec(p, fi + 1, in + (size_t)q * stride, stride * r, out + (size_t)q * m, m);
    int tstep = p->n / n; /* twiddles of length-n stage from the size-N table */
    cplx y[16];
    for (int k = 0; k < m; k++) {
        for (int q = 0; q < r; q++) y[q] = out[(size_t)q * m + k];
        for (int s = 0; s < r; s++) {
            cplx acc = 0;
            long kk = k + (long)s * m;
            for (int q = 0; q < r; q++) {
                long e = ((long)q * kk) % n;
                acc += y[q] * p->tw[(size_t)e * tstep];
            }
            out[(size_t)s * m + k] = acc;
        }
        /* y held the old column; outputs written after all reads of this k */
    }
}

/* in-place forward DFT X_k = Σ x_j exp(-2πi jk/n); work has ≥ 2*max(n, m) entries */
static void fft_exec(const fft_plan *p, cplx *x, cplx *work) {
    int n = p->n;
    if (!p->blu) {
        /* fft_rec reads all inputs of a stage before writing (column buffer y),
         * but sub-stages write into `out` slices; use work as the output */
        fft_rec(p, 0, x, 1, work, n);
        memcpy(x, work, sizeof(cplx) * (size_t)n);
        return;
    }
    int m = p->m;
    cplx *a = work;          /* m */
    cplx *w2 = work + m;     /* m (sub work) */
    for (int k = 0; k < n; k++) a[k] = x[k] * p->chirp[k];
    for (int k = n; k < m; k++) a[k] = 0;
    fft_exec(p->sub, a, w2);
    for (int k = 0; k < m; k++) a[k] *= p->bfft[k];
    /* inverse via conjugation */
    for (int k = 0; k < m; k++) a[k] = conj(a[k]);
    fft_exec(p->sub, a, w2);
    double inv = 1.0 / (double)m;
    for (int k = 0; k < n; k++) x[k] = conj(a[k]) * inv * p->chirp[k];
}

static size_t fft_work_len(const fft_plan *p) {
    if (!p->blu) return (size_t)p->n;
    return (size_t)2 * p->m + fft_work_len(p->sub);
}

/* plan cache (created before any parallel region; read-only afterwards) */
typedef struct { int n; fft_plan *p; } plan_entry;
static plan_entry *g_plans = NULL;
static int g_nplans = 0, g_capplans = 0;
static fft_plan *get_plan(int n) {
    fft_plan *found = NULL;
#pragma omp critical(or_plan_cache)
    {
        for (int i = 0; i < g_nplans; i++)
            if (g_plans[i].n == n) { found = g_plans[i].p; break; }
        if (!found) {
            if (g_nplans == g_capplans) {
                g_capplans = g_capplans ? 2 * g_capplans : 64;
                g_plans = (plan_entry *)realloc(g_plans, sizeof(plan_entry) * (size_t)g_capplans);
            }
            found = fft_plan_create(n);
            g_plans[g_nplans].n = n;
            g_plans[g_nplans].p = found;
            g_nplans++;
        }
    }
    return found;
}

/* FFTW R2HC: r_k = Re X_k (k ≤ n/2), i_k = Im X_k stored at n-k (0<k<(n+1)/2) */
static void r2hc_p(const fft_plan *p, const double *x, double *out, cplx *buf, cplx *work) {
    int n = p->n;
    for (int j = 0; j < n; j++) buf[j] = x[j];
    fft_exec(p, buf, work);
    out[0] = creal(buf[0]);
    for (int k = 1; k < (n + 1) / 2; k++) {
        out[k] = creal(buf[k]);
        out[n - k] = cimag(buf[k]);
    }
    if (n % 2 == 0) out[n / 2] = creal(buf[n / 2]);
}

/* FFTW HC2R: unnormalised inverse of R2HC, x_j = Σ_k X_k exp(+2πi jk/n) */
static void hc2r_p(const fft_plan *p, const double *h, double *out, cplx *buf, cplx *work) {
    int n = p->n;
    buf[0] = h[0];
    for (int k = 1; k < (n + 1) / 2; k++) {
        buf[k] = h[k] + I * h[n - k];
        buf[n - k] = h[k] - I * h[n - k];
    }
    if (n % 2 == 0) buf[n / 2] = h[n / 2];
    /* inverse DFT = conj(DFT(conj(X))) */
    for (int k = 0; k < n; k++) buf[k] = conj(buf[k]);
    fft_exec(p, buf, work);
    for (int j = 0; j < n; j++) out[j] = creal(buf[j]); /* conj leaves Re unchanged */
}

int32_t or_r2hc(const double *x, int32_t n, double *out) {
    if (n < 1) { set_err("n < 1"); return SS_BAD_ARG; }
    const fft_plan *p = get_plan(n);
    cplx *buf = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *work = (cplx *)malloc(sizeof(cplx) * fft_work_len(p));
    r2hc_p(p, x, out, buf, work);
    free(buf); free(work);
    return SS_OK;
}
int32_t or_hc2r(const double *x, int32_t n, double *out) {
    if (n < 1) { set_err("n < 1"); return SS_BAD_ARG; }
    const fft_plan *p = get_plan(n);
    cplx *buf = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    cplx *work = (cplx *)malloc(sizeof(cplx) * fft_work_len(p));
    hc2r_p(p, x, out, buf, work);
    free(buf); free(work);
    return SS_OK;
}

/* FFTW REDFT00: Y_k = x_0 + (-1)^k x_{n-1} + 2 Σ_{j=1}^{n-2} x_j cos(πjk/(n-1)).
 * Direct O(n²) sum with an exactly reduced cosine table (n ≤ a few hundred). */
typedef struct { int n; double *cosv; } dct_table; /* cos(π t/(n-1)), t = 0..2(n-1)-1 */
static dct_table *g_dct = NULL;
static int g_ndct = 0;
static const double *get_dct(int n) {
    const double *found = NULL;
#pragma omp critical(or_dct_cache)
    {
        for (int i = 0; i < g_ndct; i++)
            if (g_dct[i].n == n) { found = g_dct[i].cosv; break; }
        if (!found) {
            g_dct = (dct_table *)realloc(g_dct, sizeof(dct_table) * (size_t)(g_ndct + 1));
            int per = 2 * (n - 1);
            double *c = (double *)malloc(sizeof(double) * (size_t)(per > 0 ? per : 1));
            for (int t = 0; t < per; t++) c[t] = cos(PI * (double)t / (double)(n - 1));
            g_dct[g_ndct].n = n;
            g_dct[g_ndct].cosv = c;
            g_ndct++;
            found = c;
        }
    }
    return found;
}
static void redft00_t(const double *c, const double *x, int n, double *y) {
    if (n == 1) { y[0] = x[0]; return; }
    int per = 2 * (n - 1);
    for (int k = 0; k < n; k++) {
        double s = 0.0;
        for (int j = 1; j <= n - 2; j++) s += x[j] * c[((long)j * k) % per];
        y[k] = x[0] + ((k & 1) ? -x[n - 1] : x[n - 1]) + 2.0 * s;
    }
}
int32_t or_redft00(const double *x, int32_t n, double *out) {
    if (n < 1) { set_err("n < 1"); return SS_BAD_ARG; }
    redft00_t(n > 1 ? get_dct(n) : NULL, x, n, out);
    return SS_OK;
}

/* ======================================================================
 * Cubic B-spline basis (src/CubicBSpline.jl)
 * ====================================================================== */

enum { GBC_R0 = 0, GBC_A1 = 1, GBC_A2 = 2, GBC_PER = 3, GBC_R3 = 4 };

struct or_spline {
    double xmin, xmax, DX, DXrecip, l_q;
    int nc, mubar, quad, bDim, mishDim;
    double qpts[64], qwts[64];
    /* GammaBC (src/CubicBSpline.jl:321-424) */
    int Mdim, Min, rankL, rankR, lk, rk;
    double aL, bL, aR, bR;
    int r3x;
    double *PQb;   /* full P+Q, band storage PQb[i*7 + (j-i+3)] (|i-j| ≤ 3) */
    double *L4;    /* banded Cholesky factor of Γ(P+Q)Γᵀ, L4[j*4+d] = L[j+d][j] */
    int periodic;  /* PERIODIC on either side: dense factor (DenseSplineFactor) */
    double *Ld;    /* periodic: dense lower Cholesky factor, Ld[i + j*n] = L[i][j] */
    double *mish;
};

/* _quadrature_rule, src/CubicBSpline.jl:172-200 (GL tables :128-155) */
static int quadrature_rule(int mb, int quad, double *qp, double *qw) {
    if (mb < 1) { set_err("mubar must be >= 1, got %d", mb); return SS_BAD_ARG; }
    if (quad == SS_QUAD_GAUSS) {
        double nodes[5], w[5];
        if (mb > 5) { set_err("Gauss-Legendre tables only for mubar 1-5, got %d", mb); return SS_BAD_ARG; }
        if (mb == 1) { nodes[0] = 0.0; w[0] = 2.0; }
        if (mb == 2) { nodes[0] = -1.0 / sqrt(3.0); nodes[1] = 1.0 / sqrt(3.0); w[0] = w[1] = 1.0; }
        if (mb == 3) {
            nodes[0] = -sqrt(3.0 / 5.0); nodes[1] = 0.0; nodes[2] = sqrt(3.0 / 5.0);
            w[0] = 5.0 / 9.0; w[1] = 8.0 / 9.0; w[2] = 5.0 / 9.0;
        }
        if (mb == 4) {
            double a = sqrt(3.0 / 7.0 + 2.0 / 7.0 * sqrt(6.0 / 5.0));
            double b = sqrt(3.0 / 7.0 - 2.0 / 7.0 * sqrt(6.0 / 5.0));
            nodes[0] = -a; nodes[1] = -b; nodes[2] = b; nodes[3] = a;
            w[0] = (18.0 - sqrt(30.0)) / 36.0; w[1] = (18.0 + sqrt(30.0)) / 36.0;
            w[2] = (18.0 + sqrt(30.0)) / 36.0; w[3] = (18.0 - sqrt(30.0)) / 36.0;
        }
        if (mb == 5) {
            double a = sqrt(5.0 + 2.0 * sqrt(10.0 / 7.0)) / 3.0;
            double b = sqrt(5.0 - 2.0 * sqrt(10.0 / 7.0)) / 3.0;
            nodes[0] = -a; nodes[1] = -b; nodes[2] = 0.0; nodes[3] = b; nodes[4] = a;
            w[0] = (322.0 - 13.0 * sqrt(70.0)) / 900.0; w[1] = (322.0 + 13.0 * sqrt(70.0)) / 900.0;
            w[2] = 128.0 / 225.0;
            w[3] = (322.0 + 13.0 * sqrt(70.0)) / 900.0; w[4] = (322.0 - 13.0 * sqrt(70.0)) / 900.0;
        }
        for (int k = 0; k < mb; k++) { qp[k] = (nodes[k] + 1.0) / 2.0; qw[k] = w[k] / 2.0; }
        return SS_OK;
    }
    if (quad == SS_QUAD_REGULAR) {
        if (mb > 64) { set_err("mubar > 64 unsupported"); return SS_BAD_ARG; }
        for (int k = 1; k <= mb; k++) { qp[k - 1] = (double)(2 * k - 1) / (double)(2 * mb); qw[k - 1] = 1.0 / mb; }
        return SS_OK;
    }
    set_err("unknown quadrature %d", quad);
    return SS_BAD_ARG;
}

/* basis(sp, m, x, derivative), src/CubicBSpline.jl:585-628 */
static double basis(const or_spline *s, int m, double x, int d) {
    double b = 0.0;
    double xm = s->xmin + (m * s->DX);
    double delta = (x - xm) * s->DXrecip;
    double z = fabs(delta);
    if (z < 2.0) {
        if (d == 0) {
            z = 2.0 - z;
            b = (z * z * z) * (1.0 / 6.0);
            z -= 1.0;
            if (z > 0) b -= (z * z * z) * (4.0 / 6.0);
        } else if (d == 1) {
            z = 2.0 - z;
            b = (z * z) * (1.0 / 6.0);
            z -= 1.0;
            if (z > 0) b -= (z * z) * (4.0 / 6.0);
            b *= ((delta > 0) ? -1.0 : 1.0) * 3.0 * s->DXrecip;
        } else if (d == 2) {
            z = 2.0 - z;
            b = z;
            z -= 1.0;
            if (z > 0) b -= z * 4;
            b *= s->DXrecip * s->DXrecip;
        } else if (d == 3) {
            if (z > 1.0) b = 1.0;
            else if (z < 1.0) b = -3.0;
            b *= ((delta > 0) ? -1.0 : 1.0) * s->DXrecip * s->DXrecip * s->DXrecip;
        }
    }
    return b;
}
double or_basis(const or_spline *s, int32_t m, double x, int32_t d) {
    if (x < s->xmin || x > s->xmax) return NAN; /* DomainError in the reference */
    return basis(s, m, x, d);
}

/* GammaBC(sp), src/CubicBSpline.jl:382-424 */
static int gamma_setup(or_spline *s, const ss_spline_bc *bcl, const ss_spline_bc *bcr) {
    ss_spline_bc r0 = {SS_SBC_R0, 0, 0.0, 0.0};
    if (!bcl) bcl = &r0;
    if (!bcr) bcr = &r0;
    s->r3x = 0;
    switch (bcl->kind) {
    case SS_SBC_RANK1: s->rankL = 1; s->lk = GBC_A1; s->aL = bcl->alpha; s->bL = bcl->beta; break;
    case SS_SBC_RANK2: s->rankL = 2; s->lk = GBC_A2; s->aL = bcl->alpha; s->bL = bcl->beta; break;
    case SS_SBC_R0: s->rankL = 0; s->lk = GBC_R0; s->aL = s->bL = 0.0; break;
    case SS_SBC_R3: case SS_SBC_R3X:
        s->rankL = 3; s->lk = GBC_R3; s->aL = s->bL = 0.0; if (bcl->kind == SS_SBC_R3X) s->r3x = 1; break;
    case SS_SBC_PERIODIC: s->rankL = 1; s->lk = GBC_PER; s->aL = s->bL = 0.0; break;  /* :395-397 */
    default: set_err("GammaBC: unrecognised BCL kind %d", bcl->kind); return SS_UNSUPPORTED_BC;
    }
    switch (bcr->kind) {
    case SS_SBC_RANK1: s->rankR = 1; s->rk = GBC_A1; s->aR = bcr->alpha; s->bR = bcr->beta; break;
    case SS_SBC_RANK2: s->rankR = 2; s->rk = GBC_A2; s->aR = bcr->alpha; s->bR = bcr->beta; break;
    case SS_SBC_R0: s->rankR = 0; s->rk = GBC_R0; s->aR = s->bR = 0.0; break;
    case SS_SBC_R3: case SS_SBC_R3X:
        s->rankR = 3; s->rk = GBC_R3; s->aR = s->bR = 0.0; if (bcr->kind == SS_SBC_R3X) s->r3x = 1; break;
    case SS_SBC_PERIODIC: s->rankR = 2; s->rk = GBC_PER; s->aR = s->bR = 0.0; break;  /* :414-416 */
    default: set_err("GammaBC: unrecognised BCR kind %d", bcr->kind); return SS_UNSUPPORTED_BC;
    }
    s->Mdim = s->nc + 3;
    s->Min = s->Mdim - s->rankL - s->rankR;
    s->periodic = (s->lk == GBC_PER || s->rk == GBC_PER);
    if (s->Min < 1) { set_err("no interior coefficients (num_cells too small for the BCs)"); return SS_BAD_SHAPE; }
    return SS_OK;
}

/* dense Γ entry, getindex src/CubicBSpline.jl:336-376 (1-based i, j) */
static double gamma_at(const or_spline *g, int i, int j) {
    double val = (j == i + g->rankL) ? 1.0 : 0.0;
    if (g->lk == GBC_A1) {
        if (j == 1) { if (i == 1) val += g->aL; if (i == 2) val += g->bL; }
    } else if (g->lk == GBC_A2) {
        if (j == 1 && i == 1) val += g->aL;
        else if (j == 2 && i == 1) val += g->bL;
    } else if (g->lk == GBC_PER) {
        if (j == 1 && i == g->Min) val += 1.0;
    }
    if (g->rk == GBC_A1) {
        if (j == g->Mdim) { if (i == g->Min) val += g->aR; if (i == g->Min - 1) val += g->bR; }
    } else if (g->rk == GBC_A2) {
        if (j == g->Mdim && i == g->Min) val += g->aR;
        else if (j == g->Mdim - 1 && i == g->Min) val += g->bR;
    } else if (g->rk == GBC_PER) {  /* src/CubicBSpline.jl:366-369 */
        if (j == g->Mdim - 1 && i == 1) val += 1.0;
        if (j == g->Mdim && i == 2) val += 1.0;
    }
    return val;
}

/* out (Min) ← Γ b (Mdim), src/CubicBSpline.jl:427-458 */
static void gamma_apply(const or_spline *g, const double *b, double *out) {
    int Min = g->Min, rL = g->rankL, Mdim = g->Mdim;
    for (int i = 0; i < Min; i++) out[i] = b[i + rL];
    if (g->lk == GBC_A1) { out[0] += g->aL * b[0]; out[1] += g->bL * b[0]; }
    else if (g->lk == GBC_A2) { out[0] += g->aL * b[0] + g->bL * b[1]; }
    else if (g->lk == GBC_PER) { out[Min - 1] += b[0]; }
    if (g->rk == GBC_A1) { out[Min - 1] += g->aR * b[Mdim - 1]; out[Min - 2] += g->bR * b[Mdim - 1]; }
    else if (g->rk == GBC_A2) { out[Min - 1] += g->aR * b[Mdim - 1] + g->bR * b[Mdim - 2]; }
    else if (g->rk == GBC_PER) { out[0] += b[Mdim - 2]; out[1] += b[Mdim - 1]; }
}

/* out (Mdim) ← Γᵀ x (Min), src/CubicBSpline.jl:461-500 */
static void gamma_adjoint(const or_spline *g, const double *x, double *out) {
    int Min = g->Min, rL = g->rankL, rR = g->rankR, Mdim = g->Mdim;
    for (int j = 0; j < rL; j++) out[j] = 0.0;
    for (int j = Mdim - rR; j < Mdim; j++) out[j] = 0.0;
    for (int i = 0; i < Min; i++) out[i + rL] = x[i];
    if (g->lk == GBC_A1) out[0] = g->aL * x[0] + g->bL * x[1];
    else if (g->lk == GBC_A2) { out[0] = g->aL * x[0]; out[1] = g->bL * x[0]; }
    else if (g->lk == GBC_PER) out[0] = x[Min - 1];
    if (g->rk == GBC_A1) out[Mdim - 1] = g->aR * x[Min - 1] + g->bR * x[Min - 2];
    else if (g->rk == GBC_A2) { out[Mdim - 2] = g->bR * x[Min - 1]; out[Mdim - 1] = g->aR * x[Min - 1]; }
    else if (g->rk == GBC_PER) { out[Mdim - 2] = x[0]; out[Mdim - 1] = x[1]; }
}

/* cholesky_dense_factor / DenseSplineFactor (src/banded_cholesky.jl:70, 250-260;
 * LAPACK potrf's A = L Lᵀ, lower): the periodic case, whose Γ wrap-around
 * couples the first and last interior coefficients.  A column-major n × n,
 * overwritten by L in its lower triangle. */
static int dense_chol(double *A, int n) {
    for (int j = 0; j < n; j++) {
        double d = A[j + (size_t)j * n];
        for (int k = 0; k < j; k++) d -= A[j + (size_t)k * n] * A[j + (size_t)k * n];
        if (d <= 0.0) { set_err("PosDefException(%d)", j + 1); return SS_NOT_SPD; }
        const double ljj = sqrt(d);
        A[j + (size_t)j * n] = ljj;
        for (int i = j + 1; i < n; i++) {
            double t = A[i + (size_t)j * n];
            for (int k = 0; k < j; k++) t -= A[i + (size_t)k * n] * A[j + (size_t)k * n];
            A[i + (size_t)j * n] = t / ljj;
        }
        for (int i = 0; i < j; i++) A[i + (size_t)j * n] = 0.0;
    }
    return SS_OK;
}
static void dense_solve(const double *L, int n, const double *b, double *x) {
    for (int i = 0; i < n; i++) {
        double t = b[i];
        for (int k = 0; k < i; k++) t -= L[i + (size_t)k * n] * x[k];
        x[i] = t / L[i + (size_t)i * n];
    }
    for (int i = n - 1; i >= 0; i--) {
        double t = x[i];
        for (int k = i + 1; k < n; k++) t -= L[k + (size_t)i * n] * x[k];
        x[i] = t / L[i + (size_t)i * n];
    }
}

/* _band_factor3!, src/banded_cholesky.jl:166-197 (0-based; L4[j*4+d] = L[j+d][j]) */
static int band_factor3(double *L4, int n) {
    for (int j = 0; j < n; j++) {
        double d = L4[j * 4 + 0];
        int ks = j - 3 > 0 ? j - 3 : 0;
        for (int k = ks; k < j; k++) {
            double ljk = L4[k * 4 + (j - k)];
            d -= ljk * ljk;
        }
        if (d <= 0.0) { set_err("PosDefException(%d)", j + 1); return SS_NOT_SPD; }
        double ljj = sqrt(d);
        L4[j * 4] = ljj;
        double inv = 1.0 / ljj;
        int ihi = j + 3 < n - 1 ? j + 3 : n - 1;
        for (int i = j + 1; i <= ihi; i++) {
            double s = L4[j * 4 + (i - j)];
            int kst = i - 3 > 0 ? i - 3 : 0;
            for (int k = kst; k < j; k++) s -= L4[k * 4 + (i - k)] * L4[k * 4 + (j - k)];
            L4[j * 4 + (i - j)] = s * inv;
        }
    }
    return SS_OK;
}

/* _band_forward_solve3! / _band_backward_solve3!, src/banded_cholesky.jl:202-231 */
static void band_solve3(const double *L4, int n, const double *b, double *x) {
    for (int i = 0; i < n; i++) {
        double s = b[i];
        int ks = i - 3 > 0 ? i - 3 : 0;
        for (int k = ks; k < i; k++) s -= L4[k * 4 + (i - k)] * x[k];
        x[i] = s / L4[i * 4];
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = x[i];
        int kh = i + 3 < n - 1 ? i + 3 : n - 1;
        for (int k = i + 1; k <= kh; k++) s -= L4[i * 4 + (k - i)] * x[k];
        x[i] = s / L4[i * 4];
    }
}

/* cholesky_banded3 on a dense symmetric matrix, src/banded_cholesky.jl:99-147 */
int32_t or_band_chol(const double *A, int32_t n, double *L4) {
    for (int j = 0; j < n; j++)
        for (int i = j + 4; i < n; i++)
            if (A[i + (size_t)j * n] != 0.0) {
                set_err("cholesky_banded3 expects half-bandwidth <= 3, A[%d,%d] outside", i + 1, j + 1);
                return SS_BAD_ARG;
            }
    for (int j = 0; j < n; j++)
        for (int d = 0; d < 4; d++) L4[j * 4 + d] = (j + d < n) ? A[(j + d) + (size_t)j * n] : 0.0;
    return band_factor3(L4, n);
}
int32_t or_band_solve(const double *L4, int32_t n, const double *b, double *x) {
    band_solve3(L4, n, b, x);
    return SS_OK;
}

/* calcPQfactor, src/CubicBSpline.jl:733-783 */
static int pq_setup(or_spline *s) {
    int Mdim = s->Mdim;
    double eps_q = pow((s->l_q * s->DX) / (2 * PI), 6);
    double *P = (double *)calloc((size_t)Mdim * 7, sizeof(double));
    double *Q = (double *)calloc((size_t)Mdim * 7, sizeof(double));
    for (int mi1 = 1; mi1 <= Mdim; mi1++) {
        for (int mi2 = 1; mi2 <= Mdim; mi2++) {
            if (abs(mi1 - mi2) > 3) continue;
            int m1 = mi1 - 2, m2 = mi2 - 2;
            for (int mc = 0; mc <= s->nc - 1; mc++) {
                if (mc < m1 - 2 || mc > m1 + 1) continue;
                if (mc < m2 - 2 || mc > m2 + 1) continue;
                for (int mu = 0; mu < s->mubar; mu++) {
                    double x = s->xmin + mc * s->DX + s->qpts[mu] * s->DX;
                    double pm1 = basis(s, m1, x, 0), qm1 = basis(s, m1, x, 3);
                    double pm2 = basis(s, m2, x, 0), qm2 = basis(s, m2, x, 3);
                    P[(mi1 - 1) * 7 + (mi2 - mi1 + 3)] += s->DX * s->qwts[mu] * pm1 * pm2;
                    Q[(mi1 - 1) * 7 + (mi2 - mi1 + 3)] += s->DX * s->qwts[mu] * eps_q * qm1 * qm2;
                }
            }
        }
    }
    s->PQb = (double *)calloc((size_t)Mdim * 7, sizeof(double));
    for (int i = 0; i < Mdim * 7; i++) s->PQb[i] = P[i] + Q[i];
    /* PQopen = Γ P Γᵀ + Γ Q Γᵀ, computed on the ±6 band (Γ rows have ≤ 3 entries);
     * periodic: every entry (the wrap-around couples the two ends) */
    int n = s->Min;
    double *A = (double *)calloc((size_t)n * n, sizeof(double));
    for (int i = 1; i <= n; i++) {
        const int jlo = s->periodic ? 1 : (i - 6 > 1 ? i - 6 : 1), jhi = s->periodic ? n : (i + 6 < n ? i + 6 : n);
        for (int j = jlo; j <= jhi; j++) {
            double accP = 0.0, accQ = 0.0;
            for (int a = 1; a <= Mdim; a++) {
                double ga = gamma_at(s, i, a);
                if (ga == 0.0) continue;
                for (int b = (a - 3 > 1 ? a - 3 : 1); b <= (a + 3 < Mdim ? a + 3 : Mdim); b++) {
                    double gb = gamma_at(s, j, b);
                    if (gb == 0.0) continue;
                    accP += ga * P[(a - 1) * 7 + (b - a + 3)] * gb;
                    accQ += ga * Q[(a - 1) * 7 + (b - a + 3)] * gb;
                }
            }
            A[(i - 1) + (size_t)(j - 1) * n] = accP + accQ;
        }
    }
    free(P); free(Q);
    s->L4 = (double *)calloc((size_t)n * 4, sizeof(double));
    int st;
    if (s->periodic) {  /* calcPQfactor: is_periodic → cholesky_dense_factor (:777-781) */
        st = dense_chol(A, n);
        s->Ld = A;
        for (int j = 0; j < n; j++)
            for (int d = 0; d < 4 && j + d < n; d++) s->L4[j * 4 + d] = A[(j + d) + (size_t)j * n];
        return st;
    }
    st = or_band_chol(A, n, s->L4);
    free(A);
    return st;
}

/* calcMishPoints, src/CubicBSpline.jl:887-897 */
static void spline_mish(const or_spline *s, double *x) {
    for (int mc = 0; mc < s->nc; mc++)
        for (int mu = 0; mu < s->mubar; mu++)
            x[mu + s->mubar * mc] = s->xmin + mc * s->DX + s->qpts[mu] * s->DX;
}

int32_t or_spline_create(double xmin, double xmax, int32_t nc, int32_t mubar, int32_t quad,
                         double l_q, const ss_spline_bc *bcl, const ss_spline_bc *bcr,
                         or_spline **out) {
    *out = NULL;
    if (nc < 1) { set_err("num_cells must be >= 1"); return SS_BAD_ARG; }
    if (!(xmax > xmin)) { set_err("xmax must exceed xmin"); return SS_BAD_ARG; }
    or_spline *s = (or_spline *)calloc(1, sizeof *s);
    s->xmin = xmin; s->xmax = xmax; s->nc = nc; s->mubar = mubar; s->quad = quad; s->l_q = l_q;
    s->DX = (xmax - xmin) / nc;
    s->DXrecip = 1.0 / s->DX;
    s->bDim = nc + 3;
    s->mishDim = nc * mubar;
    int st = quadrature_rule(mubar, quad, s->qpts, s->qwts);
    if (st == SS_OK) st = gamma_setup(s, bcl, bcr);
    if (st == SS_OK) st = pq_setup(s);
    if (st != SS_OK) { or_spline_destroy(s); return st; }
    s->mish = (double *)malloc(sizeof(double) * (size_t)s->mishDim);
    spline_mish(s, s->mish);
    *out = s;
    return SS_OK;
}
void or_spline_destroy(or_spline *s) {
    if (!s) return;
    free(s->PQb); free(s->L4); free(s->Ld); free(s->mish); free(s);
}
int32_t or_spline_info(const or_spline *s, int32_t *bDim, int32_t *mishDim, int32_t *Min) {
    *bDim = s->bDim; *mishDim = s->mishDim; *Min = s->Min;
    return SS_OK;
}
int32_t or_spline_mish(const or_spline *s, double *x) { spline_mish(s, x); return SS_OK; }

/* SBtransform (b = Σ DX w φ_m(x) u), src/CubicBSpline.jl:1000-1030, 1107-1111 */
static void spline_sb(const or_spline *s, const double *u, double *b) {
    int Mdim = s->bDim;
    for (int mi = 1; mi <= Mdim; mi++) {
        int m = mi - 2;
        double acc = 0.0;
        for (int mc = 0; mc <= s->nc - 1; mc++) {
            if (mc < m - 2 || mc > m + 1) continue;
            for (int mu = 0; mu < s->mubar; mu++) {
                int i = mu + s->mubar * mc;
                double x = s->xmin + mc * s->DX + s->qpts[mu] * s->DX;
                acc += s->DX * s->qwts[mu] * basis(s, m, x, 0) * u[i];
            }
        }
        b[mi - 1] = acc;
    }
}
int32_t or_spline_sb(const or_spline *s, const double *u, double *b) { spline_sb(s, u, b); return SS_OK; }

/* SAtransform!, src/CubicBSpline.jl:1368-1396 (R3X: b̃ = b − PQ·ahat, a = Γᵀ(..) + ahat) */
static void spline_sa(const or_spline *s, const double *b, const double *ahat, double *a,
                      double *t1, double *t2, double *t3) {
    const double *bb = b;
    int Mdim = s->bDim;
    if (s->r3x) {
        for (int i = 0; i < Mdim; i++) {
            double acc = 0.0;
            for (int j = (i - 3 > 0 ? i - 3 : 0); j <= (i + 3 < Mdim - 1 ? i + 3 : Mdim - 1); j++)
                acc += s->PQb[i * 7 + (j - i + 3)] * (ahat ? ahat[j] : 0.0);
            t1[i] = b[i] - acc;
        }
        bb = t1;
    }
    gamma_apply(s, bb, t2);
    if (s->periodic) dense_solve(s->Ld, s->Min, t2, t3);
    else band_solve3(s->L4, s->Min, t2, t3);
    gamma_adjoint(s, t3, a);
    if (s->r3x && ahat)
        for (int i = 0; i < Mdim; i++) a[i] += ahat[i];
}
int32_t or_spline_sa(const or_spline *s, const double *b, const double *ahat, double *a) {
    double *t = (double *)malloc(sizeof(double) * 3 * (size_t)s->bDim);
    spline_sa(s, b, ahat, a, t, t + s->bDim, t + 2 * s->bDim);
    free(t);
    return SS_OK;
}

/* SItransform at points, src/CubicBSpline.jl:1554-1567 */
static double si_point(const or_spline *s, const double *a, double x, int d) {
    double u = 0.0;
    long xm = (long)ceil((x - s->xmin - (2.0 * s->DX)) * s->DXrecip);
    for (long m = xm; m <= xm + 3; m++)
        if (m >= -1 && m <= s->nc + 1) u += basis(s, (int)m, x, d) * a[m + 1];
    return u;
}
int32_t or_spline_si(const or_spline *s, const double *a, int32_t d, double *u) {
    for (int i = 0; i < s->mishDim; i++) u[i] = si_point(s, a, s->mish[i], d);
    return SS_OK;
}
int32_t or_spline_si_points(const or_spline *s, const double *a, const double *pts, int32_t n,
                            int32_t d, double *u) {
    for (int i = 0; i < n; i++) u[i] = si_point(s, a, pts[i], d);
    return SS_OK;
}
int32_t or_spline_gamma_dense(const or_spline *s, double *G) {
    for (int j = 1; j <= s->Mdim; j++)
        for (int i = 1; i <= s->Min; i++) G[(i - 1) + (size_t)(j - 1) * s->Min] = gamma_at(s, i, j);
    return SS_OK;
}
int32_t or_spline_pq_dense(const or_spline *s, double *PQ) {
    int n = s->bDim;
    memset(PQ, 0, sizeof(double) * (size_t)n * n);
    for (int i = 0; i < n; i++)
        for (int j = (i - 3 > 0 ? i - 3 : 0); j <= (i + 3 < n - 1 ? i + 3 : n - 1); j++)
            PQ[i + (size_t)j * n] = s->PQb[i * 7 + (j - i + 3)];
    return SS_OK;
}
/* set_ahat_r3x! with _border_matrix, src/CubicBSpline.jl:1422-1470 (3×3 solve by Cramer) */
int32_t or_spline_set_ahat_r3x(const or_spline *s, double u0, double u1, double u2,
                               int32_t side, double *ahat) {
    double x = side == 0 ? s->xmin : s->xmax;
    int ms[3];
    if (side == 0) { ms[0] = -1; ms[1] = 0; ms[2] = 1; }
    else { ms[0] = s->nc - 1; ms[1] = s->nc; ms[2] = s->nc + 1; }
    double M[3][3];
    for (int c = 0; c < 3; c++)
        for (int d = 0; d < 3; d++) M[d][c] = basis(s, ms[c], x, d);
    double rhs[3] = {u0, u1, u2};
    double det = M[0][0] * (M[1][1] * M[2][2] - M[1][2] * M[2][1]) - M[0][1] * (M[1][0] * M[2][2] - M[1][2] * M[2][0]) +
                 M[0][2] * (M[1][0] * M[2][1] - M[1][1] * M[2][0]);
    double sol[3];
    for (int c = 0; c < 3; c++) {
        double T[3][3];
        memcpy(T, M, sizeof T);
        for (int d = 0; d < 3; d++) T[d][c] = rhs[d];
        sol[c] = (T[0][0] * (T[1][1] * T[2][2] - T[1][2] * T[2][1]) - T[0][1] * (T[1][0] * T[2][2] - T[1][2] * T[2][0]) +
                  T[0][2] * (T[1][0] * T[2][1] - T[1][1] * T[2][0])) / det;
    }
    int off = side == 0 ? 0 : s->bDim - 3;
    for (int c = 0; c < 3; c++) ahat[off + c] = sol[c];
    return SS_OK;
}

/* ======================================================================
 * Fourier ring (src/Fourier.jl, src/phase_filter.jl)
 * ====================================================================== */

typedef struct {
    int yDim, kmax, bDim;
    double ymin;
    double *cosk, *sink; /* PhaseFilter(fp), src/phase_filter.jl:62-70 */
    const fft_plan *plan;
} or_ring;

static void ring_init(or_ring *rg, int yDim, int kmax, int bDim, double ymin) {
    rg->yDim = yDim; rg->kmax = kmax; rg->bDim = bDim; rg->ymin = ymin;
    rg->cosk = (double *)malloc(sizeof(double) * (size_t)(kmax > 0 ? kmax : 1));
    rg->sink = (double *)malloc(sizeof(double) * (size_t)(kmax > 0 ? kmax : 1));
    for (int k = 1; k <= kmax; k++) {
        rg->cosk[k - 1] = cos(k * ymin);
        rg->sink[k - 1] = sin(k * ymin);
    }
    rg->plan = get_plan(yDim);
}
static void ring_free(or_ring *rg) { free(rg->cosk); free(rg->sink); }

/* FBtransform!, src/Fourier.jl:388-395 + apply_phasefilter_forward!, src/phase_filter.jl:105-143 */
static void ring_fb(const or_ring *rg, const double *u, double *b, double *scr, cplx *buf, cplx *work) {
    int yDim = rg->yDim, kmax = rg->kmax, bDim = rg->bDim;
    r2hc_p(rg->plan, u, scr, buf, work);
    double scale = 1.0 / yDim;
    for (int i = 0; i < yDim; i++) scr[i] *= scale;
    b[0] = scr[0];
    for (int k = 1; k <= kmax; k++) {
        double re = scr[k], im = scr[yDim - k];
        double c = rg->cosk[k - 1], s = rg->sink[k - 1];
        b[k] = c * re + s * im;
        b[bDim - k] = -s * re + c * im;
    }
    if (bDim > 1 + 2 * kmax)
        for (int i = kmax + 1; i <= bDim - kmax - 1; i++) b[i] = 0.0;
}
/* FAtransform!, src/Fourier.jl:429-432 + apply_phasefilter_inverse!, src/phase_filter.jl:154-190 */
static void ring_fa(const or_ring *rg, const double *b, double *a) {
    int yDim = rg->yDim, kmax = rg->kmax, bDim = rg->bDim;
    a[0] = b[0];
    for (int k = 1; k <= kmax; k++) {
        double br = b[k], bi = b[bDim - k];
        double c = rg->cosk[k - 1], s = rg->sink[k - 1];
        a[k] = c * br - s * bi;
        a[yDim - k] = s * br + c * bi;
    }
    for (int i = kmax + 1; i <= yDim - kmax - 1; i++) a[i] = 0.0;
}
/* FIxcoefficients, src/Fourier.jl:495-503 (ax entries beyond kmax stay 0) */
static void ring_fix_coef(int yDim, int kmax, const double *a, double *ax) {
    for (int i = 0; i < yDim; i++) ax[i] = 0.0;
    for (int k = 1; k <= kmax; k++) {
        ax[k] = -k * a[yDim - k];
        ax[yDim - k] = k * a[k];
    }
}
/* FItransform! / FIxtransform / FIxxtransform, src/Fourier.jl:463-468, 540-546, 575-581 */
static void ring_fi(const fft_plan *p, int kmax, const double *a, int d, double *u, double *ax,
                    double *ax2, cplx *buf, cplx *work) {
    int yDim = p->n;
    if (d == 0) { hc2r_p(p, a, u, buf, work); return; }
    ring_fix_coef(yDim, kmax, a, ax);
    if (d == 1) { hc2r_p(p, ax, u, buf, work); return; }
    memcpy(ax2, ax, sizeof(double) * (size_t)yDim);
    ring_fix_coef(yDim, kmax, ax2, ax);
    hc2r_p(p, ax, u, buf, work);
}

static size_t ring_work_len(int yDim) { return fft_work_len(get_plan(yDim)); }

int32_t or_fourier_fb(int32_t yDim, int32_t kmax, int32_t bDim, double ymin, const double *u, double *b) {
    or_ring rg;
    ring_init(&rg, yDim, kmax, bDim, ymin);
    double *scr = (double *)malloc(sizeof(double) * (size_t)yDim);
    cplx *buf = (cplx *)malloc(sizeof(cplx) * (size_t)yDim);
    cplx *work = (cplx *)malloc(sizeof(cplx) * ring_work_len(yDim));
    ring_fb(&rg, u, b, scr, buf, work);
    free(scr); free(buf); free(work); ring_free(&rg);
    return SS_OK;
}
int32_t or_fourier_fa(int32_t yDim, int32_t kmax, int32_t bDim, double ymin, const double *b, double *a) {
    or_ring rg;
    ring_init(&rg, yDim, kmax, bDim, ymin);
    ring_fa(&rg, b, a);
    ring_free(&rg);
    return SS_OK;
}
int32_t or_fourier_fi(int32_t yDim, int32_t kmax, const double *a, int32_t d, double *u) {
    double *ax = (double *)malloc(sizeof(double) * 2 * (size_t)yDim);
    cplx *buf = (cplx *)malloc(sizeof(cplx) * (size_t)yDim);
    cplx *work = (cplx *)malloc(sizeof(cplx) * ring_work_len(yDim));
    ring_fi(get_plan(yDim), kmax, a, d, u, ax, ax + yDim, buf, work);
    free(ax); free(buf); free(work);
    return SS_OK;
}

/* ======================================================================
 * Chebyshev column (src/Chebyshev.jl)
 * ====================================================================== */

typedef struct {
    int N, bDim, bcb, bct;
    double zmin, zmax;
    int gkind;          /* 0: vector γ (scalar broadcast), 1: matrix γ */
    double *gamma;      /* N (vector) or N*N column-major */
    double *filt;       /* bDim diagonal weights (truncation → 1) */
    const double *costab;
} or_cheb;

/* calcGammaBC, src/Chebyshev.jl:991-1177 */
static int cheb_gamma(int N, int bcb, int bct, double **gout, int *is_matrix) {
    double *g;
    if (bcb == SS_CBC_R0 && bct == SS_CBC_R0) {
        g = (double *)calloc((size_t)N, sizeof(double));
        *is_matrix = 0; *gout = g; return SS_OK;
    }
    if (bcb == SS_CBC_R1T0 && bct == SS_CBC_R0) {
        g = (double *)malloc(sizeof(double) * (size_t)N);
        for (int i = 0; i < N; i++) g[i] = 1.0;
        for (int i = 1; i < N - 1; i++) g[i] *= 2.0;
        for (int i = 0; i < N; i++) g[i] *= (-0.5 / (N - 1));
        *is_matrix = 0; *gout = g; return SS_OK;
    }
    g = (double *)calloc((size_t)N * N, sizeof(double));
    *is_matrix = 1; *gout = g;
#define G(i, j) g[(i) + (size_t)(j) * N]
    double *cv = (double *)malloc(sizeof(double) * (size_t)N);
    for (int i = 0; i < N; i++) cv[i] = 1.0;
    cv[0] *= 2.0; cv[N - 1] *= 2.0;
    /* helpers for the component matrices */
    double *B = (double *)calloc((size_t)N * N, sizeof(double)); /* R1T1 bottom */
    double *T = (double *)calloc((size_t)N * N, sizeof(double)); /* R1T1 top */
    double *D = (double *)calloc((size_t)N * N, sizeof(double)); /* R1T0 top (R0/R1T0 form) */
    double *gl = (double *)malloc(sizeof(double) * (size_t)N);    /* R1T0 bottom vector */
    {
        double sf = 0.0;
        for (int i = 0; i < N; i++) { double n = i; sf += -(n * n) / (cv[i] * (N - 1)); }
        for (int i = 0; i < N; i++) {
            double n = i;
            for (int j = 0; j < N; j++) B[i + (size_t)j * N] = n * n / (sf * cv[j] * (N - 1));
        }
    }
    {
        double sf = 0.0;
        for (int i = 0; i < N; i++) {
            double n = i;
            sf += -(n * n) * pow(-1.0, n) * pow(-1.0, n + 1) / (cv[i] * (N - 1));
        }
        for (int i = 0; i < N; i++) {
            double n = i;
            for (int j = 0; j < N; j++)
                T[i + (size_t)j * N] = pow(-1.0, (j + 1) + 1) * pow(-1.0, n + 1) * n * n / (sf * cv[j] * (N - 1));
        }
    }
    for (int i = 0; i < N; i++)
        for (int j = 0; j < N; j++) {
            double v = 1.0;
            v *= -1.0 * pow(-1.0, i) * pow(-1.0, j) / (N - 1);
            D[i + (size_t)j * N] = v;
        }
    for (int j = 0; j < N; j++) { D[0 + (size_t)j * N] *= 0.5; D[(N - 1) + (size_t)j * N] *= 0.5; }
    for (int i = 0; i < N; i++) gl[i] = 1.0;
    for (int i = 1; i < N - 1; i++) gl[i] *= 2.0;
    for (int i = 0; i < N; i++) gl[i] *= (-0.5 / (N - 1));

    int st = SS_OK;
    if (bcb == SS_CBC_R1T1 && bct == SS_CBC_R0) {
        memcpy(g, B, sizeof(double) * (size_t)N * N);
    } else if (bcb == SS_CBC_R0 && bct == SS_CBC_R1T0) {
        memcpy(g, D, sizeof(double) * (size_t)N * N);
    } else if (bcb == SS_CBC_R0 && bct == SS_CBC_R1T1) {
        memcpy(g, T, sizeof(double) * (size_t)N * N);
    } else if (bcb == SS_CBC_R1T0 && bct == SS_CBC_R1T0) {
        /* gammaBC[:,j] += gammaL */
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) G(i, j) = D[i + (size_t)j * N] + gl[i];
    } else if (bcb == SS_CBC_R1T1 && bct == SS_CBC_R1T1) {
        for (size_t q = 0; q < (size_t)N * N; q++) g[q] = B[q] + T[q];
    } else if (bcb == SS_CBC_R1T0 && bct == SS_CBC_R1T1) {
        /* gammaBCB (vector) .+ gammaBCT (matrix): broadcast adds gl[i] to row i */
        for (int i = 0; i < N; i++)
            for (int j = 0; j < N; j++) G(i, j) = gl[i] + T[i + (size_t)j * N];
    } else if (bcb == SS_CBC_R1T1 && bct == SS_CBC_R1T0) {
        for (size_t q = 0; q < (size_t)N * N; q++) g[q] = B[q] + D[q];
    } else {
        set_err("Chebyshev boundary condition combination not implemented (%d,%d)", bcb, bct);
        st = SS_UNSUPPORTED_BC;
    }
#undef G
    free(cv); free(B); free(T); free(D); free(gl);
    if (st != SS_OK) { free(g); *gout = NULL; }
    return st;
}

int32_t or_cheb_gamma(int32_t N, int32_t bcb, int32_t bct, double *G, int32_t *is_matrix) {
    double *g; int ism;
    int st = cheb_gamma(N, bcb, bct, &g, &ism);
    if (st != SS_OK) return st;
    memcpy(G, g, sizeof(double) * (size_t)(ism ? N * N : N));
    *is_matrix = ism;
    free(g);
    return SS_OK;
}

static int cheb_init(or_cheb *c, int N, int bDim, int bcb, int bct, double zmin, double zmax) {
    c->N = N; c->bDim = bDim; c->bcb = bcb; c->bct = bct; c->zmin = zmin; c->zmax = zmax;
    int st = cheb_gamma(N, bcb, bct, &c->gamma, &c->gkind);
    if (st != SS_OK) return st;
    /* calcFilterMatrix, src/Chebyshev.jl:364-378 */
    c->filt = (double *)malloc(sizeof(double) * (size_t)bDim);
    for (int i = 1; i <= bDim; i++)
        c->filt[i - 1] = (bDim < N) ? 1.0 : exp(-36.0 * pow((double)i / N, 36));
    c->costab = get_dct(N);
    return SS_OK;
}
static void cheb_free(or_cheb *c) { free(c->gamma); free(c->filt); }

/* CBtransform!, src/Chebyshev.jl:417-426 */
static void cheb_cb(const or_cheb *c, const double *u, double *b, double *scr) {
    redft00_t(c->costab, u, c->N, scr);
    double scale = 1.0 / (2 * (c->N - 1));
    for (int i = 0; i < c->N; i++) scr[i] *= scale;
    for (int i = 0; i < c->bDim; i++) b[i] = c->filt[i] * scr[i];
}
/* CAtransform!, src/Chebyshev.jl:473-499 */
static void cheb_ca(const or_cheb *c, const double *b, double *a, double *bfill) {
    int N = c->N;
    for (int i = 0; i < c->bDim; i++) bfill[i] = b[i];
    for (int i = c->bDim; i < N; i++) bfill[i] = 0.0;
    if (c->gkind == 1) {
        for (int j = 0; j < N; j++) {
            double acc = 0.0;
            for (int i = 0; i < N; i++) acc += c->gamma[i + (size_t)j * N] * bfill[i];
            a[j] = acc + bfill[j];
        }
    } else {
        double dot = 0.0;
        for (int i = 0; i < N; i++) dot += c->gamma[i] * bfill[i];
        for (int j = 0; j < N; j++) a[j] = bfill[j] + dot;
    }
}
/* CIxcoefficients, src/Chebyshev.jl:636-646 (ax[N] stays 0) */
static void cheb_cix_coef(const or_cheb *c, const double *a, double *ax) {
    int N = c->N;
    ax[N - 1] = 0.0;
    ax[N - 2] = 2.0 * (N - 1) * a[N - 1];
    for (int k = N - 1; k >= 2; k--) ax[k - 2] = (2.0 * (k - 1) * a[k - 1]) + ax[k];
    double sc = -0.5 * (c->zmax - c->zmin);
    for (int i = 0; i < N; i++) ax[i] /= sc;
}
/* CItransform! / CIxtransform / CIxxtransform, src/Chebyshev.jl:530-535, 683-687, 716-722 */
static void cheb_ci(const or_cheb *c, const double *a, int d, double *u, double *ax, double *ax2) {
    if (d == 0) { redft00_t(c->costab, a, c->N, u); return; }
    cheb_cix_coef(c, a, ax);
    if (d == 1) { redft00_t(c->costab, ax, c->N, u); return; }
    memcpy(ax2, ax, sizeof(double) * (size_t)c->N);
    cheb_cix_coef(c, ax2, ax);
    redft00_t(c->costab, ax, c->N, u);
}

int32_t or_cheb_cb(int32_t zDim, int32_t bDim, const double *u, double *b) {
    or_cheb c;
    int st = cheb_init(&c, zDim, bDim, SS_CBC_R0, SS_CBC_R0, 0.0, 1.0);
    if (st) return st;
    double *scr = (double *)malloc(sizeof(double) * (size_t)zDim);
    cheb_cb(&c, u, b, scr);
    free(scr); cheb_free(&c);
    return SS_OK;
}
int32_t or_cheb_ca(int32_t zDim, int32_t bDim, int32_t bcb, int32_t bct, const double *b, double *a) {
    or_cheb c;
    int st = cheb_init(&c, zDim, bDim, bcb, bct, 0.0, 1.0);
    if (st) return st;
    double *bf = (double *)malloc(sizeof(double) * (size_t)zDim);
    cheb_ca(&c, b, a, bf);
    free(bf); cheb_free(&c);
    return SS_OK;
}
int32_t or_cheb_ci(int32_t zDim, double zmin, double zmax, const double *a, int32_t d, double *u) {
    or_cheb c;
    int st = cheb_init(&c, zDim, zDim, SS_CBC_R0, SS_CBC_R0, zmin, zmax);
    if (st) return st;
    double *ax = (double *)malloc(sizeof(double) * 2 * (size_t)zDim);
    cheb_ci(&c, a, d, u, ax, ax + zDim);
    free(ax); cheb_free(&c);
    return SS_OK;
}
/* calcMishPoints, src/Chebyshev.jl:329-343 */
int32_t or_cheb_mish(int32_t N, double zmin, double zmax, double *z) {
    double scale = -0.5 * (zmax - zmin), offset = 0.5 * (zmin + zmax);
    for (int n = 1; n <= N; n++) z[n - 1] = cos((n - 1) * PI / (N - 1)) * scale + offset;
    return SS_OK;
}

/* ======================================================================
 * Grid drivers (src/factory.jl, src/transforms_cylindrical.jl)
 * ====================================================================== */

struct or_grid {
    int geom, nvars, iDim, b, K, pOL, kz, bk, nslots;
    long jDim, np, nspec, nblocks;
    or_spline **spl;    /* per variable (the reference's 3 (or b_kDim) splines per var are identical) */
    or_ring *rings;     /* RL: [v*iDim + r]; RLZ: [r] (shared across z-modes and vars) */
    or_cheb *cols;      /* per variable (RLZ) */
    long *ring_off;     /* physical offset of ring r (RL: Σ L; RLZ: Σ L*kz) */
    double **ahat;      /* per variable: nblocks*b, NULL when not registered */
    int has_ahat;
    double **fw, **cw;  /* filter weights per variable (NULL: none) */
    double *rmish;
    int skip_sa;        /* inverse driver takes spline coefficients a directly */
};

static int ring_L(const or_grid *g, int r) { return 4 + 4 * (r + g->pOL); } /* _cyl_ring_dims, factory.jl:153-156 */

int32_t or_grid_create(const ss_grid_params *p, or_grid **out) {
    *out = NULL;
    if (!p) { set_err("null params"); return SS_BAD_ARG; }
    if (p->geometry != SS_GEOM_RL && p->geometry != SS_GEOM_RLZ) { set_err("geometry must be RL or RLZ"); return SS_BAD_ARG; }
    if (p->nvars < 1 || p->num_cells < 1 || p->mubar < 1 || p->patchOffsetL < 0) { set_err("bad sizes"); return SS_BAD_SHAPE; }
    or_grid *g = (or_grid *)calloc(1, sizeof *g);
    g->geom = p->geometry;
    g->nvars = p->nvars;
    g->iDim = p->num_cells * p->mubar;
    g->b = p->num_cells + 3;
    g->pOL = p->patchOffsetL;
    g->K = g->iDim + g->pOL;
    if (g->geom == SS_GEOM_RLZ) {
        g->kz = p->kDim;
        if (g->kz < 2) { free(g); set_err("RLZ needs kDim >= 2"); return SS_BAD_SHAPE; }
        g->bk = p->b_kDim > 0 ? p->b_kDim : (int)fmin((double)g->kz, floor((2.0 * g->kz - 1) / 3.0) + 1);
        if (g->bk > g->kz || g->bk < 1) { free(g); set_err("b_kDim out of range"); return SS_BAD_SHAPE; }
        g->nslots = 7;
    } else {
        g->kz = 1; g->bk = 1; g->nslots = 5;
    }
    g->jDim = 0;
    g->ring_off = (long *)malloc(sizeof(long) * (size_t)(g->iDim + 1));
    for (int r = 1; r <= g->iDim; r++) {
        g->ring_off[r - 1] = g->jDim * g->kz;
        g->jDim += ring_L(g, r);
    }
    g->ring_off[g->iDim] = g->jDim * g->kz;
    g->np = g->jDim * g->kz;
    g->nblocks = (long)g->bk * (1 + 2L * g->K);
    g->nspec = g->nblocks * g->b;
    g->spl = (or_spline **)calloc((size_t)g->nvars, sizeof(or_spline *));
    int st = SS_OK;
    for (int v = 0; v < g->nvars && st == SS_OK; v++) {
        double lq = p->l_q ? p->l_q[v] : 2.0;
        st = or_spline_create(p->iMin, p->iMax, p->num_cells, p->mubar, p->quadrature, lq,
                              p->BCL ? &p->BCL[v] : NULL, p->BCR ? &p->BCR[v] : NULL, &g->spl[v]);
    }
    if (st != SS_OK) { or_grid_destroy(g); return st; }
    /* rings: _fill_fourier_rings_cyl!, src/factory.jl:608-624 */
    int nr = g->geom == SS_GEOM_RL ? g->nvars * g->iDim : g->iDim;
    g->rings = (or_ring *)calloc((size_t)nr, sizeof(or_ring));
    for (int q = 0; q < nr; q++) {
        int v = g->geom == SS_GEOM_RL ? q / g->iDim : 0;
        int r = q % g->iDim + 1;
        int ri = r + g->pOL;
        int L = 4 + 4 * ri, kmax = ri;
        /* RLZ: rings shared by all variables, var_kmax of src/factory.jl:730-733
           (the caller's resolved value, else the last variable's entry) */
        int var_kmax = -1;
        if (g->geom == SS_GEOM_RL) var_kmax = p->max_wavenumber ? p->max_wavenumber[v] : -1;
        else if (p->ring_kmax_set) var_kmax = p->ring_kmax;
        else if (p->max_wavenumber && g->nvars > 0) var_kmax = p->max_wavenumber[g->nvars - 1];
        if (var_kmax >= 0) kmax = var_kmax < ri ? var_kmax : ri;
        double dl = 2 * PI / L;
        double offset = 0.5 * dl * (ri - 1);
        ring_init(&g->rings[q], L, kmax, ri * 2 + 1, offset);
    }
    if (g->geom == SS_GEOM_RLZ) {
        g->cols = (or_cheb *)calloc((size_t)g->nvars, sizeof(or_cheb));
        for (int v = 0; v < g->nvars && st == SS_OK; v++)
            st = cheb_init(&g->cols[v], g->kz, g->bk, p->BCB ? p->BCB[v] : SS_CBC_R0,
                           p->BCT ? p->BCT[v] : SS_CBC_R0, p->kMin, p->kMax);
        if (st != SS_OK) { or_grid_destroy(g); return st; }
    }
    g->ahat = (double **)calloc((size_t)g->nvars, sizeof(double *));
    g->fw = (double **)calloc((size_t)g->nvars, sizeof(double *));
    g->cw = (double **)calloc((size_t)g->nvars, sizeof(double *));
    g->rmish = (double *)malloc(sizeof(double) * (size_t)g->iDim);
    spline_mish(g->spl[0], g->rmish);
    *out = g;
    return SS_OK;
}

void or_grid_destroy(or_grid *g) {
    if (!g) return;
    if (g->spl) for (int v = 0; v < g->nvars; v++) or_spline_destroy(g->spl[v]);
    free(g->spl);
    if (g->rings) {
        int nr = g->geom == SS_GEOM_RL ? g->nvars * g->iDim : g->iDim;
        for (int q = 0; q < nr; q++) ring_free(&g->rings[q]);
    }
    free(g->rings);
    if (g->cols) for (int v = 0; v < g->nvars; v++) cheb_free(&g->cols[v]);
    free(g->cols);
    if (g->ahat) for (int v = 0; v < g->nvars; v++) free(g->ahat[v]);
    if (g->fw) for (int v = 0; v < g->nvars; v++) free(g->fw[v]);
    if (g->cw) for (int v = 0; v < g->nvars; v++) free(g->cw[v]);
    free(g->ahat); free(g->fw); free(g->cw);
    free(g->ring_off); free(g->rmish);
    free(g);
}

int32_t or_grid_dims(const or_grid *g, ss_dims *d) {
    d->iDim = g->iDim; d->b_iDim = g->b; d->jDim = g->jDim;
    long bj = 0;
    for (int r = 1; r <= g->iDim; r++) bj += 1 + 2L * (r + g->pOL);
    d->b_jDim = bj;
    d->kDim = g->kz; d->b_kDim = g->bk; d->kDim_wn = g->K; d->nvars = g->nvars;
    d->nslots = g->nslots; d->n_physical = g->np; d->n_spectral = g->nspec; d->n_blocks = g->nblocks;
    return SS_OK;
}

int32_t or_grid_set_ahat(or_grid *g, int32_t v, int32_t block, const double *ahat) {
    if (v < 0 || v >= g->nvars || block < 0 || block >= g->nblocks) { set_err("ahat index out of range"); return SS_BAD_ARG; }
    if (!g->ahat[v]) g->ahat[v] = (double *)calloc((size_t)g->nblocks * g->b, sizeof(double));
    memcpy(g->ahat[v] + (size_t)block * g->b, ahat, sizeof(double) * (size_t)g->b);
    g->has_ahat = 1;
    return SS_OK;
}
int32_t or_grid_set_filter(or_grid *g, int32_t v, const double *fw, const double *cw) {
    if (v < 0 || v >= g->nvars) { set_err("var out of range"); return SS_BAD_ARG; }
    free(g->fw[v]); g->fw[v] = NULL;
    free(g->cw[v]); g->cw[v] = NULL;
    if (fw) { g->fw[v] = (double *)malloc(sizeof(double) * (size_t)(g->K + 1)); memcpy(g->fw[v], fw, sizeof(double) * (size_t)(g->K + 1)); }
    if (cw) { g->cw[v] = (double *)malloc(sizeof(double) * (size_t)g->bk); memcpy(g->cw[v], cw, sizeof(double) * (size_t)g->bk); }
    return SS_OK;
}

/* getGridpoints RL :75-90, RLZ :454-476 */
int32_t or_grid_points(const or_grid *g, double *out) {
    long np = g->np;
    double *zm = NULL;
    if (g->geom == SS_GEOM_RLZ) { zm = (double *)malloc(sizeof(double) * (size_t)g->kz); or_cheb_mish(g->kz, g->cols[0].zmin, g->cols[0].zmax, zm); }
    long q = 0;
    for (int r = 1; r <= g->iDim; r++) {
        const or_ring *rg = &g->rings[r - 1];
        for (int l = 1; l <= rg->yDim; l++) {
            double lam = rg->ymin + (2 * PI * (l - 1) / rg->yDim);
            for (int z = 0; z < g->kz; z++) {
                out[q] = g->rmish[r - 1];
                out[q + np] = lam;
                if (zm) out[q + 2 * np] = zm[z];
                q++;
            }
        }
    }
    free(zm);
    return SS_OK;
}
int32_t or_grid_radial_points(const or_grid *g, double *out) { memcpy(out, g->rmish, sizeof(double) * (size_t)g->iDim); return SS_OK; }
int32_t or_grid_ring_points(const or_grid *g, int32_t r, double *out) {
    if (r < 1 || r > g->iDim) { set_err("ring out of range"); return SS_BAD_ARG; }
    const or_ring *rg = &g->rings[r - 1];
    for (int l = 1; l <= rg->yDim; l++) out[l - 1] = rg->ymin + (2 * PI * (l - 1) / rg->yDim); /* src/Fourier.jl:337-346 */
    return SS_OK;
}
int32_t or_grid_column_points(const or_grid *g, double *out) {
    if (g->geom != SS_GEOM_RLZ) { set_err("RL grid has no columns"); return SS_BAD_ARG; }
    return or_cheb_mish(g->kz, g->cols[0].zmin, g->cols[0].zmax, out);
}
int32_t or_grid_factor(const or_grid *g, int32_t v, double *L4, int32_t *n_out) {
    const or_spline *s = g->spl[v];
    memcpy(L4, s->L4, sizeof(double) * 4 * (size_t)s->Min);
    *n_out = s->Min;
    return SS_OK;
}

/* applyFilter! RL :320-364 / RLZ :372-428 (weights precomputed by the host;
 * a weight ≈ 1 is skipped, ≈ 0 zeroes the block, as the reference does) */
static void apply_filter(or_grid *g, int v, double *spec) {
    if (!g->fw[v] && !g->cw[v]) return;
    long slots = 1 + 2L * g->K;
    for (int zb = 0; zb < g->bk; zb++) {
        double cwt = g->cw[v] ? g->cw[v][zb] : 1.0;
        for (long s = 0; s < slots; s++) {
            int k = (int)((s + 1) / 2);
            double w = cwt * (g->fw[v] ? g->fw[v][k] : 1.0);
            if (w == 1.0) continue;
            double *blk = spec + ((size_t)zb * slots + s) * g->b;
            for (int m = 0; m < g->b; m++) blk[m] = (w == 0.0) ? 0.0 : blk[m] * w;
        }
    }
}

typedef struct {
    double *scr, *u, *b, *ax, *ax2, *t;
    cplx *buf, *work;
} or_ws;
static void ws_alloc(or_ws *w, long maxL, size_t wl, int b, int kz) {
    long n = maxL > 4L * b ? maxL : 4L * b;
    if (n < 4L * kz) n = 4L * kz;
    w->scr = (double *)malloc(sizeof(double) * (size_t)n);
    w->u = (double *)malloc(sizeof(double) * (size_t)n);
    w->b = (double *)malloc(sizeof(double) * (size_t)n);
    w->ax = (double *)malloc(sizeof(double) * (size_t)n);
    w->ax2 = (double *)malloc(sizeof(double) * (size_t)n);
    w->t = (double *)malloc(sizeof(double) * (size_t)n * 3);
    w->buf = (cplx *)malloc(sizeof(cplx) * (size_t)n);
    w->work = (cplx *)malloc(sizeof(cplx) * (wl > (size_t)n ? wl : (size_t)n));
}
static void ws_free(or_ws *w) {
    free(w->scr); free(w->u); free(w->b); free(w->ax); free(w->ax2); free(w->t); free(w->buf); free(w->work);
}
static size_t max_work(const or_grid *g) {
    size_t m = 0;
    for (int r = 1; r <= g->iDim; r++) { size_t w = fft_work_len(g->rings[r - 1].plan); if (w > m) m = w; }
    return m;
}

/* spectralTransform (RL), src/transforms_cylindrical.jl:159-222
 * spectralTransform (RLZ), src/transforms_cylindrical.jl:530-618
 * The per-ring and per-column work items are independent; they run in
 * parallel over rings/columns (the reference runs them in order). */
int32_t or_spectral_transform(or_grid *g, const double *phys, double *spec) {
    int iDim = g->iDim, b = g->b, K = g->K, bk = g->bk, kz = g->kz;
    long slots = 1 + 2L * K;
    long maxL = ring_L(g, iDim);
    size_t wl = max_work(g);
    /* ringb[v][zb][r][k]: ring B-coefficients (bDim = 2ri+1 per ring) */
    for (int v = 0; v < g->nvars; v++) {
        const double *ph = phys + (size_t)g->np * v;
        double *sp = spec + (size_t)g->nspec * v;
        /* per ring r and z-mode: b vector of length 2ri+1 */
        double **rb = (double **)malloc(sizeof(double *) * (size_t)iDim * bk);
#pragma omp parallel num_threads(g_threads)
        {
            or_ws w;
            ws_alloc(&w, maxL, wl, b, kz);
            double *tempcb = (double *)malloc(sizeof(double) * (size_t)bk * maxL);
#pragma omp for schedule(dynamic, 1)
            for (int r = 1; r <= iDim; r++) {
                int ri = r + g->pOL;
                int L = 4 + 4 * ri;
                int bD = 2 * ri + 1;
                const or_ring *rg = g->geom == SS_GEOM_RL ? &g->rings[(size_t)v * iDim + r - 1] : &g->rings[r - 1];
                const double *seg = ph + g->ring_off[r - 1];
                if (g->geom == SS_GEOM_RL) {
                    double *bb = (double *)malloc(sizeof(double) * (size_t)bD);
                    ring_fb(rg, seg, bb, w.scr, w.buf, w.work);
                    rb[r - 1] = bb;
                } else {
                    const or_cheb *col = &g->cols[v];
                    for (int l = 0; l < L; l++) {
                        cheb_cb(col, seg + (size_t)l * kz, w.b, w.scr);
                        for (int k = 0; k < bk; k++) tempcb[(size_t)k * L + l] = w.b[k];
                    }
                    for (int zb = 0; zb < bk; zb++) {
                        double *bb = (double *)malloc(sizeof(double) * (size_t)bD);
                        ring_fb(rg, tempcb + (size_t)zb * L, bb, w.scr, w.buf, w.work);
                        rb[(size_t)zb * iDim + r - 1] = bb;
                    }
                }
            }
            free(tempcb);
            ws_free(&w);
        }
        /* spline stage per (z_b, slot) */
        const or_spline *s = g->spl[v];
#pragma omp parallel num_threads(g_threads)
        {
            double *um = (double *)malloc(sizeof(double) * (size_t)iDim);
            double *bv = (double *)malloc(sizeof(double) * (size_t)b);
#pragma omp for schedule(static)
            for (long q = 0; q < (long)bk * slots; q++) {
                int zb = (int)(q / slots);
                long sl = q % slots;
                int k = (int)((sl + 1) / 2);
                for (int r = 1; r <= iDim; r++) {
                    double val = 0.0;
                    const double *bb = rb[(size_t)zb * iDim + r - 1];
                    int ri = r + g->pOL;
                    if (sl == 0) val = bb[0];
                    else if (k <= ri) val = (sl & 1) ? bb[k] : bb[(2 * ri + 1) - k];
                    um[r - 1] = val;
                }
                spline_sb(s, um, bv);
                memcpy(sp + ((size_t)zb * slots + sl) * b, bv, sizeof(double) * (size_t)b);
            }
            free(um); free(bv);
        }
        for (long q = 0; q < (long)iDim * bk; q++) free(rb[q]);
        free(rb);
        apply_filter(g, v, sp);
    }
    return SS_OK;
}

/* gridTransform (RL), src/transforms_cylindrical.jl:259-428
 * gridTransform (RLZ), src/transforms_cylindrical.jl:659-853 (the SA solve,
 * repeated per dr there, is done once: identical inputs give identical a). */
int32_t or_grid_transform(or_grid *g, const double *spec, double *phys) {
    int iDim = g->iDim, b = g->b, K = g->K, bk = g->bk, kz = g->kz;
    long slots = 1 + 2L * K;
    long maxL = ring_L(g, iDim);
    size_t wl = max_work(g);
    long np = g->np;
    int nv = g->nvars;
    for (int v = 0; v < nv; v++) {
        const double *sp = spec + (size_t)g->nspec * v;
        const or_spline *s = g->spl[v];
        /* prof[d][zb][slot][r]: spline value / ∂r / ∂rr per slot at each radius */
        size_t psz = (size_t)bk * slots * iDim;
        double *prof = (double *)malloc(sizeof(double) * psz * 3);
#pragma omp parallel num_threads(g_threads)
        {
            double *a = (double *)malloc(sizeof(double) * (size_t)b);
            double *t = (double *)malloc(sizeof(double) * 3 * (size_t)b);
#pragma omp for schedule(static)
            for (long q = 0; q < (long)bk * slots; q++) {
                const double *ah = (g->has_ahat && g->ahat[v]) ? g->ahat[v] + (size_t)q * b : NULL;
                if (g->skip_sa) memcpy(a, sp + (size_t)q * b, sizeof(double) * (size_t)b);
                else spline_sa(s, sp + (size_t)q * b, ah, a, t, t + b, t + 2 * b);
                for (int d = 0; d < 3; d++)
                    for (int r = 0; r < iDim; r++)
                        prof[(size_t)d * psz + (size_t)q * iDim + r] = si_point(s, a, s->mish[r], d);
            }
            free(a); free(t);
        }
        /* rings */
#pragma omp parallel num_threads(g_threads)
        {
            or_ws w;
            ws_alloc(&w, maxL, wl, b, kz);
            /* RLZ: ring outputs for the 5 variants, [var][zb][l] */
            double *rbuf = (double *)malloc(sizeof(double) * (size_t)5 * bk * maxL);
            double *ca = (double *)malloc(sizeof(double) * (size_t)kz * 4);
#pragma omp for schedule(dynamic, 1)
            for (int r = 1; r <= iDim; r++) {
                int ri = r + g->pOL;
                int L = 4 + 4 * ri;
                int bD = 2 * ri + 1;
                const or_ring *rg = g->geom == SS_GEOM_RL ? &g->rings[(size_t)v * iDim + r - 1] : &g->rings[r - 1];
                for (int zb = 0; zb < bk; zb++) {
                    for (int d = 0; d < 3; d++) {
                        /* ring b from spline (d = 0 value, 1 ∂r, 2 ∂rr) */
                        const double *pd = prof + (size_t)d * psz + (size_t)zb * slots * iDim;
                        w.b[0] = pd[r - 1];
                        for (int k = 1; k <= K; k++) {
                            if (k <= ri) {
                                w.b[k] = pd[(size_t)(2 * k - 1) * iDim + r - 1];
                                w.b[bD - k] = pd[(size_t)(2 * k) * iDim + r - 1];
                            }
                        }
                        ring_fa(rg, w.b, w.scr); /* a (length L) */
                        if (d == 0) {
                            for (int dl = 0; dl < 3; dl++) {
                                double *dst;
                                if (g->geom == SS_GEOM_RL) {
                                    int slot = dl == 0 ? 1 : (dl == 1 ? 4 : 5);
                                    dst = phys + np * ((size_t)v + (size_t)nv * (slot - 1)) + g->ring_off[r - 1];
                                } else {
                                    int var = dl == 0 ? 0 : (dl == 1 ? 1 : 2);
                                    dst = rbuf + ((size_t)var * bk + zb) * L;
                                }
                                ring_fi(rg->plan, rg->kmax, w.scr, dl, dst, w.ax, w.ax2, w.buf, w.work);
                            }
                        } else {
                            double *dst;
                            if (g->geom == SS_GEOM_RL) {
                                int slot = d == 1 ? 2 : 3;
                                dst = phys + np * ((size_t)v + (size_t)nv * (slot - 1)) + g->ring_off[r - 1];
                            } else {
                                int var = d == 1 ? 3 : 4;
                                dst = rbuf + ((size_t)var * bk + zb) * L;
                            }
                            ring_fi(rg->plan, rg->kmax, w.scr, 0, dst, w.ax, w.ax2, w.buf, w.work);
                        }
                    }
                }
                if (g->geom == SS_GEOM_RLZ) {
                    const or_cheb *col = &g->cols[v];
                    /* variants: 0 (dr0 dl0) → slots 1,6,7; 1 → 4; 2 → 5; 3 (dr1) → 2; 4 (dr2) → 3 */
                    for (int var = 0; var < 5; var++) {
                        for (int l = 0; l < L; l++) {
                            for (int zb = 0; zb < bk; zb++) w.b[zb] = rbuf[((size_t)var * bk + zb) * L + l];
                            cheb_ca(col, w.b, ca, w.scr);
                            long off = g->ring_off[r - 1] + (long)l * kz;
                            if (var == 0) {
                                cheb_ci(col, ca, 0, phys + np * ((size_t)v + 0 * (size_t)nv) + off, w.ax, w.ax2);
                                cheb_ci(col, ca, 1, phys + np * ((size_t)v + 5 * (size_t)nv) + off, w.ax, w.ax2);
                                cheb_ci(col, ca, 2, phys + np * ((size_t)v + 6 * (size_t)nv) + off, w.ax, w.ax2);
                            } else {
                                int slot = var == 1 ? 4 : (var == 2 ? 5 : (var == 3 ? 2 : 3));
                                cheb_ci(col, ca, 0, phys + np * ((size_t)v + (size_t)nv * (slot - 1)) + off, w.ax, w.ax2);
                            }
                        }
                    }
                }
            }
            free(rbuf); free(ca);
            ws_free(&w);
        }
        free(prof);
    }
    return SS_OK;
}

/* ======================================================================
 * RL / RLZ multi-patch chain (src/multipatch.jl)
 * ====================================================================== */

typedef struct {
    int primary, secondary;     /* patch indices */
    int pside, sside;           /* 0 = left, 1 = right */
    double C[9];                /* 3×3 coupling matrix, row-major */
    int node[3];                /* 0-based indices into the primary's a */
} or_iface;

struct or_chain {
    int n;
    or_grid **g;
    int nif;
    or_iface *ifs;
    int nlayers;
    int *layer_of;              /* patch → topological layer */
    double **state;             /* per patch: nvars × 3 × b (spline objects k0, real, imag .ahat) */
};
typedef struct or_chain or_chain;

/* _build_coupling_matrix, src/multipatch.jl:42-53 (COUPLING_MATRIX_1X / _2X :21-33) */
static int coupling_matrix(double pDX, double sDX, double *C) {
    double ratio = pDX / sDX, tol = 1e-12 * (pDX > sDX ? pDX : sDX);
    static const double M1[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    static const double M2[9] = {0.5, 0.5, 0.0, 0.125, 0.75, 0.125, 0.0, 0.5, 0.5};
    if (fabs(ratio - 1.0) < tol) { memcpy(C, M1, sizeof M1); return SS_OK; }
    if (fabs(ratio - 2.0) < tol) { memcpy(C, M2, sizeof M2); return SS_OK; }
    set_err("Only 1:1 and 2:1 coarse-to-fine ratios are supported, got %g:1", ratio);
    return SS_BAD_ARG;
}

/* PatchChain (src/multipatch.jl:825-848) + _topological_sort (:666-724) */
int32_t or_chain_create(or_grid **grids, int32_t n, or_chain **out) {
    *out = NULL;
    if (n < 2) { set_err("PatchChain requires at least 2 grids, got %d", n); return SS_BAD_ARG; }
    for (int k = 0; k < n; k++)
        if (grids[k]->geom != grids[0]->geom || grids[k]->nvars != grids[0]->nvars ||
            (grids[0]->geom == SS_GEOM_RLZ && grids[k]->bk != grids[0]->bk)) {
            set_err("the chain supports RL or RLZ patches with equal variable counts (and Chebyshev modes)");
            return SS_BAD_ARG;
        }
    or_chain *c = (or_chain *)calloc(1, sizeof *c);
    c->n = n;
    c->g = (or_grid **)malloc(sizeof(or_grid *) * (size_t)n);
    memcpy(c->g, grids, sizeof(or_grid *) * (size_t)n);
    c->nif = n - 1;
    c->ifs = (or_iface *)calloc((size_t)(n - 1), sizeof(or_iface));
    for (int k = 0; k < n - 1; k++) {
        const or_spline *L = grids[k]->spl[0], *R = grids[k + 1]->spl[0];
        or_iface *f = &c->ifs[k];
        if (L->DX >= R->DX) { f->primary = k; f->secondary = k + 1; f->pside = 1; f->sside = 0; }
        else { f->primary = k + 1; f->secondary = k; f->pside = 0; f->sside = 1; }
        const or_spline *P = grids[f->primary]->spl[0], *S = grids[f->secondary]->spl[0];
        int st = coupling_matrix(P->DX, S->DX, f->C);
        if (st) { free(c->ifs); free(c->g); free(c); return st; }
        for (int v = 0; v < grids[0]->nvars; v++)
            if (!grids[f->secondary]->spl[v]->r3x || grids[f->primary]->spl[v]->r3x) {
                set_err("chain interface %d: secondary needs R3X and primary must not be R3X", k);
                free(c->ifs); free(c->g); free(c);
                return SS_UNSUPPORTED_BC;
            }
        /* hollow nest node indices (src/multipatch.jl:290-316) */
        int b = P->bDim;
        if (f->pside == 1) { f->node[0] = b - 3; f->node[1] = b - 2; f->node[2] = b - 1; }
        else { f->node[0] = 0; f->node[1] = 1; f->node[2] = 2; }
    }
    c->layer_of = (int *)calloc((size_t)n, sizeof(int));
    /* Kahn layers: a secondary sits one layer after its latest primary */
    int changed = 1, guard = 0;
    while (changed && guard++ < n + 2) {
        changed = 0;
        for (int i = 0; i < c->nif; i++) {
            int need = c->layer_of[c->ifs[i].primary] + 1;
            if (c->layer_of[c->ifs[i].secondary] < need) { c->layer_of[c->ifs[i].secondary] = need; changed = 1; }
        }
    }
    c->nlayers = 0;
    for (int i = 0; i < n; i++) if (c->layer_of[i] + 1 > c->nlayers) c->nlayers = c->layer_of[i] + 1;
    c->state = (double **)calloc((size_t)n, sizeof(double *));
    for (int i = 0; i < n; i++)
        c->state[i] = (double *)calloc((size_t)grids[i]->nvars * 3 * grids[i]->b, sizeof(double));
    *out = c;
    return SS_OK;
}

/* PatchEmbedded (src/multipatch.jl:891-925): grids nested outermost first; each
 * inner grid takes R3X data from its parent at both ends through stacked
 * interfaces (the parent's node at the inner boundary, :190-207, 270-276),
 * pushed right-of-inner-left first, then its right end. */
int32_t or_chain_create_embedded(or_grid **grids, int32_t n, or_chain **out) {
    *out = NULL;
    if (n < 2) { set_err("PatchEmbedded requires at least 2 grids, got %d", n); return SS_BAD_ARG; }
    for (int k = 0; k < n; k++)
        if (grids[k]->geom != grids[0]->geom || grids[k]->nvars != grids[0]->nvars ||
            (grids[0]->geom == SS_GEOM_RLZ && grids[k]->bk != grids[0]->bk)) {
            set_err("embedded patches must share geometry, variable count (and Chebyshev modes)");
            return SS_BAD_ARG;
        }
    or_chain *c = (or_chain *)calloc(1, sizeof *c);
    c->n = n;
    c->g = (or_grid **)malloc(sizeof(or_grid *) * (size_t)n);
    memcpy(c->g, grids, sizeof(or_grid *) * (size_t)n);
    c->nif = 2 * (n - 1);
    c->ifs = (or_iface *)calloc((size_t)c->nif, sizeof(or_iface));
    for (int k = 1; k < n; k++) {
        const or_spline *P = grids[k - 1]->spl[0], *S = grids[k]->spl[0];
        if (fabs(P->DX / S->DX - 1.0) < 1e-12 * (P->DX > S->DX ? P->DX : S->DX)) {
            set_err("PatchEmbedded requires refinement at each level (grids %d and %d have DX=%g)", k, k + 1, P->DX);
            free(c->ifs); free(c->g); free(c);
            return SS_BAD_ARG;
        }
        for (int side = 0; side < 2; side++) {
            or_iface *f = &c->ifs[2 * (k - 1) + side];
            f->primary = k - 1;
            f->secondary = k;
            f->pside = side == 0 ? 1 : 0;  /* (outer, inner, :right, :left), then (:left, :right) */
            f->sside = side == 0 ? 0 : 1;
            int st = coupling_matrix(P->DX, S->DX, f->C);
            if (st) { free(c->ifs); free(c->g); free(c); return st; }
            for (int v = 0; v < grids[0]->nvars; v++)
                if (!grids[k]->spl[v]->r3x) {
                    set_err("embedded grid %d needs R3X (FixedBC) at both ends", k + 1);
                    free(c->ifs); free(c->g); free(c);
                    return SS_UNSUPPORTED_BC;
                }
            const double xb = f->sside == 0 ? S->xmin : S->xmax;
            const long m = lround((xb - P->xmin) / P->DX);
            const double xn = P->xmin + (double)m * P->DX;
            if (fabs(xn - xb) > 1e-12 * P->DX || m + 1 < 1 || m + 1 > P->bDim - 2) {
                set_err("inner boundary %g does not align with a node of its parent", xb);
                free(c->ifs); free(c->g); free(c);
                return SS_BAD_ARG;
            }
            /* node index m + 2 (1-based) and its neighbours, 0-based */
            f->node[0] = (int)m; f->node[1] = (int)m + 1; f->node[2] = (int)m + 2;
        }
    }
    c->layer_of = (int *)calloc((size_t)n, sizeof(int));
    for (int i = 0; i < n; i++) c->layer_of[i] = i;  /* outer → inner */
    c->nlayers = n;
    c->state = (double **)calloc((size_t)n, sizeof(double *));
    for (int i = 0; i < n; i++)
        c->state[i] = (double *)calloc((size_t)grids[i]->nvars * 3 * grids[i]->b, sizeof(double));
    *out = c;
    return SS_OK;
}

void or_chain_destroy(or_chain *c) {
    if (!c) return;
    for (int i = 0; i < c->n; i++) free(c->state[i]);
    free(c->state); free(c->layer_of); free(c->ifs); free(c->g); free(c);
}

/* _rl_kernel! (src/multipatch.jl:417-478) and _rlz_kernel! (:496-571): SA of
 * each primary wavenumber slot (RLZ: of every Chebyshev level z_b, blocks
 * z_b·(1+2K) + q), 3 interface coefficients × coupling matrix, written into
 * the secondary spline object's ahat (the k0 / real / imag objects are shared
 * by all wavenumbers and levels) and the whole ahat vector copied into the
 * per-wavenumber registry slot (src/multipatch_registry.jl:45-62). */
static void chain_update_interface(or_chain *c, const or_iface *f, const double *spec_p) {
    or_grid *P = c->g[f->primary], *S = c->g[f->secondary];
    int bp = P->b, bs = S->b;
    int Kp = P->K, Ks = S->K, Kc = Kp < Ks ? Kp : Ks;
    int nz = P->geom == SS_GEOM_RLZ ? P->bk : 1;
    double *a = (double *)malloc(sizeof(double) * (size_t)bp);
    double *t = (double *)malloc(sizeof(double) * 3 * (size_t)bp);
    for (int v = 0; v < S->nvars; v++) {
        const double *sp = spec_p + (size_t)P->nspec * v;
        for (int zb = 0; zb < nz; zb++)
            for (int q = 0; q <= 2 * Kc; q++) {
                /* q: 0 = k0, odd = real k=(q+1)/2, even = imag */
                int obj = (q == 0) ? 0 : ((q & 1) ? 1 : 2);
                /* SAtransform!(primary spline object): an R3X primary (an inner grid of an
                 * embedded multigrid) solves with that object's current background */
                const double *pah = P->spl[v]->r3x ? c->state[f->primary] + ((size_t)v * 3 + obj) * bp : NULL;
                spline_sa(P->spl[v], sp + ((size_t)zb * (1 + 2 * Kp) + q) * bp, pah, a, t, t + bp, t + 2 * bp);
                double ex[3] = {a[f->node[0]], a[f->node[1]], a[f->node[2]]};
                double *st = c->state[f->secondary] + ((size_t)v * 3 + obj) * bs;
                double *dst = (f->sside == 0) ? st : st + bs - 3;
                for (int r = 0; r < 3; r++) dst[r] = f->C[r * 3] * ex[0] + f->C[r * 3 + 1] * ex[1] + f->C[r * 3 + 2] * ex[2];
                or_grid_set_ahat(S, v, zb * (1 + 2 * Ks) + q, st);
            }
    }
    free(a); free(t);
}

/* multiGridTransform! (src/multipatch.jl:769-786) */
int32_t or_multi_grid_transform(or_chain *c, const double **spectral, double **physical) {
    for (int L = 0; L < c->nlayers; L++) {
        for (int i = 0; i < c->n; i++)
            if (c->layer_of[i] == L) {
                int st = or_grid_transform(c->g[i], spectral[i], physical[i]);
                if (st) return st;
            }
        for (int k = 0; k < c->nif; k++)
            if (c->layer_of[c->ifs[k].primary] == L) chain_update_interface(c, &c->ifs[k], spectral[c->ifs[k].primary]);
    }
    return SS_OK;
}

/* ======================================================================
 * Elliptic per-wavenumber solve on RL grids
 * (∂rr + (1/r)∂r + (1/r²)∂λλ − k²(r)) u = f
 *
 * The reference has no RL elliptic solve (its Kron assembly uses ring 1 only,
 * src/solver.jl:354-359).  Per Fourier wavenumber m the radial problem
 *   u_m'' + u_m'/r − (m²/r² + k²(r)) u_m = f_m
 * is discretised with the reference's own pieces: the B-spline values and
 * derivatives at the mish points (spline_basis_matrix / _1st_ / _2nd_,
 * src/CubicBSpline.jl:1729-1816), tested with the SB projection weights
 * (_build_sb_matrix, :1000-1030, the same Galerkin form as the P+Q system),
 * and the Γ fold of the boundary conditions (src/solver.jl:721-756):
 *   G_m = Γ_m [Σ_i w_{·,i} (Lφ_j)(r_i)] Γ_mᵀ,  G_m x = Γ_m b_m,  a = Γ_mᵀ x
 * where b_m is the spectral B-vector of f (spectralTransform!).  Axis
 * regularity: u_0'(0) = 0 (R1T1), u_m(0) = 0 for m ≥ 1 (R1T0); u(R) = 0
 * (R1T0) at the outer edge.  Direct solve: dense LU with partial pivoting.
 * ====================================================================== */

struct or_elliptic {
    or_grid *g;
    or_spline *s0, *s1;   /* m = 0 and m ≥ 1 templates (Γ differs) */
    double *k2;           /* k²(r) at the mish points */
};
typedef struct or_elliptic or_elliptic;

int32_t or_elliptic_create(or_grid *g, const double *k2, or_elliptic **out) {
    *out = NULL;
    if (g->geom != SS_GEOM_RL) { set_err("the elliptic solve needs an RL grid"); return SS_BAD_ARG; }
    const or_spline *t = g->spl[0];
    ss_spline_bc r1t0 = {SS_SBC_RANK1, 0, -4.0, -1.0}, r1t1 = {SS_SBC_RANK1, 0, 0.0, 1.0};
    or_elliptic *e = (or_elliptic *)calloc(1, sizeof *e);
    e->g = g;
    int st = or_spline_create(t->xmin, t->xmax, t->nc, t->mubar, t->quad, t->l_q, &r1t1, &r1t0, &e->s0);
    if (st == SS_OK) st = or_spline_create(t->xmin, t->xmax, t->nc, t->mubar, t->quad, t->l_q, &r1t0, &r1t0, &e->s1);
    if (st) { or_spline_destroy(e->s0); free(e); return st; }
    e->k2 = (double *)malloc(sizeof(double) * (size_t)t->mishDim);
    memcpy(e->k2, k2, sizeof(double) * (size_t)t->mishDim);
    *out = e;
    return SS_OK;
}
void or_elliptic_destroy(or_elliptic *e) {
    if (!e) return;
    or_spline_destroy(e->s0); or_spline_destroy(e->s1); free(e->k2); free(e);
}

/* dense G_m (Min × Min, column-major) */
int32_t or_elliptic_operator(const or_elliptic *e, int32_t m, double *G, int32_t *n_out) {
    const or_spline *s = m == 0 ? e->s0 : e->s1;
    int b = s->bDim, n = s->Min;
    double *Gf = (double *)calloc((size_t)b * b, sizeof(double));
    for (int mc = 0; mc < s->nc; mc++)
        for (int mu = 0; mu < s->mubar; mu++) {
            int i = mu + s->mubar * mc;
            double x = s->mish[i];
            double m2 = (double)m * (double)m;
            double c1 = 1.0 / x, c0 = -(m2 / (x * x) + e->k2[i]);
            long xm = (long)ceil((x - s->xmin - (2.0 * s->DX)) * s->DXrecip);
            for (long jj = xm; jj <= xm + 3; jj++) {
                if (jj < -1 || jj > s->nc + 1) continue;
                double Lphi = basis(s, (int)jj, x, 2) + c1 * basis(s, (int)jj, x, 1) + c0 * basis(s, (int)jj, x, 0);
                for (int ti = (mc - 1 > -1 ? mc - 1 : -1); ti <= mc + 2; ti++) {
                    if (ti < -1 || ti > s->nc + 1) continue;
                    double w = s->DX * s->qwts[mu] * basis(s, ti, x, 0);
                    Gf[(ti + 1) + (size_t)(jj + 1) * b] += w * Lphi;
                }
            }
        }
    /* G = Γ Gf Γᵀ */
    for (int c = 1; c <= n; c++)
        for (int r = 1; r <= n; r++) {
            double acc = 0.0;
            for (int a = 1; a <= b; a++) {
                double ga = gamma_at(s, r, a);
                if (ga == 0.0) continue;
                for (int bb = 1; bb <= b; bb++) {
                    double gb = gamma_at(s, c, bb);
                    if (gb == 0.0) continue;
                    acc += ga * Gf[(a - 1) + (size_t)(bb - 1) * b] * gb;
                }
            }
            G[(r - 1) + (size_t)(c - 1) * n] = acc;
        }
    free(Gf);
    *n_out = n;
    return SS_OK;
}

static int dense_lu_solve(double *A, int n, double *x) {
    /* in place LU with partial pivoting, then the solve of A x = x */
    for (int k = 0; k < n; k++) {
        int p = k;
        double mx = fabs(A[k + (size_t)k * n]);
        for (int i = k + 1; i < n; i++)
            if (fabs(A[i + (size_t)k * n]) > mx) { mx = fabs(A[i + (size_t)k * n]); p = i; }
        if (mx == 0.0) { set_err("singular operator"); return SS_NOT_SPD; }
        if (p != k) {
            for (int j = 0; j < n; j++) { double t = A[k + (size_t)j * n]; A[k + (size_t)j * n] = A[p + (size_t)j * n]; A[p + (size_t)j * n] = t; }
            double t = x[k]; x[k] = x[p]; x[p] = t;
        }
        for (int i = k + 1; i < n; i++) {
            double l = A[i + (size_t)k * n] / A[k + (size_t)k * n];
            A[i + (size_t)k * n] = l;
            for (int j = k + 1; j < n; j++) A[i + (size_t)j * n] -= l * A[k + (size_t)j * n];
            x[i] -= l * x[k];
        }
    }
    for (int i = n - 1; i >= 0; i--) {
        double s = x[i];
        for (int j = i + 1; j < n; j++) s -= A[i + (size_t)j * n] * x[j];
        x[i] = s / A[i + (size_t)i * n];
    }
    return SS_OK;
}

/* spectral B-vectors of f (spectralTransform!) → coefficients a per slot; the
 * caller's spectral array is overwritten with a (the input of the SI stage). */
int32_t or_elliptic_solve_spectral(const or_elliptic *e, double *spec) {
    or_grid *g = e->g;
    int b = g->b;
    long slots = 1 + 2L * g->K;
    int nmax = e->s0->Min > e->s1->Min ? e->s0->Min : e->s1->Min;
    double *G = (double *)malloc(sizeof(double) * (size_t)nmax * nmax);
    double *G0 = (double *)malloc(sizeof(double) * (size_t)nmax * nmax);
    double *x = (double *)malloc(sizeof(double) * (size_t)b);
    int lastm = -1, n = 0;
    for (int v = 0; v < g->nvars; v++) {
        double *sp = spec + (size_t)g->nspec * v;
        for (long q = 0; q < slots; q++) {
            int m = (int)((q + 1) / 2);
            const or_spline *s = m == 0 ? e->s0 : e->s1;
            if (m != lastm) { or_elliptic_operator(e, m, G0, &n); lastm = m; }
            memcpy(G, G0, sizeof(double) * (size_t)n * n);
            gamma_apply(s, sp + (size_t)q * b, x);
            int st = dense_lu_solve(G, n, x);
            if (st) { free(G); free(G0); free(x); return st; }
            gamma_adjoint(s, x, sp + (size_t)q * b);
        }
        lastm = -1;
    }
    free(G); free(G0); free(x);
    return SS_OK;
}

/* splineTransform!(sharedSpectral, tile), src/tiling.jl:1490-1516 (RL, blocks
 * p = 2k) and 1862-1892 (RLZ, blocks z_b·(1+2K) + (k−1)·2 + 1): every block of
 * b_iDim B-values goes through the two-argument SAtransform(spline, b)
 * (src/CubicBSpline.jl:1355-1359: Γᵀ (PQ)⁻¹ Γ b, no R3X background) into the
 * same rows of `acoef`.  Both layouts are one run of b-row blocks per variable. */
int32_t or_grid_spline_transform(const or_grid *g, const double *shared, double *acoef) {
    const int b = g->b;
    const long nblk = (long)g->bk * (1 + 2L * g->K);
    double *t = (double *)malloc(sizeof(double) * 3 * (size_t)b);
    for (int v = 0; v < g->nvars; v++)
        for (long q = 0; q < nblk; q++) {
            const size_t o = (size_t)g->nspec * v + (size_t)q * b;
            spline_sa(g->spl[v], shared + o, NULL, acoef + o, t, t + b, t + 2 * b);
        }
    free(t);
    return SS_OK;
}

/* a-coefficients in spectral layout → physical (the SI + ring stages of gridTransform!) */
int32_t or_grid_transform_coeffs(or_grid *g, const double *acoef, double *phys) {
    /* SA with the identity: run the inverse driver on a grid whose SA is skipped */
    int saved = g->skip_sa;
    g->skip_sa = 1;
    int st = or_grid_transform(g, acoef, phys);
    g->skip_sa = saved;
    return st;
}
