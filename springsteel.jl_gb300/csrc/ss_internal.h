// ss_internal.h — internal structures of the GB300 transform backend.
//
// Host-side setup (FP64) lives in ss_setup.cpp; device kernels in
// ss_kernels.cu; the C ABI in ss_api.cu.  All device tables are built once at
// ss_grid_create (the analogue of createGrid's template caches,
// src/CubicBSpline.jl:931-977, src/Fourier.jl:189-204) and stay resident.
#pragma once

#include <cstdint>
#include <string>
#include <array>
#include <map>
#include <vector>

#include <vector_types.h>

#include "springsteel_gpu.h"

#ifdef __CUDACC__
#define SS_HD __host__ __device__
#else
#define SS_HD
#endif

namespace ss {

// ---------------------------------------------------------------- errors
void set_error(const char *fmt, ...);
struct Status {
    int32_t code = SS_OK;
};

// ----------------------------------------------------------- FFT plans
// Complex DFT of length N evaluated by mixed-radix Stockham passes in
// shared memory, or (N with a prime factor > 13) by Bluestein's chirp-z
// convolution of smooth length M >= 2N-1.
constexpr int kMaxRadices = 24;
// largest odd prime handled by a direct radix pass (≈ (R−1) FMAs per element,
// below Bluestein's two length-≥2N FFTs up to about here); larger factors go
// through Bluestein
constexpr int kMaxPrimeRadix = 199;
struct FftPlan {
    int N;
    int nrad;
    int rad[kMaxRadices];
    int64_t tw;      // pool offset of W_N^t, t < N
    int blu;
    int M;
    int mnrad;
    int mrad[kMaxRadices];
    int64_t mtw;     // pool offset of W_M^t, t < M
    int64_t chirp;   // pool offset of exp(-πi k²/N), k < N
    int64_t filt;    // pool offset of FFT_M(conj chirp filter)/M
    // Rader pass for one prime factor p > the direct-pass limit (first radix of
    // rad[], stored as p): generator g, the (p−1)-point inner plan, and
    // H = FFT_{p−1}(h)/(p−1) with h_d = W_p^{g^{−d}}
    int rp, rg;
    // length of the cyclic convolution's inner DFTs: p − 1, or a smooth M ≥ 2p − 3
    // when p − 1 has a prime factor above the padding limit (the convolution is
    // then taken with u zero-padded to M and h wrapped, Rader 1968 with a
    // zero-padded convolution)
    int rM;
    int rnrad;
    int rrad[kMaxRadices];
    int64_t rtw;     // pool offset of W_rM^t, t < rM
    int64_t rH;      // pool offset of H, rM entries
    int64_t rperm;   // pool offset of (g^a mod p, g^{−a} mod p), a < p−1, as exact reals
    // pool offsets of the DFT matrices of the direct prime passes (radix > 13) in
    // rad[] and rrad[]; −1 for every other radix (prime_matrix_width)
    int64_t pm[kMaxRadices];
    int64_t rpm[kMaxRadices];
    // pool offsets of the per-pass twiddle rows of the radix passes (R ≤ 13,
    // Ns > 1) of rad[], rrad[] and mrad[]; −1 for every other pass
    // (pass_row_width)
    int64_t pt[kMaxRadices];
    int64_t rpt[kMaxRadices];
    int64_t mpt[kMaxRadices];
};

// Entries per twiddle row of a radix-R pass: R − 1 rounded up to even, so that
// binary32 rows are whole 16-byte loads.  Row k (k < Ns) of the pass holds
// W_N^{r·k·N/(Ns·R)} for r = 1..R−1 at entry r − 1, then (1, 0) padding.
SS_HD constexpr int pass_row_width(int R) { return (R - 1 + 1) / 2 * 2; }

// Output pairs (s, R−s) one work unit of a direct prime pass computes: one row
// load of the pass's DFT matrix feeds kPrimeTile outputs.
constexpr int kPrimeTile = 4;
// Columns of a radix-R prime matrix: s = 0..(R−1)/2, rounded up to whole tiles.
// Entry (q, s), q = 1..(R−1)/2, at (q − 1)·width + s holds
// (cos 2πqs/R, −sin 2πqs/R); the columns beyond (R−1)/2 hold the same formula
// and their outputs are dropped.
SS_HD inline int prime_matrix_width(int R) { return ((R - 1) / 2 + kPrimeTile) / kPrimeTile * kPrimeTile; }

// One Fourier ring (src/factory.jl:608-624): L = 4+4ri points, kmax, bDim = 2ri+1.
struct RingDesc {
    int L;
    int ri;
    int kmax;
    int plan;          // index of the length-L/2 complex plan
    int64_t utw;       // pool offset of W_L^t, t < L/2 (real-packing twiddles)
    int64_t phase;     // offset of cos(k ymin), sin(k ymin) (k = 1..kmax) in the phase pool
    int64_t jofs;      // Σ_{r'<r} L_r'   (ring start in jDim numbering)
    int64_t fofs;      // Σ_{r'<r} (1+2ri') (packed coefficient row start)
};

// Compute-type layouts of the device tables (ss_types.cuh): TL_F64 double,
// TL_DF64 (hi, lo) binary32 pairs, TL_F32 float.
enum { TL_F64 = 0, TL_DF64 = 1, TL_F32 = 2 };

// Per-variable spline template on the device (FP64 factor, B-spline weights).
struct SplineDev {
    int bDim, Min, rankL, rankR, lk, rk, r3x;
    int periodic;       // PERIODIC on a side: L has 3 dense bottom rows (tail), A has corners
    double aL, bL, aR, bR;
    double *L4;         // Min*4: L[j+d][j] at j*4+d   (FP64 banded Cholesky factor)
    double *dinv;       // Min: 1/L[j][j]
    double *PQb;        // bDim*7 full P+Q band (R3X only)
    float *L4f;         // FP32-rounded factor (FP32 mode)
    float *dinvf;
    double *Aband;      // FP64 open-form Γ(P+Q)Γᵀ band, Aband[j*4+d] = A[j+d][j] (FP32 refinement residual)
    double *tail;       // periodic: rows n-3..n-1 of L, tail[r*n + j] = L[n-3+r][j] (j ≤ n-3+r); else null
    float *tailf;       // the same, FP32-rounded
    double *acorner;    // periodic: A[n-3+r][c] for c < 3 where |n-3+r-c| > 3 (else 0), 3 × 3
    const void *sbw_t;  // bDim*(4 mubar) SB weights (row mi, tap), compute layout
    const void *siw_t;  // 3*mishDim*4 SI weights (derivative, point, tap), compute layout
    int *si_m0;         // mishDim: first coefficient index of the 4-tap window
};

// Per-variable Chebyshev column tables (src/Chebyshev.jl), compute layout.
struct ChebDev {
    int N, bk, nrank, half;
    double dscale;        // -0.5*(zmax - zmin)
    const void *fwd_t;    // bk × ceil(N/2): folded forward DCT-I rows (scale, filter folded)
    const void *inv_e_t;  // half_out × ne: inverse DCT-I, even-k columns
    const void *inv_o_t;  // half_out × no: inverse DCT-I, odd-k columns
    const void *gu_t;     // nrank × bk   (Γ = Σ u vᵀ restricted to the first bk rows)
    const void *gv_t;     // nrank × N
    // the same tables transposed and zero-padded to multiples of 4 for the
    // register-tiled kernels (coalesced loads, 16-byte aligned rows)
    const void *inv_et_t;  // ne × JP,   JP  = 4⌈half/4⌉:  inv_e[j][k] at [k][j]
    const void *inv_ot_t;  // no × JP
    const void *fwd_et_t;  // half × KEP, KEP = 4⌈⌈bk/2⌉/4⌉: fwd[2i][j] at [j][i]
    const void *fwd_ot_t;  // half × KOP, KOP = 4⌈⌊bk/2⌋/4⌉: fwd[2i+1][j] at [j][i]
    // CA, the CIx recurrence D (÷ dscale) and the folded DCT-I composed:
    // u = M_d b for derivative order d = 0, 1, 2, split into output halves
    // (u[j] = (Me b)[j] + (Mo b)[j], u[N-1-j] = (Me b)[j] − (Mo b)[j]).  Half pe
    // reads only the inputs of parity (pe + d) mod 2 plus s = Uᵀ b (the rank
    // term of Γ); stored as [d][pe][kcap rows: those inputs, then s][JP]
    const void *inv_m_t;
    int kcap, _kpad;
};
SS_HD inline int cheb_pad4(int n) { return n > 0 ? (n + 3) / 4 * 4 : 4; }

enum { BC_R0 = 0, BC_A1 = 1, BC_A2 = 2, BC_PER = 3, BC_R3 = 4 };

// ---------------------------------------------------------- host setup
struct SplineHost {
    double xmin, xmax, DX, DXrecip, l_q;
    int nc, mubar, bDim, mishDim;
    std::vector<double> qp, qw, mish;
    int Mdim, Min, rankL, rankR, lk, rk, r3x;
    double aL, bL, aR, bR;
    std::vector<double> PQb, L4, Aopen, sbw, siw;  // Aopen: open-form band before factoring
    std::vector<int> si_m0;
    int periodic = 0;
    std::vector<double> tail, acorner;  // periodic factor rows n-3..n-1 and out-of-band corners of A
};
int32_t build_spline(double xmin, double xmax, int nc, int mubar, int quad, double l_q,
                     const ss_spline_bc &bcl, const ss_spline_bc &bcr, SplineHost &out);

struct ChebHost {
    int N, bk, nrank, half;
    double dscale;
    std::vector<double> fwd, inv_e, inv_o, gu, gv, mish;
};
int32_t build_cheb(int N, int bk, int bcb, int bct, double zmin, double zmax, ChebHost &out);
// SI weights at arbitrary radii: window start m0[i], w[(d·n + i)·4 + tap], d = 0, 1, 2
int32_t spline_point_weights(const SplineHost &s, const double *x, int n, std::vector<int> &m0,
                             std::vector<double> &w);

// Pool of complex twiddles (interleaved re, im) in FP64.
struct TwiddlePool {
    std::vector<double> v;  // 2 doubles per complex entry
    int64_t push_table(int n, int sign, int len);   // exp(sign 2πi t/n), t < len
    int64_t push(const std::vector<double> &cplx_interleaved);
    int64_t size() const { return (int64_t)v.size() / 2; }
};
struct PlanSet {
    std::vector<FftPlan> plans;
    std::vector<int> plan_of_N;     // index by N (−1 if absent)
    std::vector<int64_t> utw_of_L;  // by L
    std::vector<int64_t> mtw_of_M;  // by M
    std::vector<int64_t> pm_of_R;   // by prime radix R
    int max_smem_cplx = 0;          // largest complex buffer (N or M)
    int max_prime = kMaxPrimeRadix; // direct prime passes up to here, Rader or Bluestein above
    bool rader = true;              // Rader passes for larger primes (else Bluestein)
    int pad_prime = kMaxPrimeRadix; // Rader inner lengths with a prime factor above this are zero-padded
    int plan_for(int N, TwiddlePool &pool);
    int64_t unpack_for(int L, TwiddlePool &pool);
    int64_t prime_matrix(int R, TwiddlePool &pool);
    std::map<std::array<int, 3>, int64_t> pt_of;  // by (N, Ns, R)
    int64_t pass_table(int N, int Ns, int R, TwiddlePool &pool);
    void pass_tables(int n, const int *rad, int nrad, int s0, int Ns0, int64_t *pt, TwiddlePool &pool);
};
// entries of a Rader plan's data region: the N sequence entries, or the N/p
// inner sequences of rM entries when those are longer
SS_HD inline int rader_data_len(const FftPlan &p) { return p.N / p.rp * p.rM > p.N ? p.N / p.rp * p.rM : p.N; }
// complex entries of one ping-pong buffer per sequence: M (Bluestein); for a
// Rader plan its data region plus a tail of N/p entries that holds the x_0
// terms; else N
SS_HD inline int fft_buffer_len(const FftPlan &p) { return p.blu ? p.M : (p.rp ? rader_data_len(p) + p.N / p.rp : p.N); }

}  // namespace ss
