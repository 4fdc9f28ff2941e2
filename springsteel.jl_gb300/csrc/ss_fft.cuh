// ss_fft.cuh — CTA-cooperative complex DFTs in shared memory for sm_103a.
//
// The ring transforms of the reference call FFTW's R2HC/HC2R on rings of
// L = 4+4ri points (src/Fourier.jl:192-193, 388-395, 463-468).  Ring lengths
// have arbitrary prime factors, so a length-N complex DFT (N = L/2 after real
// packing) is evaluated by mixed-radix Stockham autosort passes: radices
// 4,2,3,5,7,11,13 in registers with per-pass twiddle rows; odd primes up to the
// plan set's limit as output-pair passes that read a per-prime DFT matrix; a
// larger prime factor p gets one Rader pass (a (p−1)-point cyclic convolution
// by two inner Stockham DFTs, zero-padded to a smooth length when p − 1 has a
// large prime factor), and lengths with no such plan fall back to Bluestein's
// chirp-z convolution of smooth length M >= 2N-1.  Twiddle rows, DFT matrices
// and index tables come from FP64-accurate tables built on the host
// (ss_setup.cpp), stored in the compute type's layout.
//
// Every routine transforms `ns` sequences of the same plan, `ss` complex
// entries apart in shared memory, with one barrier per pass for all of them.
// The CTA's threads walk the work units (butterfly position fastest, so a warp
// touches consecutive shared-memory entries) with carries, without a division
// per unit.
#pragma once

#include <cuda_runtime.h>

#include "ss_internal.h"
#include "ss_types.cuh"

namespace ss {

// In-register DFT of size R; SIGN = -1 forward (exp(-2πi ...)), +1 inverse.
template <int R, int SIGN, typename T>
__device__ __forceinline__ void dft_small(cpx<T> *v) {
    if constexpr (R == 2) {
        cpx<T> a = v[0], b = v[1];
        v[0] = c_add(a, b);
        v[1] = c_sub(a, b);
    } else if constexpr (R == 4) {
        cpx<T> t0 = c_add(v[0], v[2]), t1 = c_sub(v[0], v[2]);
        cpx<T> t2 = c_add(v[1], v[3]), d = c_sub(v[1], v[3]);
        // t3 = SIGN * i * d
        cpx<T> t3 = (SIGN < 0) ? cpx<T>{d.y, -d.x} : cpx<T>{-d.y, d.x};
        v[0] = c_add(t0, t2);
        v[2] = c_sub(t0, t2);
        v[1] = c_add(t1, t3);
        v[3] = c_sub(t1, t3);
    } else {
        // odd prime R: pair q with R-q
        constexpr int H = (R - 1) / 2;
        cpx<T> a[H], b[H];
#pragma unroll
        for (int q = 1; q <= H; q++) {
            a[q - 1] = c_add(v[q], v[R - q]);
            b[q - 1] = c_sub(v[q], v[R - q]);
        }
        cpx<T> x0 = v[0];
        cpx<T> s0 = x0;
#pragma unroll
        for (int q = 0; q < H; q++) s0 = c_add(s0, a[q]);
#pragma unroll
        for (int s = 1; s <= H; s++) {
            cpx<T> re = x0, im = c_zero<T>();
#pragma unroll
            for (int q = 1; q <= H; q++) {
                const int e = (q * s) % R;
                const T cs = rcos<T>(R, e), sn = rsin<T>(R, e);
                re.x = re.x + a[q - 1].x * cs;
                re.y = re.y + a[q - 1].y * cs;
                im.x = im.x + b[q - 1].x * sn;
                im.y = im.y + b[q - 1].y * sn;
            }
            // forward: X_s = re - i*im, X_{R-s} = re + i*im  (inverse: signs swap)
            cpx<T> iim = {-im.y, im.x};
            if (SIGN < 0) {
                v[s] = c_sub(re, iim);
                v[R - s] = c_add(re, iim);
            } else {
                v[s] = c_add(re, iim);
                v[R - s] = c_sub(re, iim);
            }
        }
        v[0] = s0;
    }
}

// j / d for 0 ≤ j < 2^22 and d ≥ 1 via a float reciprocal and one correction
// (the quotient estimate is off by at most one), instead of an integer division
__device__ __forceinline__ int div_small(int j, int d, float inv_d) {
    int q = __float2int_rz((float)j * inv_d);
    if (q * d > j) q--;
    else if ((q + 1) * d <= j) q++;
    return q;
}

// Work units (n, g), n < Nn, spread over the CTA's threads: unit
// threadIdx.x + i·blockDim.x in (n fastest) order, advanced by adding
// blockDim.x with one carry instead of a division per unit:
//   for (UnitWalk u(Nn); u.g < G; u.next()) { ... u.n, u.g ... }
struct UnitWalk {
    int n, g, dq, dm, Nn;
    __device__ __forceinline__ explicit UnitWalk(int Nn_) : Nn(Nn_) {
        const int T = blockDim.x;
        const float inv = __frcp_rn((float)Nn);  // div_small corrects the estimate: exact quotients
        dq = div_small(T, Nn, inv);
        dm = T - dq * Nn;
        g = div_small(threadIdx.x, Nn, inv);
        n = threadIdx.x - g * Nn;
    }
    __device__ __forceinline__ void next() {
        n += dm;
        g += dq;
        if (n >= Nn) {
            n -= Nn;
            g++;
        }
    }
};

// n consecutive complex entries of a twiddle table row (n even for binary32:
// the row starts 16-byte aligned and loads two entries per access).
template <typename T, int n>
__device__ __forceinline__ void ld_cplx_row(const typename Tab<T>::cplx_t *__restrict__ row, cpx<T> *w) {
    if constexpr (std::is_same<T, float>::value) {
        static_assert(n % 2 == 0, "binary32 rows are whole 16-byte loads");
        const float4 *r4 = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int u = 0; u < n / 2; u++) {
            const float4 v = __ldg(r4 + u);
            w[2 * u] = {v.x, v.y};
            w[2 * u + 1] = {v.z, v.w};
        }
    } else {
#pragma unroll
        for (int u = 0; u < n; u++) w[u] = ld_cplx<T>(row, u);
    }
}

// One Stockham pass over ns sequences: Ns = product of the radices already
// applied.  Work unit (k, jq, g): butterfly j = jq·Ns + k of sequence g, in
// the order j fastest, then g (unit threadIdx.x + i·blockDim.x); the thread's
// coordinates advance by the CTA stride, pre-split into (k, jq, g) steps, with
// two carries.  Inputs at j + r·N/R, outputs at jq·Ns·R + k + r·Ns.  ptab: the
// pass's twiddle rows (pass_row_width), null when Ns = 1.
template <int R, int SIGN, typename T>
__device__ __forceinline__ void stockham_pass(const cpx<T> *__restrict__ src, cpx<T> *__restrict__ dst, int N,
                                              int Ns, const void *__restrict__ ptab, int ns, int ss) {
    constexpr int RW = pass_row_width(R);
    using CT = typename Tab<T>::cplx_t;
    const int NR = N / R, NJ = NR / Ns;
    const float inv_nr = __frcp_rn((float)NR), inv_ns = __frcp_rn((float)Ns);
    const int TB = blockDim.x;
    int g = div_small(threadIdx.x, NR, inv_nr);
    const int j0 = threadIdx.x - g * NR;
    int jq = div_small(j0, Ns, inv_ns);
    int k = j0 - jq * Ns;
    const int dg = div_small(TB, NR, inv_nr);
    const int dj = TB - dg * NR;
    const int dq = div_small(dj, Ns, inv_ns);
    const int dk = dj - dq * Ns;
    const CT *tab = reinterpret_cast<const CT *>(ptab);
    while (g < ns) {
        const int j = jq * Ns + k;
        const cpx<T> *sp = src + (g * ss + j);
        cpx<T> *dp = dst + (g * ss + j + jq * Ns * (R - 1));
        cpx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = sp[r * NR];
        if (tab) {
            cpx<T> w[RW];
            ld_cplx_row<T, RW>(tab + k * RW, w);
#pragma unroll
            for (int r = 1; r < R; r++) {
                const cpx<T> a = v[r], b = w[r - 1];
                if (SIGN < 0) v[r] = {a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
                else v[r] = {a.x * b.x + a.y * b.y, a.y * b.x - a.x * b.y};  // a · conj(b)
            }
        }
        dft_small<R, SIGN>(v);
#pragma unroll
        for (int r = 0; r < R; r++) dp[r * Ns] = v[r];
        k += dk;
        jq += dq;
        g += dg;
        if (k >= Ns) {
            k -= Ns;
            jq++;
        }
        if (jq >= NJ) {
            jq -= NJ;
            g++;
        }
    }
}

template <typename T>
__device__ __forceinline__ const void *tab_at(const void *pool, int64_t off) {
    return (const void *)((const typename Tab<T>::cplx_t *)pool + off);
}

// Radix-R pass for an odd prime R > 13 (up to the plan set's direct limit).  A
// first sweep twiddles each butterfly's inputs (skipped when Ns = 1) and
// replaces them in place by the pairs a_q = v_q + v_{R−q} (at q) and
// b_q = v_q − v_{R−q} (at R−q), q = 1..(R−1)/2; then each work unit computes
// S conjugate output pairs (s, R−s) of one butterfly for IT sequences:
//   re = v_0 + Σ_q a_q cos(2πqs/R),  im = Σ_q b_q sin(2πqs/R),
//   X_s = re ∓ i·im, X_{R−s} = re ± i·im  (upper signs forward), X_0 = v_0 + Σ a_q.
// cos/sin(2πe/R) are the N-point twiddles at e·N/R.  Every a_q, b_q load feeds S
// output pairs and every twiddle load IT sequences: an S × IT register tile of
// the R × R DFT matrix product.
template <typename T> constexpr int kPrimeOut = sizeof(T) == 4 ? 2 : 4;  // output pairs per unit
template <typename T> constexpr int kPrimeSeqs = 1;                      // sequences per unit

// kPrimeTile consecutive entries of one row of a prime pass's DFT matrix
// (prime_matrix_width); binary32 rows load two entries per 16-byte access.
template <typename T>
__device__ __forceinline__ void ld_prime_row(const typename Tab<T>::cplx_t *__restrict__ row, cpx<T> *w) {
    if constexpr (std::is_same<T, float>::value) {
        const float4 *r4 = reinterpret_cast<const float4 *>(row);
#pragma unroll
        for (int u = 0; u < kPrimeTile / 2; u++) {
            const float4 v = __ldg(r4 + u);
            w[2 * u] = {v.x, v.y};
            w[2 * u + 1] = {v.z, v.w};
        }
    } else {
#pragma unroll
        for (int u = 0; u < kPrimeTile; u++) w[u] = ld_cplx<T>(row, u);
    }
}

template <int SIGN, typename T>
__device__ void prime_pass(cpx<T> *__restrict__ src, cpx<T> *__restrict__ dst, int N, int Ns, int R,
                           const void *__restrict__ tw, const void *__restrict__ mat, int ns, int ss) {
    const int NR = N / R, H = (R - 1) / 2;
    const int tstride = N / (Ns * R), rstep = N / R;
    const float inv_ns = 1.0f / (float)Ns;
    {
        constexpr int IT = 1;
        const int G = (ns + IT - 1) / IT;
        const float inv_h = 1.0f / (float)H;
        for (UnitWalk uw_(NR * H); uw_.g < (G); uw_.next()) {
        const int u = uw_.n, g = uw_.g;
            const int j = div_small(u, H, inv_h), q = u - j * H + 1;
            cpx<T> w1 = {T(1.0f), T(0.0f)}, w2 = w1;
            bool twd = false;
            if (Ns > 1) {
                const int k = j - div_small(j, Ns, inv_ns) * Ns;
                if (k > 0) {
                    w1 = ld_cplx<T>(tw, (int64_t)q * k * tstride);
                    w2 = ld_cplx<T>(tw, (int64_t)(R - q) * k * tstride);
                    if (SIGN > 0) { w1.y = -w1.y; w2.y = -w2.y; }
                    twd = true;
                }
            }
#pragma unroll
            for (int t = 0; t < IT; t++) {
                const int sq = g * IT + t;
                if (sq >= ns) break;
                cpx<T> *sv = src + (size_t)sq * ss + j;
                cpx<T> vq = sv[q * NR], vr = sv[(R - q) * NR];
                if (twd) {
                    vq = c_mul(vq, w1);
                    vr = c_mul(vr, w2);
                }
                sv[q * NR] = c_add(vq, vr);
                sv[(R - q) * NR] = c_sub(vq, vr);
            }
        }
        __syncthreads();
    }
    if (mat) {
        // Matrix form: unit (butterfly j, output tile s0..s0+kPrimeTile−1) of one
        // sequence walks q with running pointers; row q of the matrix gives the
        // tile's (cos, −sin)(2πqs/R) in kPrimeTile/2 (binary32) or kPrimeTile loads.
        constexpr int S = kPrimeTile;
        const int SW = prime_matrix_width(R), Gs = SW / S;
        const float inv_gs = 1.0f / (float)Gs;
        using CT = typename Tab<T>::cplx_t;
        for (UnitWalk uw_(NR * Gs); uw_.g < ns; uw_.next()) {
            const int u = uw_.n, sq = uw_.g;
            const int j = div_small(u, Gs, inv_gs), s0 = (u - j * Gs) * S;
            const int jq = div_small(j, Ns, inv_ns), k = j - jq * Ns;
            const cpx<T> *sv = src + (size_t)sq * ss + j;
            const cpx<T> x0 = sv[0];
            cpx<T> re[S], im[S];
#pragma unroll
            for (int i = 0; i < S; i++) { re[i] = x0; im[i] = c_zero<T>(); }
            const cpx<T> *pa = sv + NR, *pb = sv + (R - 1) * NR;
            const CT *row = reinterpret_cast<const CT *>(mat) + s0;
#pragma unroll 2
            for (int q = 1; q <= H; q++) {
                const cpx<T> a = *pa, b = *pb;
                pa += NR;
                pb -= NR;
                cpx<T> w[S];
                ld_prime_row<T>(row, w);
                row += SW;
#pragma unroll
                for (int i = 0; i < S; i++) {
                    re[i].x = re[i].x + a.x * w[i].x;
                    re[i].y = re[i].y + a.y * w[i].x;
                    im[i].x = im[i].x - b.x * w[i].y;
                    im[i].y = im[i].y - b.y * w[i].y;
                }
            }
            cpx<T> *d = dst + (size_t)sq * ss + jq * Ns * R + k;
#pragma unroll
            for (int i = 0; i < S; i++) {
                const int s = s0 + i;
                if (s > H) break;
                if (s == 0) {
                    d[0] = re[i];
                    continue;
                }
                const cpx<T> iim = {-im[i].y, im[i].x};
                if (SIGN < 0) {
                    d[s * Ns] = c_sub(re[i], iim);
                    d[(R - s) * Ns] = c_add(re[i], iim);
                } else {
                    d[s * Ns] = c_add(re[i], iim);
                    d[(R - s) * Ns] = c_sub(re[i], iim);
                }
            }
        }
        return;
    }
    // s = 0 gives X_0 = v_0 + Σ a_q through the unit twiddle; entries with s > H
    // are computed and dropped
    constexpr int S = kPrimeOut<T>, IT = kPrimeSeqs<T>;
    const int Gs = (H + 1 + S - 1) / S;
    const int G = (ns + IT - 1) / IT;
    const float inv_gs = 1.0f / (float)Gs;
    for (UnitWalk uw_(NR * Gs); uw_.g < (G); uw_.next()) {
        const int u = uw_.n, g = uw_.g;
        const int j = div_small(u, Gs, inv_gs), s0 = (u - j * Gs) * S;
        const int jq = div_small(j, Ns, inv_ns), k = j - jq * Ns;
        const int idxD = jq * Ns * R + k;
        cpx<T> re[S][IT], im[S][IT];
        int e[S];
#pragma unroll
        for (int t = 0; t < IT; t++) {
            const int sq = min(g * IT + t, ns - 1);  // a clamped duplicate is computed and not stored
            const cpx<T> x0 = src[(size_t)sq * ss + j];
#pragma unroll
            for (int i = 0; i < S; i++) { re[i][t] = x0; im[i][t] = c_zero<T>(); }
        }
#pragma unroll
        for (int i = 0; i < S; i++) e[i] = 0;
        for (int q = 1; q <= H; q++) {
            cpx<T> a[IT], b[IT];
#pragma unroll
            for (int t = 0; t < IT; t++) {
                const cpx<T> *sv = src + (size_t)min(g * IT + t, ns - 1) * ss + j;
                a[t] = sv[q * NR];
                b[t] = sv[(R - q) * NR];
            }
#pragma unroll
            for (int i = 0; i < S; i++) {
                e[i] += s0 + i;  // e = q·s mod R (s ≤ R − 1 keeps one subtraction enough)
                if (e[i] >= R) e[i] -= R;
                const cpx<T> w = ld_cplx<T>(tw, (int64_t)e[i] * rstep);  // (cos, −sin)(2πe/R)
#pragma unroll
                for (int t = 0; t < IT; t++) {
                    re[i][t].x = re[i][t].x + a[t].x * w.x;
                    re[i][t].y = re[i][t].y + a[t].y * w.x;
                    im[i][t].x = im[i][t].x - b[t].x * w.y;
                    im[i][t].y = im[i][t].y - b[t].y * w.y;
                }
            }
        }
#pragma unroll
        for (int t = 0; t < IT; t++) {
            const int sq = g * IT + t;
            if (sq >= ns) break;
            cpx<T> *d = dst + (size_t)sq * ss + idxD;
#pragma unroll
            for (int i = 0; i < S; i++) {
                const int s = s0 + i;
                if (s > H) break;
                if (s == 0) {
                    d[0] = re[i][t];
                    continue;
                }
                const cpx<T> iim = {-im[i][t].y, im[i][t].x};
                if (SIGN < 0) {
                    d[s * Ns] = c_sub(re[i][t], iim);
                    d[(R - s) * Ns] = c_add(re[i][t], iim);
                } else {
                    d[s * Ns] = c_add(re[i][t], iim);
                    d[(R - s) * Ns] = c_sub(re[i][t], iim);
                }
            }
        }
    }
}

// Stockham passes rad[s_begin..nrad) over ping-pong buffers, Ns0 = product of the
// radices already applied; returns the buffer holding the result.
// pm: pool offsets of the prime passes' DFT matrices, parallel to rad (null: none).
// pt: pool offsets of the radix passes' twiddle rows, parallel to rad.
template <int SIGN, typename T>
__device__ cpx<T> *stockham_plain(cpx<T> *a, cpx<T> *b, int N, const int *rad, int nrad, const void *tw, int ns,
                                  int ss, const void *pool, const int64_t *pm, const int64_t *pt, int s_begin = 0,
                                  int Ns0 = 1) {
    int Ns = Ns0;
    for (int s = s_begin; s < nrad; s++) {
        const int R = rad[s];
        const void *pst = (Ns > 1 && pt[s] >= 0) ? tab_at<T>(pool, pt[s]) : nullptr;
        switch (R) {
        case 4: stockham_pass<4, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        case 2: stockham_pass<2, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        case 3: stockham_pass<3, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        case 5: stockham_pass<5, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        case 7: stockham_pass<7, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        case 11: stockham_pass<11, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        case 13: stockham_pass<13, SIGN>(a, b, N, Ns, pst, ns, ss); break;
        default: {
            const int64_t mo = pm ? pm[s] : -1;
            prime_pass<SIGN, T>(a, b, N, Ns, R, tw, mo >= 0 ? tab_at<T>(pool, mo) : nullptr, ns, ss);
            break;
        }
        }
        __syncthreads();
        cpx<T> *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Radix-p pass by Rader's algorithm (p prime, first pass: Ns = 1, no input
// twiddles) over `nb` sequences of length N, `ss` apart.  Per butterfly j
// (NR = N/p of them) of sequence b:
//   u_a = x_{g^a} (a < p−1) into dst[(b·NR + j)·rM + a] (every inner
//   sequence rM apart, zero from p−1 to rM), x_0 into dst[tail + b·NR + j];
//   c = u ⊛ h by two rM-point DFTs (inner plan) and H = DFT_rM(h')/rM, h' = h
//   (rM = p − 1) or h wrapped into a zero-padded length-rM sequence;
//   X_0 = x_0 + DFT(u)_0 (into src[tail + b·NR + j]), X_{g^{−b}} = x_0 + c_b.
// The inverse transform runs as conj(forward(conj x)).  `tail` lies beyond
// every sequence's N outputs, so the scatter never overwrites a tail entry it
// still reads.  Returns the buffer holding the pass's outputs (either a or b).
template <int SIGN, typename T>
__device__ cpx<T> *rader_pass(cpx<T> *src, cpx<T> *dst, int N, const FftPlan &pl, const void *pool, int nb, int ss,
                              int tail) {
    const int p = pl.rp, P1 = p - 1, NR = N / p, M = pl.rM;  // inner sequences M ≥ p − 1 apart
    const float inv_p = 1.0f / (float)p;
    const void *H = tab_at<T>(pool, pl.rH);
    const void *perm = tab_at<T>(pool, pl.rperm);  // (g^a, g^{−a}) mod p
    for (UnitWalk uw_(N); uw_.g < (nb); uw_.next()) {
        const int e = uw_.n, b = uw_.g;  // gather: (j, a), a = p−1 → x_0
        const int j = div_small(e, p, inv_p), a = e - j * p;
        const int q = a < P1 ? ld_index_pair<T>(perm, a).x : 0;
        cpx<T> v = src[(size_t)b * ss + j + q * NR];
        if (SIGN > 0) v.y = -v.y;
        dst[a < P1 ? (size_t)(b * NR + j) * M + a : (size_t)tail + b * NR + j] = v;
    }
    const int ni = nb * NR;  // inner sequences
    if (M > P1)  // zero padding of each inner sequence
        for (UnitWalk uw_(M - P1); uw_.g < ni; uw_.next()) dst[(size_t)uw_.g * M + P1 + uw_.n] = c_zero<T>();
    __syncthreads();
    cpx<T> *r1 = stockham_plain<-1, T>(dst, src, M, pl.rrad, pl.rnrad, tab_at<T>(pool, pl.rtw), ni, M, pool, pl.rpm, pl.rpt);
    for (UnitWalk uw_(M); uw_.g < (ni); uw_.next()) {
        const int k = uw_.n, sq = uw_.g;
        cpx<T> *u = r1 + (size_t)sq * M + k;
        const cpx<T> U = *u;
        if (k == 0) src[tail + sq] = c_add(dst[tail + sq], U);  // X_0 into src's tail
        *u = c_mul(U, ld_cplx<T>(H, k));
    }
    __syncthreads();
    cpx<T> *other = (r1 == dst) ? src : dst;
    cpx<T> *r2 = stockham_plain<1, T>(r1, other, M, pl.rrad, pl.rnrad, tab_at<T>(pool, pl.rtw), ni, M, pool, pl.rpm, pl.rpt);
    cpx<T> *out = (r2 == dst) ? src : dst;
    for (UnitWalk uw_(N); uw_.g < (nb); uw_.next()) {
        const int e = uw_.n, b = uw_.g;  // scatter: (j, b'), b' = p−1 → X_0
        const int j = div_small(e, p, inv_p), bb = e - j * p;
        cpx<T> X;
        int s;
        if (bb == P1) {
            X = src[(size_t)tail + b * NR + j];
            s = 0;
        } else {
            X = c_add(dst[(size_t)tail + b * NR + j], r2[(size_t)(b * NR + j) * M + bb]);
            s = ld_index_pair<T>(perm, bb).y;
        }
        if (SIGN > 0) X.y = -X.y;
        out[(size_t)b * ss + j * p + s] = X;  // Ns = 1: butterfly j's outputs at j·p + s
    }
    __syncthreads();
    return out;
}

// A plan's Stockham DFT: the Rader pass first when the plan has one, then the
// remaining radix passes; returns the buffer holding the result.
template <int SIGN, typename T>
__device__ cpx<T> *stockham(cpx<T> *a, cpx<T> *b, int N, const int *rad, int nrad, const void *tw, int ns, int ss,
                            const FftPlan *pl, const void *pool, int tail) {
    if (pl && pl->rp) {
        cpx<T> *o = rader_pass<SIGN, T>(a, b, N, *pl, pool, ns, ss, tail);
        if (o != a) { b = a; a = o; }
        return stockham_plain<SIGN, T>(a, b, N, rad, nrad, tw, ns, ss, pool, pl->pm, pl->pt, 1, pl->rp);
    }
    return stockham_plain<SIGN, T>(a, b, N, rad, nrad, tw, ns, ss, pool, pl->pm, pl->pt);
}

// Sequence stride of a plan inside a CTA's ping-pong buffers: N, or M for
// Bluestein.  A buffer holds `cap` sequences (the CTA's item batch) and, for a
// Rader plan, cap × rader_data_len entries (sequences or inner sequences)
// followed by a tail of cap·N/p entries.
__host__ __device__ inline int fft_seq_stride(const FftPlan &p) { return p.blu ? p.M : p.N; }

// Length-N DFTs of the nb sequences in `a` (sign SIGN), sequence i at
// a + i·fft_seq_stride(p).  Both buffers hold cap × fft_buffer_len(plan)
// entries (cap ≥ nb).  Returns the buffer with the results, laid out like the
// input.
template <int SIGN, typename T>
__device__ cpx<T> *dft(cpx<T> *a, cpx<T> *b, const FftPlan &p, const void *pool, int nb, int cap) {
    if (!p.blu)
        return stockham<SIGN, T>(a, b, p.N, p.rad, p.nrad, tab_at<T>(pool, p.tw), nb, p.N, &p, pool,
                                 p.rp ? cap * rader_data_len(p) : 0);
    const int N = p.N, M = p.M;
    const void *chirp = tab_at<T>(pool, p.chirp);
    const void *filt = tab_at<T>(pool, p.filt);
    // X_k = c_k Σ_j (x_j c_j) conj(c_{k-j}) with c_k = exp(-πi k²/N); the
    // inverse DFT is conj(forward(conj x)).
    for (UnitWalk uw_(M); uw_.g < (nb); uw_.next()) {
        const int k = uw_.n, bi = uw_.g;
        cpx<T> *ab = a + (size_t)bi * M;
        cpx<T> v = c_zero<T>();
        if (k < N) {
            v = ab[k];
            if (SIGN > 0) v.y = -v.y;
            v = c_mul(v, ld_cplx<T>(chirp, k));
        }
        ab[k] = v;
    }
    __syncthreads();
    cpx<T> *r = stockham_plain<-1, T>(a, b, M, p.mrad, p.mnrad, tab_at<T>(pool, p.mtw), nb, M, pool, nullptr, p.mpt);
    for (UnitWalk uw_(M); uw_.g < (nb); uw_.next()) {
        const int k = uw_.n, bi = uw_.g;
        cpx<T> *rb = r + (size_t)bi * M;
        rb[k] = c_mul(rb[k], ld_cplx<T>(filt, k));
    }
    __syncthreads();
    cpx<T> *other = (r == a) ? b : a;
    cpx<T> *q = stockham_plain<1, T>(r, other, M, p.mrad, p.mnrad, tab_at<T>(pool, p.mtw), nb, M, pool, nullptr, p.mpt);
    for (UnitWalk uw_(N); uw_.g < (nb); uw_.next()) {
        const int k = uw_.n, bi = uw_.g;
        cpx<T> *qb = q + (size_t)bi * M;
        cpx<T> v = c_mul(qb[k], ld_cplx<T>(chirp, k));
        if (SIGN > 0) v.y = -v.y;
        qb[k] = v;
    }
    __syncthreads();
    return q;
}

}  // namespace ss
