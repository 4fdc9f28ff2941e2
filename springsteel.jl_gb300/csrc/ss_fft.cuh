// ss_fft.cuh — CTA-cooperative complex DFT in shared memory for sm_103a.
//
// The ring transforms of the reference call FFTW's R2HC/HC2R on rings of
// L = 4+4ri points (src/Fourier.jl:192-193, 388-395, 463-468).  Ring lengths
// have arbitrary prime factors, so a length-N complex DFT (N = L/2 after real
// packing) is evaluated by mixed-radix Stockham autosort passes (radices
// 4,2,3,5,7,11,13 in registers, odd primes up to the plan set's limit as
// output-pair passes); a larger prime factor p gets one Rader pass (a
// (p−1)-point cyclic convolution by two inner Stockham DFTs), and lengths with
// no such plan fall back to Bluestein's chirp-z convolution of smooth length
// M >= 2N-1.  Twiddles and index tables come from FP64-accurate tables built
// on the host (ss_setup.cpp), stored in the compute type's layout.
//
// Every routine transforms a batch of `nb` independent sequences of the same
// plan, `bs` complex entries apart in shared memory: one barrier per pass
// serves the whole batch, and every thread loops over (sequence, index) pairs.
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

// One Stockham pass over the batch: Ns = product of the radices already applied.
template <int R, int SIGN, typename T>
__device__ __forceinline__ void stockham_pass(const cpx<T> *__restrict__ src, cpx<T> *__restrict__ dst, int N,
                                              int Ns, const void *__restrict__ tw, int nb, int bs) {
    const int NR = N / R;
    const int tstride = N / (Ns * R);
    const int total = nb * NR;
    const float inv_ns = 1.0f / (float)Ns;
    for (int t = threadIdx.x; t < total; t += blockDim.x) {
        const int bi = nb == 1 ? 0 : t / NR, j = t - bi * NR;  // no division for a single sequence
        const cpx<T> *s = src + (size_t)bi * bs;
        cpx<T> *d = dst + (size_t)bi * bs;
        const int jq = div_small(j, Ns, inv_ns);
        const int k = j - jq * Ns;
        cpx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = s[j + r * NR];
        if (k > 0) {
            const int step = tstride * k;
#pragma unroll
            for (int r = 1; r < R; r++) {
                cpx<T> w = ld_cplx<T>(tw, (int64_t)r * step);
                if (SIGN > 0) w.y = -w.y;
                v[r] = c_mul(v[r], w);
            }
        }
        dft_small<R, SIGN>(v);
        const int idxD = jq * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) d[idxD + r * Ns] = v[r];
    }
}

template <typename T>
__device__ __forceinline__ const void *tab_at(const void *pool, int64_t off) {
    return (const void *)((const typename Tab<T>::cplx_t *)pool + off);
}

// Radix-R pass for an odd prime R > 13 (up to kMaxPrimeRadix).  A first
// sweep twiddles each butterfly's inputs (skipped when Ns = 1) and replaces
// them in place by the pairs a_q = v_q + v_{R−q} (at q) and b_q = v_q − v_{R−q}
// (at R−q), q = 1..(R−1)/2; then each work item computes kPrimeGroup conjugate
// output pairs (s, R−s) of one butterfly:
//   re = v_0 + Σ_q a_q cos(2πqs/R),  im = Σ_q b_q sin(2πqs/R),
//   X_s = re ∓ i·im, X_{R−s} = re ± i·im  (upper signs forward), X_0 = v_0 + Σ a_q.
// cos/sin(2πe/R) are the N-point twiddles at e·N/R.  Four FMAs per term and
// output pair instead of a length ≥ 2N−1 chirp-z convolution; each a_q, b_q
// load from shared memory serves all of the item's pairs.
template <typename T> constexpr int kPrimeGroup = sizeof(T) == 4 ? 2 : 4;  // output pairs per work item of a prime pass
template <int SIGN, typename T>
__device__ void prime_pass(cpx<T> *__restrict__ src, cpx<T> *__restrict__ dst, int N, int Ns, int R,
                           const void *__restrict__ tw, int nb, int bs) {
    const int NR = N / R, H = (R - 1) / 2;
    const int tstride = N / (Ns * R), rstep = N / R;
    const float inv_ns = 1.0f / (float)Ns, inv_h = 1.0f / (float)H;
    {
        const int per = NR * H;
        for (int t = threadIdx.x; t < nb * per; t += blockDim.x) {
            const int bi = nb == 1 ? 0 : t / per, rest = t - bi * per;
            const int j = div_small(rest, H, inv_h), q = rest - j * H + 1;
            cpx<T> *sv = src + (size_t)bi * bs + j;
            cpx<T> vq = sv[q * NR], vr = sv[(R - q) * NR];
            if (Ns > 1) {
                const int k = j - div_small(j, Ns, inv_ns) * Ns;
                if (k > 0) {
                    cpx<T> w1 = ld_cplx<T>(tw, (int64_t)q * k * tstride);
                    cpx<T> w2 = ld_cplx<T>(tw, (int64_t)(R - q) * k * tstride);
                    if (SIGN > 0) { w1.y = -w1.y; w2.y = -w2.y; }
                    vq = c_mul(vq, w1);
                    vr = c_mul(vr, w2);
                }
            }
            sv[q * NR] = c_add(vq, vr);
            sv[(R - q) * NR] = c_sub(vq, vr);
        }
        __syncthreads();
    }
    // each work item: S consecutive output pairs s = s0 .. s0+S−1 of one
    // butterfly, so every a_q, b_q load feeds S pairs (s = 0 gives X_0 = v_0 + Σ a_q
    // through the unit twiddle; entries with s > H are computed and dropped).
    // S = 2 for binary32, whose ring kernels run at 64 registers per thread.
    constexpr int S = kPrimeGroup<T>;
    const int G = (H + 1 + S - 1) / S;
    const int per = NR * G;
    const float inv_g = 1.0f / (float)G;
    for (int t = threadIdx.x; t < nb * per; t += blockDim.x) {
        const int bi = nb == 1 ? 0 : t / per, rest = t - bi * per;
        const int j = div_small(rest, G, inv_g), s0 = (rest - j * G) * S;
        const cpx<T> *sv = src + (size_t)bi * bs + j;
        cpx<T> *d = dst + (size_t)bi * bs;
        const int jq = div_small(j, Ns, inv_ns), k = j - jq * Ns;
        const int idxD = jq * Ns * R + k;
        const cpx<T> x0 = sv[0];
        cpx<T> re[S], im[S];
        int e[S];
#pragma unroll
        for (int i = 0; i < S; i++) { re[i] = x0; im[i] = c_zero<T>(); e[i] = 0; }
        for (int q = 1; q <= H; q++) {
            const cpx<T> a = sv[q * NR], b = sv[(R - q) * NR];
#pragma unroll
            for (int i = 0; i < S; i++) {
                e[i] += s0 + i;  // e = q·s mod R (s ≤ R − 1 keeps one subtraction enough)
                if (e[i] >= R) e[i] -= R;
                const cpx<T> w = ld_cplx<T>(tw, (int64_t)e[i] * rstep);  // (cos, −sin)(2πe/R)
                re[i].x = re[i].x + a.x * w.x;
                re[i].y = re[i].y + a.y * w.x;
                im[i].x = im[i].x - b.x * w.y;
                im[i].y = im[i].y - b.y * w.y;
            }
        }
#pragma unroll
        for (int i = 0; i < S; i++) {
            const int s = s0 + i;
            if (s > H) break;
            if (s == 0) {
                d[idxD] = re[i];
                continue;
            }
            const cpx<T> iim = {-im[i].y, im[i].x};
            if (SIGN < 0) {
                d[idxD + s * Ns] = c_sub(re[i], iim);
                d[idxD + (R - s) * Ns] = c_add(re[i], iim);
            } else {
                d[idxD + s * Ns] = c_add(re[i], iim);
                d[idxD + (R - s) * Ns] = c_sub(re[i], iim);
            }
        }
    }
}

// Stockham passes rad[s_begin..nrad) over ping-pong buffers, Ns0 = product of the
// radices already applied; returns the buffer holding the result.
template <int SIGN, typename T>
__device__ cpx<T> *stockham_plain(cpx<T> *a, cpx<T> *b, int N, const int *rad, int nrad, const void *tw, int nb,
                                  int bs, int s_begin = 0, int Ns0 = 1) {
    int Ns = Ns0;
    for (int s = s_begin; s < nrad; s++) {
        const int R = rad[s];
        switch (R) {
        case 4: stockham_pass<4, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        case 2: stockham_pass<2, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        case 3: stockham_pass<3, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        case 5: stockham_pass<5, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        case 7: stockham_pass<7, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        case 11: stockham_pass<11, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        case 13: stockham_pass<13, SIGN>(a, b, N, Ns, tw, nb, bs); break;
        default: prime_pass<SIGN, T>(a, b, N, Ns, R, tw, nb, bs); break;
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
// twiddles).  Per butterfly j (NR = N/p of them):
//   u_a = x_{g^a} (a < p−1) into dst[j(p−1) + a], x_0 into dst's tail dst[N + j];
//   c = u ⊛ h by two (p−1)-point DFTs (inner plan) and H = DFT(h)/(p−1);
//   X_0 = x_0 + DFT(u)_0 (kept in src's tail), X_{g^{−b}} = x_0 + c_b.
// The inverse transform runs as conj(forward(conj x)).  The tails beyond the N
// data entries are never touched by the inner passes.  Returns the buffer
// holding the pass's outputs (either a or b).
template <int SIGN, typename T>
__device__ cpx<T> *rader_pass(cpx<T> *src, cpx<T> *dst, int N, const FftPlan &pl, const void *pool, int nb, int bs) {
    const int p = pl.rp, P1 = p - 1, NR = N / p;
    const float inv_p = 1.0f / (float)p, inv_p1 = 1.0f / (float)P1;
    const void *H = tab_at<T>(pool, pl.rH);
    const void *perm = tab_at<T>(pool, pl.rperm);  // (g^a, g^{−a}) mod p
    for (int t = threadIdx.x; t < nb * N; t += blockDim.x) {  // gather: (j, a), a = p−1 → x_0
        const int bi = nb == 1 ? 0 : t / N, e = t - bi * N;
        const int j = div_small(e, p, inv_p), a = e - j * p;
        const int q = a < P1 ? ld_index_pair<T>(perm, a).x : 0;
        cpx<T> v = src[(size_t)bi * bs + j + q * NR];
        if (SIGN > 0) v.y = -v.y;
        dst[(size_t)bi * bs + (a < P1 ? j * P1 + a : N + j)] = v;
    }
    __syncthreads();
    cpx<T> *r2 = dst;
    for (int bi = 0; bi < nb; bi++) {  // inner cyclic convolutions of one item at a time
        cpx<T> *d0 = dst + (size_t)bi * bs, *s0 = src + (size_t)bi * bs;
        cpx<T> *r1 = stockham_plain<-1, T>(d0, s0, P1, pl.rrad, pl.rnrad, tab_at<T>(pool, pl.rtw), NR, P1);
        for (int e = threadIdx.x; e < NR * P1; e += blockDim.x) {
            const int j = div_small(e, P1, inv_p1), k = e - j * P1;
            const cpx<T> U = r1[e];
            if (k == 0) s0[N + j] = c_add(d0[N + j], U);  // X_0 into src's tail
            r1[e] = c_mul(U, ld_cplx<T>(H, k));
        }
        __syncthreads();
        cpx<T> *other = (r1 == d0) ? s0 : d0;
        cpx<T> *rr = stockham_plain<1, T>(r1, other, P1, pl.rrad, pl.rnrad, tab_at<T>(pool, pl.rtw), NR, P1);
        r2 = (rr == d0) ? dst : src;  // same choice for every item
    }
    cpx<T> *out = (r2 == dst) ? src : dst;
    for (int t = threadIdx.x; t < nb * N; t += blockDim.x) {  // scatter: (j, b), b = p−1 → X_0
        const int bi = nb == 1 ? 0 : t / N, e = t - bi * N;
        const int j = div_small(e, p, inv_p), b = e - j * p;
        const cpx<T> *rb = r2 + (size_t)bi * bs;
        cpx<T> X;
        int s;
        if (b == P1) {
            X = src[(size_t)bi * bs + N + j];
            s = 0;
        } else {
            X = c_add(dst[(size_t)bi * bs + N + j], rb[j * P1 + b]);
            s = ld_index_pair<T>(perm, b).y;
        }
        if (SIGN > 0) X.y = -X.y;
        out[(size_t)bi * bs + j * p + s] = X;  // Ns = 1: butterfly j's outputs at j·p + s
    }
    __syncthreads();
    return out;
}

// A plan's Stockham DFT: the Rader pass first when the plan has one, then the
// remaining radix passes; returns the buffer holding the result.
template <int SIGN, typename T>
__device__ cpx<T> *stockham(cpx<T> *a, cpx<T> *b, int N, const int *rad, int nrad, const void *tw, int nb, int bs,
                            const FftPlan *pl, const void *pool) {
    if (pl && pl->rp) {
        cpx<T> *o = rader_pass<SIGN, T>(a, b, N, *pl, pool, nb, bs);
        if (o != a) { b = a; a = o; }
        return stockham_plain<SIGN, T>(a, b, N, rad, nrad, tw, nb, bs, 1, pl->rp);
    }
    return stockham_plain<SIGN, T>(a, b, N, rad, nrad, tw, nb, bs);
}

// Length-N DFTs of the nb sequences in `a` (sign SIGN), sequence i at a + i·bs.
// Both buffers hold nb × fft_buffer_len(plan) entries (bs ≥ that length).
// Returns the buffer with the results, laid out like the input.
template <int SIGN, typename T>
__device__ cpx<T> *dft(cpx<T> *a, cpx<T> *b, const FftPlan &p, const void *pool, int nb = 1, int bs = 0) {
    if (!p.blu) return stockham<SIGN, T>(a, b, p.N, p.rad, p.nrad, tab_at<T>(pool, p.tw), nb, bs, &p, pool);
    const int N = p.N, M = p.M;
    const void *chirp = tab_at<T>(pool, p.chirp);
    const void *filt = tab_at<T>(pool, p.filt);
    // X_k = c_k Σ_j (x_j c_j) conj(c_{k-j}) with c_k = exp(-πi k²/N); the
    // inverse DFT is conj(forward(conj x)).
    for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
        const int bi = nb == 1 ? 0 : t / M, k = t - bi * M;
        cpx<T> *ab = a + (size_t)bi * bs;
        cpx<T> v = c_zero<T>();
        if (k < N) {
            v = ab[k];
            if (SIGN > 0) v.y = -v.y;
            v = c_mul(v, ld_cplx<T>(chirp, k));
        }
        ab[k] = v;
    }
    __syncthreads();
    cpx<T> *r = stockham_plain<-1, T>(a, b, M, p.mrad, p.mnrad, tab_at<T>(pool, p.mtw), nb, bs);
    for (int t = threadIdx.x; t < nb * M; t += blockDim.x) {
        const int bi = nb == 1 ? 0 : t / M, k = t - bi * M;
        cpx<T> *rb = r + (size_t)bi * bs;
        rb[k] = c_mul(rb[k], ld_cplx<T>(filt, k));
    }
    __syncthreads();
    cpx<T> *other = (r == a) ? b : a;
    cpx<T> *q = stockham_plain<1, T>(r, other, M, p.mrad, p.mnrad, tab_at<T>(pool, p.mtw), nb, bs);
    for (int t = threadIdx.x; t < nb * N; t += blockDim.x) {
        const int bi = nb == 1 ? 0 : t / N, k = t - bi * N;
        cpx<T> *qb = q + (size_t)bi * bs;
        cpx<T> v = c_mul(qb[k], ld_cplx<T>(chirp, k));
        if (SIGN > 0) v.y = -v.y;
        qb[k] = v;
    }
    __syncthreads();
    return q;
}

}  // namespace ss
