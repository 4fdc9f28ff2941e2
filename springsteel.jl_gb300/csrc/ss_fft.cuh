// ss_fft.cuh — CTA-cooperative complex DFT in shared memory for sm_103a.
//
// The ring transforms of the reference call FFTW's R2HC/HC2R on rings of
// L = 4+4ri points (src/Fourier.jl:192-193, 388-395, 463-468).  Ring lengths
// have arbitrary prime factors, so a length-N complex DFT (N = L/2 after real
// packing) is evaluated either by mixed-radix Stockham autosort passes
// (radices 4,2,3,5,7,11,13 in registers) or, when N has a prime factor > 13,
// by Bluestein's chirp-z convolution of smooth length M >= 2N-1 whose two FFTs
// are again Stockham passes.  Twiddles come from FP64-accurate tables built on
// the host (ss_setup.cpp), stored in the compute type's layout.
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

// One Stockham pass: Ns = product of the radices already applied.
template <int R, int SIGN, typename T>
__device__ __forceinline__ void stockham_pass(const cpx<T> *__restrict__ src, cpx<T> *__restrict__ dst, int N,
                                              int Ns, const void *__restrict__ tw) {
    const int NR = N / R;
    const int tstride = N / (Ns * R);
    for (int j = threadIdx.x; j < NR; j += blockDim.x) {
        const int k = j % Ns;
        cpx<T> v[R];
#pragma unroll
        for (int r = 0; r < R; r++) v[r] = src[j + r * NR];
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
        const int idxD = (j / Ns) * Ns * R + k;
#pragma unroll
        for (int r = 0; r < R; r++) dst[idxD + r * Ns] = v[r];
    }
}

template <typename T>
__device__ __forceinline__ const void *tab_at(const void *pool, int64_t off) {
    return (const void *)((const typename Tab<T>::cplx_t *)pool + off);
}

// Stockham DFT over ping-pong buffers; returns the buffer holding the result.
template <int SIGN, typename T>
__device__ cpx<T> *stockham(cpx<T> *a, cpx<T> *b, int N, const int *rad, int nrad, const void *tw) {
    int Ns = 1;
    for (int s = 0; s < nrad; s++) {
        const int R = rad[s];
        switch (R) {
        case 4: stockham_pass<4, SIGN>(a, b, N, Ns, tw); break;
        case 2: stockham_pass<2, SIGN>(a, b, N, Ns, tw); break;
        case 3: stockham_pass<3, SIGN>(a, b, N, Ns, tw); break;
        case 5: stockham_pass<5, SIGN>(a, b, N, Ns, tw); break;
        case 7: stockham_pass<7, SIGN>(a, b, N, Ns, tw); break;
        case 11: stockham_pass<11, SIGN>(a, b, N, Ns, tw); break;
        case 13: stockham_pass<13, SIGN>(a, b, N, Ns, tw); break;
        default: break;
        }
        __syncthreads();
        cpx<T> *t = a;
        a = b;
        b = t;
        Ns *= R;
    }
    return a;
}

// Length-N DFT of the N values in `a` (sign SIGN).  Both buffers hold
// fft_buffer_len(plan) entries.  Returns the buffer with the N results.
template <int SIGN, typename T>
__device__ cpx<T> *dft(cpx<T> *a, cpx<T> *b, const FftPlan &p, const void *pool) {
    if (!p.blu) return stockham<SIGN, T>(a, b, p.N, p.rad, p.nrad, tab_at<T>(pool, p.tw));
    const int N = p.N, M = p.M;
    const void *chirp = tab_at<T>(pool, p.chirp);
    const void *filt = tab_at<T>(pool, p.filt);
    // X_k = c_k Σ_j (x_j c_j) conj(c_{k-j}) with c_k = exp(-πi k²/N); the
    // inverse DFT is conj(forward(conj x)).
    for (int k = threadIdx.x; k < M; k += blockDim.x) {
        cpx<T> v = c_zero<T>();
        if (k < N) {
            v = a[k];
            if (SIGN > 0) v.y = -v.y;
            v = c_mul(v, ld_cplx<T>(chirp, k));
        }
        a[k] = v;
    }
    __syncthreads();
    cpx<T> *r = stockham<-1, T>(a, b, M, p.mrad, p.mnrad, tab_at<T>(pool, p.mtw));
    for (int k = threadIdx.x; k < M; k += blockDim.x) r[k] = c_mul(r[k], ld_cplx<T>(filt, k));
    __syncthreads();
    cpx<T> *other = (r == a) ? b : a;
    cpx<T> *q = stockham<1, T>(r, other, M, p.mrad, p.mnrad, tab_at<T>(pool, p.mtw));
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        cpx<T> v = c_mul(q[k], ld_cplx<T>(chirp, k));
        if (SIGN > 0) v.y = -v.y;
        q[k] = v;
    }
    __syncthreads();
    return q;
}

}  // namespace ss
