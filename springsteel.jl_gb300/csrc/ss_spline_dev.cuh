// ss_spline_dev.cuh — device helpers of SAtransform!: the structured Γ fold
// and its adjoint (src/CubicBSpline.jl:427-500) and the banded forward/back
// substitution of the LLᵀ factor (src/banded_cholesky.jl:202-231).
#pragma once

#include "ss_internal.h"

namespace ss {

template <typename S>
__device__ __forceinline__ void gamma_fold(const SplineDev &sp, S *x, int Md, int n) {
    const int rL = sp.rankL;
    const S b0 = x[0], b1 = x[1], bM1 = x[Md - 1], bM2 = x[Md - 2];
    for (int i = 0; i < n; i++) x[i] = x[i + rL];
    if (sp.lk == BC_A1) { x[0] += (S)sp.aL * b0; x[1] += (S)sp.bL * b0; }
    else if (sp.lk == BC_A2) { x[0] += (S)sp.aL * b0 + (S)sp.bL * b1; }
    else if (sp.lk == BC_PER) { x[n - 1] += b0; }
    if (sp.rk == BC_A1) { x[n - 1] += (S)sp.aR * bM1; x[n - 2] += (S)sp.bR * bM1; }
    else if (sp.rk == BC_A2) { x[n - 1] += (S)sp.aR * bM1 + (S)sp.bR * bM2; }
    else if (sp.rk == BC_PER) { x[0] += bM2; x[1] += bM1; }
}
template <typename S>
__device__ __forceinline__ void gamma_unfold(const SplineDev &sp, S *x, int Md, int n) {
    const int rL = sp.rankL;
    const S s0v = x[0], s1v = x[1], sM1 = x[n - 1], sM2 = x[n - 2];
    for (int i = n - 1; i >= 0; i--) x[i + rL] = x[i];
    for (int j = 0; j < rL; j++) x[j] = S(0);
    for (int j = Md - sp.rankR; j < Md; j++) x[j] = S(0);
    if (sp.lk == BC_A1) x[0] = (S)sp.aL * s0v + (S)sp.bL * s1v;
    else if (sp.lk == BC_A2) { x[0] = (S)sp.aL * s0v; x[1] = (S)sp.bL * s0v; }
    else if (sp.lk == BC_PER) x[0] = sM1;
    if (sp.rk == BC_A1) x[Md - 1] = (S)sp.aR * sM1 + (S)sp.bR * sM2;
    else if (sp.rk == BC_A2) { x[Md - 2] = (S)sp.bR * sM1; x[Md - 1] = (S)sp.aR * sM1; }
    else if (sp.rk == BC_PER) { x[Md - 2] = s0v; x[Md - 1] = s1v; }
}
// forward L y = v, backward Lᵀ x = y in place (src/banded_cholesky.jl:202-231).
// `tail` (periodic splines, else null): the factor's last three rows, dense
// (tail[r·n + j] = L[n−3+r][j]), so those rows sum over every earlier y and
// every backward step also subtracts their entries below the band.
template <typename S>
__device__ __forceinline__ void band_solve(const S *Ls, const S *Di, S *x, int n, const S *tail = nullptr) {
    S y1 = S(0), y2 = S(0), y3 = S(0);
    const int r0 = tail ? n - 3 : n;
    for (int i = 0; i < n; i++) {
        S acc = x[i];
        if (i >= r0) {
            const S *row = tail + (size_t)(i - r0) * n;
            for (int j = 0; j < i; j++) acc -= row[j] * x[j];
        } else {
            if (i >= 3) acc -= Ls[(i - 3) * 4 + 3] * y3;
            if (i >= 2) acc -= Ls[(i - 2) * 4 + 2] * y2;
            if (i >= 1) acc -= Ls[(i - 1) * 4 + 1] * y1;
        }
        const S yi = acc * Di[i];
        x[i] = yi;
        y3 = y2; y2 = y1; y1 = yi;
    }
    S x1 = S(0), x2 = S(0), x3 = S(0);
    for (int i = n - 1; i >= 0; i--) {
        S acc = x[i];
        if (i + 1 < n) acc -= Ls[i * 4 + 1] * x1;
        if (i + 2 < n) acc -= Ls[i * 4 + 2] * x2;
        if (i + 3 < n) acc -= Ls[i * 4 + 3] * x3;
        if (tail)
            for (int r = max(r0, i + 4); r < n; r++) acc -= tail[(size_t)(r - r0) * n + i] * x[r];
        const S xi = acc * Di[i];
        x[i] = xi;
        x3 = x2; x2 = x1; x1 = xi;
    }
}

}  // namespace ss
