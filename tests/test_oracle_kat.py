"""Pins the FP64 oracle against the reference's own known-answer tests.

Each test restates one testset of Springsteel.jl's suite (file:line given)
with the reference's tolerance, plus an independent cross-check of the DFT /
DCT kinds (FFTW R2HC, HC2R, REDFT00) against numpy/scipy (pocketfft).
"""
import numpy as np
import pytest

import oracle as O
from springsteel_gpu import abi

R0 = (abi.SS_SBC_R0, 0.0, 0.0)
R1T0 = (abi.SS_SBC_RANK1, -4.0, -1.0)
R1T1 = (abi.SS_SBC_RANK1, 0.0, 1.0)
R1T2 = (abi.SS_SBC_RANK1, 2.0, -1.0)
R2T10 = (abi.SS_SBC_RANK2, 1.0, -0.5)
R2T20 = (abi.SS_SBC_RANK2, -1.0, 0.0)
R3 = (abi.SS_SBC_R3, 0.0, 0.0)
R3X = (abi.SS_SBC_R3X, 0.0, 0.0)


# ---- basis (test/basis.jl:26-42) -------------------------------------------
def test_basis_peak_values():
    s = O.OracleSpline(0.0, 10.0, 10)
    xm = 3.0
    assert abs(s.basis(3, xm, 0) - 4.0 / 6.0) < 1e-14
    assert abs(s.basis(3, xm, 1)) < 1e-14
    assert abs(s.basis(3, xm + 2.0, 0)) < 1e-14
    assert abs(s.basis(3, xm, 2) - (-2.0)) < 1e-12
    assert np.isnan(s.basis(3, -0.1, 0))  # DomainError in the reference


def test_mish_points_and_dims():
    # test/basis.jl:10-24: bDim = nc+3, mish points strictly inside and increasing
    s = O.OracleSpline(0.0, 10.0, 20)
    x = s.mish()
    assert s.bDim == 23 and s.mishDim == 60
    assert x[0] > 0.0 and x[-1] < 10.0 and np.all(np.diff(x) > 0)


def test_sa_variants_and_zero_ahat():
    # test/basis.jl:78-100: SA with ahat = 0 equals the plain SA
    s = O.OracleSpline(0.0, 10.0, 20)
    b = s.sb(np.sin(s.mish()))
    a1 = s.sa(b)
    a3 = s.sa(b, np.zeros_like(b))
    assert np.allclose(a1, a3, atol=1e-10)


def test_gamma_dense_matches_structured_fold():
    # GammaBC getindex vs mul!/adjoint (src/CubicBSpline.jl:336-500) through SA:
    # a = Γᵀ (Γ PQ Γᵀ)⁻¹ Γ b computed densely must equal the structured path.
    for bcl, bcr in [(R0, R0), (R1T0, R1T1), (R1T2, R2T10), (R2T20, R3), (R3, R1T0)]:
        s = O.OracleSpline(0.0, 50.0, 17, bcl=bcl, bcr=bcr)
        G = s.gamma()
        PQ = s.pq()
        b = s.sb(np.cos(s.mish() / 7.0))
        A = G @ PQ @ G.T
        a_dense = G.T @ np.linalg.solve(A, G @ b)
        a = s.sa(b)
        assert np.max(np.abs(a - a_dense)) <= 1e-10 * np.max(np.abs(a_dense))


def test_r3x_ahat_sets_boundary_values():
    # set_ahat_r3x! (src/CubicBSpline.jl:1460-1470): the R3X solution takes the
    # prescribed u, u', u'' at the boundary (test/r3x.jl:113-187 pattern)
    s = O.OracleSpline(0.0, 10.0, 12, bcl=R3X, bcr=R0)
    ahat = s.ahat_r3x(1.5, -0.25, 0.1, "left")
    b = s.sb(np.exp(-s.mish() / 5.0))
    a = s.sa(b, ahat)
    x0 = np.array([0.0])
    assert abs(s.si(a, 0, x0)[0] - 1.5) < 1e-12
    assert abs(s.si(a, 1, x0)[0] + 0.25) < 1e-12
    assert abs(s.si(a, 2, x0)[0] - 0.1) < 1e-12


# ---- banded Cholesky (test/banded_cholesky.jl:6-89) ------------------------
def spd_band3(n):
    B = np.zeros((n, n))
    for j in range(1, n + 1):
        for i in range(j, min(n, j + 3) + 1):
            B[i - 1, j - 1] = 1.0 / (1.0 + (i - j)) + 0.1 * (i + j)
    A = B @ B.T
    A = 0.5 * (A + A.T)
    A[np.diag_indices(n)] += 2.0
    return A


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 13, 53, 100, 200])
def test_band_cholesky_vs_dense(n):
    A = spd_band3(n)
    L4 = O.band_chol(A)
    b = np.arange(1, n + 1, dtype=float) + 0.5
    x_ref = np.linalg.solve(A, b)
    x = O.band_solve(L4, b)
    assert np.allclose(x, x_ref, rtol=1e-12, atol=1e-12)


def test_band_cholesky_bandwidth_assertion():
    A = spd_band3(10)
    A[0, 5] = A[5, 0] = 1.0
    with pytest.raises(O.OracleError) as e:
        O.band_chol(A)
    assert e.value.status == abi.SS_BAD_ARG


def test_band_cholesky_not_pd():
    n = 5
    A = np.zeros((n, n))
    for j in range(n):
        for i in range(max(0, j - 3), min(n, j + 4)):
            A[i, j] = -1.0 if i == j else 0.1
    with pytest.raises(O.OracleError) as e:
        O.band_chol(0.5 * (A + A.T))
    assert e.value.status == abi.SS_NOT_SPD


# ---- FFTW kinds vs pocketfft (independent implementation) -------------------
@pytest.mark.parametrize("n", [1, 2, 3, 8, 12, 17, 31, 64, 97, 126, 601, 1204, 2404, 4804])
def test_r2hc_hc2r_vs_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n)
    X = np.fft.rfft(x)
    ref = np.zeros(n)
    ref[0] = X[0].real
    for k in range(1, (n + 1) // 2):
        ref[k], ref[n - k] = X[k].real, X[k].imag
    if n % 2 == 0:
        ref[n // 2] = X[n // 2].real
    h = O.r2hc(x)
    assert np.max(np.abs(h - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))
    back = O.hc2r(h) / n
    assert np.max(np.abs(back - x)) <= 1e-13 * max(1.0, np.max(np.abs(x)))


@pytest.mark.parametrize("n", [2, 3, 8, 10, 25, 32, 33, 64])
def test_redft00_vs_scipy(n):
    import scipy.fft as sf

    x = np.random.default_rng(n).standard_normal(n)
    ref = sf.dct(x, type=1)
    assert np.max(np.abs(O.redft00(x) - ref)) <= 1e-13 * np.max(np.abs(ref))


# ---- Fourier (test/basis.jl:653-797) ---------------------------------------
def _ring_pts(yDim, ymin):
    return ymin + 2 * np.pi * np.arange(yDim) / yDim


def _ring_roundtrip(u, kmax, bDim, ymin):
    b = O.fourier_fb(u, kmax, bDim, ymin)
    a = O.fourier_fa(b, len(u), kmax, ymin)
    return O.fourier_fi(a, kmax, 0)


def test_fourier_roundtrip_ymin0():
    yDim, kmax, bDim = 64, 10, 21
    pts = _ring_pts(yDim, 0.0)
    for k in (1, 3, 10):
        u = np.sin(k * pts) + np.cos(k * pts)
        assert np.max(np.abs(_ring_roundtrip(u, kmax, bDim, 0.0) - u)) < 1e-10
    u = np.full(yDim, 3.14)
    assert np.max(np.abs(_ring_roundtrip(u, kmax, bDim, 0.0) - u)) < 1e-10
    u = np.cos(pts) + 0.5 * np.sin(3 * pts) + 0.25 * np.cos(7 * pts)
    assert np.max(np.abs(_ring_roundtrip(u, kmax, bDim, 0.0) - u)) < 1e-10


@pytest.mark.parametrize("ymin", [np.pi / 6, -np.pi / 4, np.pi / 3])
def test_fourier_roundtrip_phase_shift(ymin):
    yDim, kmax, bDim = 32, 8, 17
    pts = _ring_pts(yDim, ymin)
    for k in (1, 2, 5, 8):
        u = np.sin(k * pts) + 0.3 * np.cos(k * pts)
        assert np.max(np.abs(_ring_roundtrip(u, kmax, bDim, ymin) - u)) < 1e-10
    u = np.cos(pts) + 0.4 * np.sin(3 * pts) + 0.2 * np.cos(6 * pts)
    assert np.max(np.abs(_ring_roundtrip(u, kmax, bDim, ymin) - u)) < 1e-10


def test_fourier_amplitude_invariant_under_shift():
    for k in range(1, 5):
        bref = O.fourier_fb(np.cos(k * _ring_pts(16, 0.0)), 4, 9, 0.0)
        bsh = O.fourier_fb(np.cos(k * _ring_pts(16, np.pi / 4)), 4, 9, np.pi / 4)
        amp_ref = np.hypot(bref[k], bref[9 - k])
        amp_sh = np.hypot(bsh[k], bsh[9 - k])
        assert abs(amp_ref - amp_sh) < 1e-12


def test_fourier_derivatives():
    pts = _ring_pts(64, 0.0)
    k = 4
    b = O.fourier_fb(np.sin(k * pts), 8, 17, 0.0)
    a = O.fourier_fa(b, 64, 8, 0.0)
    assert np.max(np.abs(O.fourier_fi(a, 8, 1) - k * np.cos(k * pts))) < 1e-10
    k = 3
    b = O.fourier_fb(np.sin(k * pts), 8, 17, 0.0)
    a = O.fourier_fa(b, 64, 8, 0.0)
    assert np.max(np.abs(O.fourier_fi(a, 8, 2) + k * k * np.sin(k * pts))) < 1e-10


# ---- Chebyshev (test/basis.jl:1060-1164) -----------------------------------
def _cheb_roundtrip(u, zmin, zmax, bDim=None, bcb=0, bct=0, d=0):
    n = len(u)
    b = O.cheb_cb(u, bDim or n)
    a = O.cheb_ca(b, n, bcb, bct)
    return O.cheb_ci(a, zmin, zmax, d)


def test_chebyshev_roundtrip():
    z = O.cheb_mish(25, 0.0, np.pi)
    assert z[0] == pytest.approx(0.0) and z[-1] == pytest.approx(np.pi)
    for u in (np.sin(z), z**3 - 2 * z**2 + z + 1.0, np.cos(z) + 0.5 * np.sin(2 * z) + 0.25 * np.cos(3 * z)):
        assert np.max(np.abs(_cheb_roundtrip(u, 0.0, np.pi) - u)) < 1e-10


def test_chebyshev_derivatives():
    z = O.cheb_mish(33, 0.0, np.pi)
    assert np.max(np.abs(_cheb_roundtrip(np.sin(z), 0.0, np.pi, d=1) - np.cos(z))) < 1e-8
    assert np.max(np.abs(_cheb_roundtrip(np.sin(z), 0.0, np.pi, d=2) + np.sin(z))) < 1e-6


@pytest.mark.parametrize("bcb,bct", [(1, 0), (0, 1), (1, 1)])
def test_chebyshev_dirichlet_zeroes_boundary(bcb, bct):
    # CAtransform! with the R1T0 Γ (src/Chebyshev.jl:1001-1079) forces u = 0 at the
    # constrained ends: z = zmin is the first CGL point, zmax the last.
    z = O.cheb_mish(32, 0.0, 20000.0)
    u = np.cos(z / 5000.0) + 0.3
    out = _cheb_roundtrip(u, 0.0, 20000.0, bDim=22, bcb=bcb, bct=bct)
    if bcb == 1:
        assert abs(out[0]) < 1e-12
    if bct == 1:
        assert abs(out[-1]) < 1e-12


def test_chebyshev_gamma_unsupported_raises():
    with pytest.raises(O.OracleError) as e:
        O.cheb_gamma(8, 3, 0)
    assert e.value.status == abi.SS_UNSUPPORTED_BC
