"""CPU checks of the elliptic-solve oracle, the MLP oracle and the tile halo sum.

The reference has no RL elliptic solve, so the oracle's per-wavenumber Galerkin
solve is pinned by a manufactured solution: the error against the analytic u
must be small and fall at the spline's rate as the grid is refined.  The MLP
oracle's gradient formulas are pinned by finite differences.
"""
import math

import numpy as np
import pytest

import mlp_oracle as M
import oracle as O
import springsteel_gpu as S
from springsteel_gpu import fields


class _HostGrid:
    """Enough of a grid for getGridpoints without a device."""

    def __init__(self, gp):
        self.params = gp
        self.dims = O.OracleGrid(gp.to_abi()).dims


def _manufactured(r, lam, R):
    s = r / R
    g0 = (1 - s * s) ** 2
    g2 = 0.3 * s * s * (1 - s * s) ** 2
    return g0 + g2 * np.cos(2 * lam)


def _forcing(r, lam, R, k2):
    # L[g(r) cos(mλ)] = (g'' + g'/r − m² g/r² − k² g) cos(mλ), done symbolically
    import sympy as sp

    rs = sp.symbols("r", positive=True)
    s = rs / R
    out = np.zeros_like(r)
    for m, g in ((0, (1 - s ** 2) ** 2), (2, sp.Rational(3, 10) * s ** 2 * (1 - s ** 2) ** 2)):
        expr = sp.diff(g, rs, 2) + sp.diff(g, rs) / rs - m * m * g / rs ** 2 - k2 * g
        f = sp.lambdify(rs, sp.simplify(expr), "numpy")
        out += f(r) * np.cos(m * lam)
    return out


@pytest.mark.parametrize("nc", [20, 40])
def test_manufactured_solution(nc):
    R, k2 = 50.0, 0.01
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=R, num_cells=nc)
    og = O.OracleGrid(gp.to_abi())
    pts = S.getGridpoints(_HostGrid(gp))
    r, lam = pts[:, 0], pts[:, 1]
    el = O.OracleElliptic(og, np.full(og.dims["iDim"], k2))
    out, _ = el.solve(_forcing(r, lam, R, k2)[:, None])
    err = np.max(np.abs(out[:, 0, 0] - _manufactured(r, lam, R)))
    assert err < (2e-3 if nc == 20 else 5e-4), err


def test_manufactured_solution_converges():
    R, k2 = 50.0, 0.01
    errs = []
    for nc in (20, 40, 80):
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=R, num_cells=nc)
        og = O.OracleGrid(gp.to_abi())
        pts = S.getGridpoints(_HostGrid(gp))
        el = O.OracleElliptic(og, np.full(og.dims["iDim"], k2))
        out, _ = el.solve(_forcing(pts[:, 0], pts[:, 1], R, k2)[:, None])
        errs.append(np.max(np.abs(out[:, 0, 0] - _manufactured(pts[:, 0], pts[:, 1], R))))
    assert errs[1] < errs[0] / 3 and errs[2] < errs[1] / 3, errs


def test_operator_band_structure():
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=30.0, num_cells=12)
    og = O.OracleGrid(gp.to_abi())
    el = O.OracleElliptic(og, fields.k2_profile(fields.radial_mish(gp), seed=3))
    for m in (0, 1, 5):
        G = el.operator(m)
        i, j = np.nonzero(G)
        assert np.max(np.abs(i - j)) <= 4
        assert np.all(np.isfinite(G))


# ---------------------------------------------------------------- MLP oracle
def test_bf16_rounding_matches_torch():
    import torch

    x = np.random.default_rng(0).normal(size=4096).astype(np.float32) * 10.0 ** np.random.default_rng(1).integers(-8, 8, 4096)
    ref = torch.from_numpy(x).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(M.bf16(x), ref)


def test_mlp_oracle_gradients_finite_difference():
    rng = np.random.default_rng(5)
    B = 8
    W = rng.normal(0, math.sqrt(2 / 256), (3, 256, 256))
    b = rng.normal(0, 0.1, (3, 256))
    x = rng.normal(size=(B, 256))
    t = rng.normal(size=(B, 256))
    n = rng.integers(100, 257, B)
    L, dW, db = M.loss_and_gradients(W, b, x, t, n, exact=True)
    h = 1e-6
    for (l, o, i) in [(0, 3, 7), (1, 100, 200), (2, 5, 17), (2, 250, 1)]:
        Wp, Wm = W.copy(), W.copy()
        Wp[l, o, i] += h
        Wm[l, o, i] -= h
        fd = (M.loss_and_gradients(Wp, b, x, t, n, exact=True)[0] - M.loss_and_gradients(Wm, b, x, t, n, exact=True)[0]) / (2 * h)
        assert abs(fd - dW[l, o, i]) <= 1e-6 * max(1.0, abs(fd)), (l, o, i, fd, dW[l, o, i])
    for (l, o) in [(0, 9), (2, 3)]:
        bp, bm = b.copy(), b.copy()
        bp[l, o] += h
        bm[l, o] -= h
        fd = (M.loss_and_gradients(W, bp, x, t, n, exact=True)[0] - M.loss_and_gradients(W, bm, x, t, n, exact=True)[0]) / (2 * h)
        assert abs(fd - db[l, o]) <= 1e-6 * max(1.0, abs(fd))


# ---------------------------------------------------------------- tiles
def test_oracle_tile_b_vectors_sum_to_patch():
    """spectralTransform! leaves B-vectors (quadrature sums), so the tiles' halo sum
    (sumSpectralTile!, src/tiling.jl:1101-1136) reproduces the patch exactly."""
    from test_gpu_multi import _sum_spectral_tile

    gp = fields.rlz_params(num_cells=24, nvars=1, kDim=8)
    op = O.OracleGrid(gp.to_abi())
    pts = S.getGridpoints(_HostGrid(gp))
    u = fields.blob_sum(pts, seed=3, nblobs=6, wmin=3.0, wmax=12.0, zmax=20000.0)
    ph = np.zeros(op.physical_shape, order="F")
    ph[:, 0, 0] = u
    ref = op.spectral_transform(ph)
    acc = np.zeros_like(ref)
    row0 = 0
    for tp in S.calcTileSizes(gp, 4):
        ot = O.OracleGrid(tp.to_abi())
        n = ot.physical_shape[0]
        pt = np.zeros(ot.physical_shape, order="F")
        pt[:, 0, 0] = u[row0:row0 + n]
        row0 += n
        _sum_spectral_tile(acc, ot.spectral_transform(pt), gp, tp)
    assert row0 == u.shape[0]
    assert np.max(np.abs(acc - ref)) <= 1e-14 * np.max(np.abs(ref))
