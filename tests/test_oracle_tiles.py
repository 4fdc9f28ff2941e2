"""Tile pipeline of the oracle: splineTransform! then tileTransform!
(src/tiling.jl:1490-1660 RL, 1862-2046 RLZ), pinned by the reference's own
round trips (test/tiling.jl:159-205, 297-330) and by the identity with
gridTransform! when no R3X background or filter is set."""
import numpy as np

import oracle as O
from springsteel_gpu import abi


def _roundtrip(g, f):
    pts = g.gridpoints()
    ph = np.zeros(g.physical_shape, order="F")
    ph[:, 0, 0] = f(pts)
    shared = g.spectral_transform(ph)
    a = g.spline_transform(shared)
    return pts, shared, a, g.tile_transform(a)


def test_rl_distributed_pipeline():
    # test/tiling.jl:159-205: RL, 12 cells on [0, 100], R0 both ends, f = sin(π r / 100)
    g = O.OracleGrid(abi.make_params(abi.SS_GEOM_RL, 12, 0.0, 100.0, 1))
    pts, shared, a, out = _roundtrip(g, lambda p: np.sin(np.pi * p[:, 0] / 100.0))
    r = pts[:, 0]
    assert np.max(np.abs(out[:, 0, 0] - np.sin(np.pi * r / 100.0))) < 5e-4
    assert np.max(np.abs(out[:, 0, 1] - (np.pi / 100.0) * np.cos(np.pi * r / 100.0))) < 0.05
    assert np.max(np.abs(out[:, 0, 3])) < 1e-10
    assert np.all(np.isfinite(out))
    # the pipeline is gridTransform! split in two: identical without ahat or filter
    ref = g.grid_transform(shared)
    assert np.max(np.abs(out - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_rlz_distributed_pipeline():
    # test/tiling.jl:297-330: RLZ, 9 cells on [0, 75], z ∈ [0, 10] with 6 levels,
    # R0 everywhere, f = sin(π r / 75) · z / 10
    g = O.OracleGrid(abi.make_params(abi.SS_GEOM_RLZ, 9, 0.0, 75.0, 1, kDim=6, kMin=0.0, kMax=10.0))
    pts, shared, a, out = _roundtrip(g, lambda p: np.sin(np.pi * p[:, 0] / 75.0) * (p[:, 2] / 10.0))
    want = np.sin(np.pi * pts[:, 0] / 75.0) * (pts[:, 2] / 10.0)
    assert np.max(np.abs(out[:, 0, 0] - want)) < 1e-3
    assert np.max(np.abs(out[:, 0, 3])) < 1e-8
    assert np.all(np.isfinite(out))
    ref = g.grid_transform(shared)
    assert np.max(np.abs(out - ref)) <= 1e-13 * max(1.0, np.max(np.abs(ref)))


def test_spline_transform_is_blockwise_sa_without_background():
    """Each block of the result is the 1-D SAtransform(spline, b) of the same block,
    even for an R3X boundary with a registered background (the two-argument form)."""
    bcl = [(abi.SS_SBC_R3X, 0.0, 0.0)]
    g = O.OracleGrid(abi.make_params(abi.SS_GEOM_RL, 6, 0.0, 30.0, 1, BCL=bcl))
    b = g.dims["b_iDim"]
    rng = np.random.default_rng(4)
    shared = np.asfortranarray(rng.standard_normal(g.spectral_shape))
    g.set_ahat(0, 1, rng.standard_normal(b))
    a = g.spline_transform(shared)
    sp = O.OracleSpline(0.0, 30.0, 6, bcl=bcl[0])
    for q in range(shared.shape[0] // b):
        want = sp.sa(shared[q * b:(q + 1) * b, 0])
        assert np.max(np.abs(a[q * b:(q + 1) * b, 0] - want)) <= 1e-13 * max(1.0, np.max(np.abs(want)))
