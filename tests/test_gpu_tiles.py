"""Tile pipeline on the GPU through the C ABI: ss_spline_transform
(splineTransform!, src/tiling.jl:1490-1516 RL, 1862-1892 RLZ) and
ss_tile_transform (tileTransform!, :1540-1660 RL, :1915-2046 RLZ) against the
oracle's restatement of both, on the same B-vectors."""
import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from test_gpu_multi import _fill
from test_gpu_parity import TOL64, TOL_FAST, _rel, slot_errors

pytestmark = pytest.mark.gpu

# binary32 bulk: coefficients from the FP32 solve refined once in FP64; the
# slots carry the binary32 rounding of the ring and column transforms
TOL = {"f64": (TOL64, TOL64), "f64_fast": (TOL64, TOL_FAST), "f32": (2e-6, 1e-4)}


def _params(geometry, precision):
    vars_ = {"u": 1, "w": 2}
    bcl = {"u": S.DirichletBC(), "w": S.NeumannBC()}
    bcr = {"u": S.NaturalBC(), "w": S.RobinBC(1.0, -2.0)}
    if geometry == "RL":
        return S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=42.0, num_cells=14, vars=vars_,
                                           BCL=bcl, BCR=bcr, patchOffsetL=3, precision=precision)
    return S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=30.0, num_cells=10, vars=vars_,
                                       BCL=bcl, BCR=bcr, kMin=0.0, kMax=10.0, kDim=12,
                                       BCB={"default": S.DirichletBC()}, BCT={"default": S.NeumannBC()},
                                       precision=precision)


@pytest.mark.parametrize("precision", ["f64", "f64_fast", "f32"])
@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
def test_spline_and_tile_transform_match_oracle(geometry, precision):
    gp = _params(geometry, precision)
    o = O.OracleGrid(gp.to_abi())
    shared = S.createGrid(gp)  # holds the B-vectors, as the reference's SharedArray does
    tile = S.createGrid(gp)
    u = _fill(shared, seed=7)
    S.spectralTransform_b(shared)
    b_gpu = shared.get_spectral()
    a_o = o.spline_transform(b_gpu)  # same B-vectors on both sides
    phys_o = o.tile_transform(a_o)
    tol_a, tol_p = TOL[precision]
    for _ in range(2):  # twice in a row: no state carried between calls
        S.splineTransform_b(shared, tile)
        a_g = tile.get_spectral()
        for v in range(a_o.shape[1]):
            assert _rel(a_g[:, v], a_o[:, v]) <= tol_a, (v, _rel(a_g[:, v], a_o[:, v]))
        S.tileTransform_b(shared, tile)
        errs = slot_errors(tile.get_physical(), phys_o, gp)
        print("tile pipeline %s %s: coefficients %.2e, slots %s" % (
            geometry, precision, max(_rel(a_g[:, v], a_o[:, v]) for v in range(a_o.shape[1])),
            np.array2string(errs.max(axis=0), precision=2)))
        assert np.all(errs <= tol_p), errs
    # in place: the tile's own spectral array as the shared one
    tile.set_spectral(b_gpu.astype(np.float32) if precision == "f32" else b_gpu)
    S.splineTransform_b(None, tile)
    a_in = tile.get_spectral()
    assert np.array_equal(a_in, a_g)
    del u
    shared.close()
    tile.close()


def test_tile_pipeline_equals_grid_transform_without_background():
    """With no R3X background and no filter, splineTransform! followed by
    tileTransform! is gridTransform! split in two (FP64, bit-level agreement not
    required: the two paths run the same solve and evaluation kernels)."""
    gp = _params("RLZ", "f64")
    g = S.createGrid(gp)
    _fill(g, seed=3)
    S.spectralTransform_b(g)
    S.gridTransform_b(g)
    ref = g.get_physical()
    S.splineTransform_b(None, g)
    S.tileTransform_b(None, g)
    out = g.get_physical()
    assert np.max(np.abs(out - ref)) <= 1e-13 * np.max(np.abs(ref))
    g.close()
