"""evaluate_unstructured and relocate_grid on the GPU through the C ABI against the
oracle's restatement (src/interpolation.jl:1628-1850, src/relocation.jl:144-439)."""
import math

import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from test_gpu_multi import _fill
from test_gpu_parity import TOL64, slot_errors

pytestmark = pytest.mark.gpu


def _grid(geometry, precision="f64"):
    kw = dict(vars={"u": 1, "w": 2}, BCL={"u": S.DirichletBC()}, BCR={"w": S.NeumannBC()}, precision=precision)
    if geometry == "RL":
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=30.0, num_cells=15, **kw)
    else:
        gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=24.0, num_cells=12, kMin=0.0, kMax=400.0,
                                         kDim=10, BCB={"default": S.DirichletBC()}, **kw)
    g = S.createGrid(gp)
    _fill(g, seed=9)
    S.spectralTransform_b(g)
    return gp, g


@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
def test_evaluate_unstructured_matches_oracle(geometry):
    gp, g = _grid(geometry)
    rng = np.random.default_rng(4)
    n = 300
    pts = np.column_stack([rng.uniform(-2.0, gp.iMax + 2.0, n), rng.uniform(-math.pi, 3 * math.pi, n)]
                          + ([rng.uniform(-20.0, gp.kMax + 20.0, n)] if geometry == "RLZ" else []))
    spec = g.get_spectral()
    ref = O.evaluate_unstructured(gp.to_abi(), spec, pts)
    got = S.evaluate_unstructured(g, pts)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    scale = np.nanmax(np.abs(ref), axis=0)
    assert np.all(np.abs(got - ref)[ok] <= TOL64 * np.repeat(scale[None], n, 0)[ok])
    fill = S.evaluate_unstructured(g, pts, out_of_bounds=-7.0)
    assert np.all(fill[~ok] == -7.0) and np.array_equal(fill[ok], got[ok])
    with pytest.raises(ValueError):
        S.evaluate_unstructured(g, pts, out_of_bounds="error")
    only_w = S.evaluate_unstructured(g, pts, vars=["w"])
    assert np.all(np.isnan(only_w[:, 0])) and np.array_equal(only_w[ok[:, 1], 1], got[ok[:, 1], 1])
    g.close()


@pytest.mark.parametrize("geometry,boundary,taper", [("RL", "azimuthal_mean", 0), ("RL", "nearest", 3),
                                                     ("RLZ", "azimuthal_mean", 2), ("RLZ", "nearest", 0)])
def test_relocate_matches_oracle(geometry, boundary, taper):
    gp, g = _grid(geometry)
    o = O.OracleGrid(gp.to_abi())
    pts = o.gridpoints()
    spec = g.get_spectral()
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, :, 0] = O.relocated_slot1(gp.to_abi(), spec, pts, 2.5, -1.5, boundary, taper)
    ref = o.grid_transform(o.spectral_transform(ph))
    g2 = S.relocate_grid(g, (2.5, -1.5), boundary=boundary, taper_width=taper)
    errs = slot_errors(g2.get_physical(), ref, gp)
    assert np.all(errs <= TOL64), errs
    # relocate_grid! in place gives the same fields and moves the centre
    S.relocate_grid_b(g, (2.5, -1.5), boundary=boundary, taper_width=taper)
    assert np.array_equal(g.get_physical(), g2.get_physical())
    assert S.grid_center(g) == (2.5, -1.5)
    g.close()
    g2.close()


def test_relocate_nan_boundary_marks_out_of_range_points():
    # test/relocation.jl:86-90: a shift of 8 on a radius-10 grid leaves NaN with :nan
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=10.0, num_cells=10)
    g = S.createGrid(gp)
    pts = S.getGridpoints(g)
    g.set_physical(np.exp(-pts[:, 0] ** 2 / 4.0)[:, None], slot=1)
    S.spectralTransform_b(g)
    S.gridTransform_b(g)
    assert np.any(np.isnan(S.relocate_grid(g, (8.0, 0.0), boundary="nan").get_physical()[:, 0, 0]))
    for b in ("nearest", "azimuthal_mean"):
        assert not np.any(np.isnan(S.relocate_grid(g, (8.0, 0.0), boundary=b).get_physical()[:, 0, 0]))
