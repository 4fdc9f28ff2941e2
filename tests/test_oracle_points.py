"""Oracle restatement of evaluate_unstructured and relocate_grid (src/interpolation.jl,
src/relocation.jl), pinned by the reference's own known-answer tests
(test/interpolation.jl:798-876, test/relocation.jl:1-120)."""
import math

import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S


def _axisym(gp, f):
    o = O.OracleGrid(gp.to_abi())
    pts = o.gridpoints()
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, 0, 0] = f(pts)
    return o, pts, o.spectral_transform(ph)


def test_unstructured_rl_axisymmetric():
    # test/interpolation.jl:798-833: sin(πr/40) on RL 10 cells, atol 0.05
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=40.0, num_cells=10)
    o, _, sp = _axisym(gp, lambda p: np.sin(math.pi * p[:, 0] / 40.0))
    pts = np.array([[10.0, 0.0], [15.0, math.pi / 4], [20.0, math.pi / 2], [25.0, math.pi],
                    [30.0, 3 * math.pi / 2], [5.0, 0.3]])
    res = O.evaluate_unstructured(gp.to_abi(), sp, pts)
    assert res.shape == (6, 1)
    assert np.max(np.abs(res[:, 0] - np.sin(math.pi * pts[:, 0] / 40.0))) < 0.05


def test_unstructured_rlz_axisymmetric():
    # test/interpolation.jl:835-875: RLZ 8 cells × 10 levels, atol 0.05
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=30.0, num_cells=8, kMin=0.0, kMax=10.0, kDim=10)
    o, _, sp = _axisym(gp, lambda p: np.sin(math.pi * p[:, 0] / 30.0))
    pts = np.array([[5.0, 0.0, 5.0], [10.0, math.pi / 4, 2.0], [15.0, math.pi / 2, 7.0], [20.0, math.pi, 4.0],
                    [25.0, 3 * math.pi / 2, 8.0]])
    res = O.evaluate_unstructured(gp.to_abi(), sp, pts)
    assert np.max(np.abs(res[:, 0] - np.sin(math.pi * pts[:, 0] / 30.0))) < 0.05


def test_unstructured_out_of_bounds():
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=40.0, num_cells=10)
    _, _, sp = _axisym(gp, lambda p: np.sin(math.pi * p[:, 0] / 40.0))
    pts = np.array([[10.0, 0.0], [45.0, 0.0]])
    res = O.evaluate_unstructured(gp.to_abi(), sp, pts)
    assert np.isfinite(res[0, 0]) and np.isnan(res[1, 0])
    assert O.evaluate_unstructured(gp.to_abi(), sp, pts, -999.0)[1, 0] == -999.0
    with pytest.raises(ValueError):
        O.evaluate_unstructured(gp.to_abi(), sp, pts, "error")


def _vortex(nc=10):
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=10.0, num_cells=nc)
    o, pts, sp = _axisym(gp, lambda p: np.exp(-p[:, 0] ** 2 / 4.0))
    return gp, o, pts, sp


def _relocate(gp, o, pts, sp, shift, boundary):
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, :, 0] = O.relocated_slot1(gp.to_abi(), sp, pts, shift[0], shift[1], boundary)
    sp2 = o.spectral_transform(ph)
    return sp2, o.grid_transform(sp2)


def test_relocation_kats():
    # test/relocation.jl:42-106
    gp, o, pts, sp = _vortex(15)
    g0 = o.grid_transform(sp)[:, 0, 0]
    sp2, g2 = _relocate(gp, o, pts, sp, (0.3, 0.2), "azimuthal_mean")
    assert not np.any(np.isnan(g2[:, 0, 0]))
    _, g3 = _relocate(gp, o, pts, sp2, (-0.3, -0.2), "azimuthal_mean")
    inner = pts[:, 0] < 8.0
    assert np.max(np.abs(g3[inner, 0, 0] - g0[inner])) < 0.2
    _, g4 = _relocate(gp, o, pts, sp, (0.1, 0.0), "azimuthal_mean")
    m = pts[:, 0] < 5.0
    assert abs(g0[m].mean() - g4[m, 0, 0].mean()) / abs(g0[m].mean()) < 0.1
    gp, o, pts, sp = _vortex()
    assert np.any(np.isnan(_relocate(gp, o, pts, sp, (8.0, 0.0), "nan")[1][:, 0, 0]))
    for b in ("nearest", "azimuthal_mean"):
        assert not np.any(np.isnan(_relocate(gp, o, pts, sp, (8.0, 0.0), b)[1][:, 0, 0]))
