"""Grid-level known-answer tests of the oracle (test/transforms.jl:521-907)."""
import numpy as np
import pytest

import oracle as O
from springsteel_gpu import abi


def _rl(nc, imax, nvars=1, pOL=0, **kw):
    return O.OracleGrid(abi.make_params(abi.SS_GEOM_RL, nc, 0.0, imax, nvars, patchOffsetL=pOL, **kw))


def _rlz(nc, imax, kdim, kmax, pOL=0, **kw):
    return O.OracleGrid(abi.make_params(abi.SS_GEOM_RLZ, nc, 0.0, imax, 1, kDim=kdim, kMin=0.0,
                                        kMax=kmax, patchOffsetL=pOL, **kw))


def _phys(g, f):
    pts = g.gridpoints()
    ph = np.zeros(g.physical_shape, order="F")
    ph[:, 0, 0] = f(pts)
    return ph, pts


def test_rl_dims_match_factory():
    g = _rl(10, 100.0)
    d = g.dims
    assert d["iDim"] == 30 and d["b_iDim"] == 13 and d["kDim_wn"] == 30
    assert d["jDim"] == sum(4 + 4 * r for r in range(1, 31))
    assert d["n_spectral"] == 13 * (1 + 2 * 30)


def test_rl_wavenumber0_roundtrip():
    # test/transforms.jl:521-555
    g = _rl(10, 100.0)
    ph, pts = _phys(g, lambda p: p[:, 0])
    sp = g.spectral_transform(ph)
    assert np.max(np.abs(sp)) > 1e-10
    out = g.grid_transform(sp)
    assert np.max(np.abs(out[:, 0, 0] - pts[:, 0])) < 1e-3
    assert np.max(np.abs(out[:, 0, 1] - 1.0)) < 0.05
    assert np.max(np.abs(out[:, 0, 2])) < 0.05


def test_rl_wavenumber1_roundtrip():
    # test/transforms.jl:557-589
    g = _rl(10, 100.0)
    ph, pts = _phys(g, lambda p: p[:, 0] * np.cos(p[:, 1]))
    out = g.grid_transform(g.spectral_transform(ph))
    assert np.max(np.abs(out[:, 0, 0] - ph[:, 0, 0])) < 1e-2
    assert np.max(np.abs(out[:, 0, 3])) > 1e-6
    # ∂λ(r cos λ) = -r sin λ, ∂λλ = -r cos λ (exact for a linear-in-r wavenumber-1 field)
    assert np.max(np.abs(out[:, 0, 3] + pts[:, 0] * np.sin(pts[:, 1]))) < 1e-9
    assert np.max(np.abs(out[:, 0, 4] + pts[:, 0] * np.cos(pts[:, 1]))) < 1e-9


def test_rl_multivariable():
    # test/transforms.jl:591-620
    g = _rl(8, 80.0, nvars=2)
    pts = g.gridpoints()
    ph = np.zeros(g.physical_shape, order="F")
    ph[:, 0, 0] = pts[:, 0]
    ph[:, 1, 0] = 2.0 * pts[:, 0]
    out = g.grid_transform(g.spectral_transform(ph))
    assert np.max(np.abs(out[:, 0, 0] - ph[:, 0, 0])) < 1e-3
    assert np.max(np.abs(out[:, 1, 0] - ph[:, 1, 0])) < 1e-3


def test_rl_derivative_accuracy():
    # test/transforms.jl:622-651
    g = _rl(12, 100.0)
    ph, _ = _phys(g, lambda p: p[:, 0] / 100.0)
    out = g.grid_transform(g.spectral_transform(ph))
    assert np.max(np.abs(out[:, 0, 1] - 0.01)) < 0.05
    assert np.max(np.abs(out[:, 0, 3])) < 0.05


def test_rlz_roundtrip():
    # test/transforms.jl:785-824
    g = _rlz(4, 60.0, 8, 10.0)
    ph, pts = _phys(g, lambda p: p[:, 0] * np.cos(p[:, 1]) * p[:, 2])
    sp = g.spectral_transform(ph)
    assert np.max(np.abs(sp)) > 1e-10
    out = g.grid_transform(sp)
    assert np.max(np.abs(out[:, 0, 0] - ph[:, 0, 0])) < 1e-2
    # ∂z = r cos λ, ∂zz = 0
    assert np.max(np.abs(out[:, 0, 5] - pts[:, 0] * np.cos(pts[:, 1]))) < 1e-9
    assert np.max(np.abs(out[:, 0, 6])) < 1e-8


def test_rlz_patch_offset_bug1_regression():
    # test/transforms.jl:826-869 (patchOffsetL = 3)
    g = _rlz(4, 40.0, 8, 10.0, pOL=3)
    ph, _ = _phys(g, lambda p: p[:, 0] * p[:, 2])
    out = g.grid_transform(g.spectral_transform(ph))
    assert np.max(np.abs(out[:, 0, 0] - ph[:, 0, 0])) < 1e-2


def test_rlz_radial_derivative():
    # test/transforms.jl:871-907
    g = _rlz(6, 100.0, 10, 20.0)
    ph, _ = _phys(g, lambda p: p[:, 0] / 100.0)
    out = g.grid_transform(g.spectral_transform(ph))
    assert np.max(np.abs(out[:, 0, 1] - 0.01)) < 0.05
    assert np.max(np.abs(out[:, 0, 3])) < 0.05


def test_rlz_physical_order_z_fastest():
    # getGridpoints RLZ (src/transforms_cylindrical.jl:454-476): z fastest, then λ, then r
    g = _rlz(2, 10.0, 5, 1.0)
    pts = g.gridpoints()
    z = g.column_points()
    assert np.allclose(pts[:5, 2], z) and np.all(pts[:5, 0] == pts[0, 0])
    assert pts[5, 1] > pts[0, 1]


def test_filter_zero_weights_kill_wavenumbers():
    # applyFilter! (src/filtering.jl:320-364) with a hard low-pass at k = 2
    g = _rl(6, 60.0)
    K = g.dims["kDim_wn"]
    w = np.ones(K + 1)
    w[3:] = 0.0
    g.set_filter(0, w)
    ph, _ = _phys(g, lambda p: p[:, 0] * (np.cos(p[:, 1]) + np.cos(4 * p[:, 1])))
    sp = g.spectral_transform(ph)
    b = g.dims["b_iDim"]
    assert np.all(sp[(2 * 3 - 1) * b:, 0] == 0.0)
    assert np.max(np.abs(sp[b:3 * b, 0])) > 0


def test_dirichlet_bc_in_z():
    g = _rlz(3, 30.0, 12, 100.0, BCB=[abi.SS_CBC_R1T0], BCT=[abi.SS_CBC_R1T0])
    ph, pts = _phys(g, lambda p: 1.0 + 0.01 * p[:, 0] * np.sin(p[:, 2] / 30.0))
    out = g.grid_transform(g.spectral_transform(ph))
    kz = g.dims["kDim"]
    assert np.max(np.abs(out[0::kz, 0, 0])) < 1e-12
    assert np.max(np.abs(out[kz - 1::kz, 0, 0])) < 1e-12


def test_periodic_spline_grid_builds():
    # PERIODIC is a GammaBC kind with a dense factor (src/banded_cholesky.jl:70, 250-260)
    g = _rl(4, 10.0, BCL=[(abi.SS_SBC_PERIODIC, 0, 0)], BCR=[(abi.SS_SBC_PERIODIC, 0, 0)])
    assert g.dims["b_iDim"] == 7


def _rlz_spectral_wavenumber_norms(gp):
    """max |coefficient| per Fourier wavenumber k of an RLZ oracle transform of a
    field rich in λ (all variables), spectral layout [z_b][k0 | k1 re | k1 im | …][b]."""
    o = O.OracleGrid(gp.to_abi())
    pts = o.gridpoints()
    ph = np.zeros(o.physical_shape, order="F")
    for v in range(o.physical_shape[1]):
        ph[:, v, 0] = sum(np.cos(k * pts[:, 1] + 0.3 * v) for k in range(12)) * (1 + pts[:, 0] / 10.0)
    sp = o.spectral_transform(ph)
    d = o.dims
    b, K = d["b_iDim"], d["kDim_wn"]
    blocks = sp.reshape(d["b_kDim"], 1 + 2 * K, b, -1)
    return np.array([np.max(np.abs(blocks[:, 0 if k == 0 else 2 * k - 1: 1 if k == 0 else 2 * k + 1]))
                     for k in range(K + 1)])


@pytest.mark.parametrize("vars_, mw, expect", [
    ({"a": 1, "b": 2, "c": 3}, {"default": -1, "a": 3, "b": 5}, 5),   # last key with an entry: b
    ({"c": 3, "b": 2, "a": 1}, {"default": -1, "a": 3, "b": 5}, 3),   # iteration order c, b, a: a wins
    ({"a": 1, "b": 2}, {"default": 4}, 4),                            # no own entry: the default
    ({"a": 1, "b": 2}, {"default": 2, "a": -1}, None),                # an own -1 lifts the default cap
])
def test_rlz_shared_ring_kmax_rule(vars_, mw, expect):
    """RLZ rings are shared by every variable; their kmax is the default entry
    overridden by each variable's own entry in vars order (src/factory.jl:730-733)."""
    import springsteel_gpu as S

    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=10.0, num_cells=4, kMin=0.0, kMax=1.0,
                                     kDim=6, vars=vars_, max_wavenumber=mw)
    assert gp.shared_ring_kmax() == (-1 if expect is None else expect)
    norms = _rlz_spectral_wavenumber_norms(gp)
    if expect is None:
        assert np.all(norms[1:12] > 1e-8)
    else:
        assert np.all(norms[: expect + 1] > 1e-8), norms
        assert np.all(norms[expect + 1:] == 0.0), norms
