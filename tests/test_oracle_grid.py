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


def test_unsupported_spline_periodic():
    with pytest.raises(O.OracleError) as e:
        _rl(4, 10.0, BCL=[(abi.SS_SBC_PERIODIC, 0, 0)], BCR=[(abi.SS_SBC_PERIODIC, 0, 0)])
    assert e.value.status == abi.SS_UNSUPPORTED_BC
