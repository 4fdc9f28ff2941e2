"""Known-answer checks of the oracle's regularGridTransform restatement
(src/transforms_cylindrical.jl:929-1020, 1168-1287) and of the regular point
sets (getRegularGridpoints, :860-898, 1100-1138), on CPU."""
import numpy as np

import oracle as O
import springsteel_gpu as S


def _rl_linear_cos():
    # f(r, λ) = r cos λ (test/interpolation.jl "RL grid" field)
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=5.0, iMax=50.0, num_cells=8)
    o = O.OracleGrid(gp.to_abi())
    pts = o.gridpoints()
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, 0, 0] = pts[:, 0] * np.cos(pts[:, 1])
    return gp, o.spectral_transform(ph)


def test_regular_points_follow_the_reference():
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=5.0, iMax=50.0, num_cells=8)
    r, lam, z = S.regular_axes(gp)
    assert len(r) == 9 and len(lam) == 2 * 24 + 1 and z is None
    assert r[0] == 5.0 and r[-1] == 50.0 and lam[0] == 0.0
    assert np.allclose(np.diff(lam), 2 * np.pi / len(lam))
    pts = S.getRegularGridpoints(gp)
    assert pts.shape == (9 * 49, 2) and np.all(pts[:49, 0] == 5.0) and np.all(pts[:49, 1] == lam)
    gz = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=10.0, num_cells=4, kMin=0.0, kMax=2.0, kDim=8)
    pz = S.getRegularGridpoints(gz)
    assert pz.shape == (5 * 25 * 9, 3) and np.all(pz[:9, 2] == np.linspace(0.0, 2.0, 9))


def test_rl_regular_output_of_r_cos_lambda():
    gp, spec = _rl_linear_cos()
    r, lam, _ = S.regular_axes(gp)
    out = O.regular_grid_transform(gp.to_abi(), spec, r, lam)
    R, L = np.meshgrid(r, lam, indexing="ij")
    R, L = R.reshape(-1), L.reshape(-1)
    assert np.max(np.abs(out[:, 0, 0] - R * np.cos(L))) < 1e-8 * 50
    assert np.max(np.abs(out[:, 0, 1] - np.cos(L))) < 1e-8
    assert np.max(np.abs(out[:, 0, 2])) < 1e-8
    assert np.max(np.abs(out[:, 0, 3] + R * np.sin(L))) < 1e-8 * 50
    assert np.max(np.abs(out[:, 0, 4] + R * np.cos(L))) < 1e-8 * 50


def test_rlz_regular_output_of_r_z_cos_lambda():
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=5.0, iMax=50.0, num_cells=8, kMin=0.0, kMax=10.0,
                                     kDim=12)
    o = O.OracleGrid(gp.to_abi())
    pts = o.gridpoints()
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, 0, 0] = pts[:, 0] * np.cos(pts[:, 1]) * pts[:, 2]
    spec = o.spectral_transform(ph)
    r, lam, z = S.regular_axes(gp)
    out = O.regular_grid_transform(gp.to_abi(), spec, r, lam, z)
    R, L, Z = [a.reshape(-1) for a in np.meshgrid(r, lam, z, indexing="ij")]
    f = R * np.cos(L) * Z
    assert np.max(np.abs(out[:, 0, 0] - f)) < 1e-7 * 500
    assert np.max(np.abs(out[:, 0, 1] - np.cos(L) * Z)) < 1e-7 * 10
    assert np.max(np.abs(out[:, 0, 3] + R * np.sin(L) * Z)) < 1e-7 * 500
    assert np.max(np.abs(out[:, 0, 5] - R * np.cos(L))) < 1e-6 * 50
