"""regularGridTransform on the GPU (ss_regular_grid_transform) against the oracle's
restatement of src/transforms_cylindrical.jl:929-1020 (RL) and 1168-1287 (RLZ),
on the reference's default regular point sets (getRegularGridpoints).

Tolerance: 1e-12 relative to each slot's scale (the parity norm of the other GPU
tests).  The RLZ ∂zz slot at the two end levels z = kMin, kMax is the one
exception: there the reference's formula (d²f/dt²·sin t − df/dt·cos t)/(s² sin³ t)
is evaluated at t ≈ 1.4e-5 (its clamp |ξ| ≤ 1 − 1e-10), where the cancellation
amplifies rounding by about 1/sin²t ≈ 5e9; those rows are compared at 1e-5.
"""
import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from springsteel_gpu import fields
from test_gpu_parity import SLOT_DERIV

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _slot_err(got, ref, gp, rows=None):
    lengths = {"r": gp.iMax - gp.iMin, "l": 1.0, "z": (gp.kMax - gp.kMin) or 1.0}
    out = np.zeros(ref.shape[1:])
    for v in range(ref.shape[1]):
        fmax = np.max(np.abs(ref[:, v, 0]))
        for s in range(ref.shape[2]):
            dirn, d = SLOT_DERIV[s]
            den = max(np.max(np.abs(ref[:, v, s])), fmax / lengths[dirn] ** d if dirn else 0.0)
            sel = slice(None) if rows is None else rows
            out[v, s] = np.max(np.abs(got[sel, v, s] - ref[sel, v, s])) / den
    return out


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_rl_regular_grid_matches_oracle(precision):
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=60.0, num_cells=30, vars={"u": 1, "w": 2},
                                     BCL={"u": S.NaturalBC(), "w": S.NeumannBC()}, precision=precision)
    g = S.createGrid(gp)
    pts = S.getGridpoints(g)
    u = np.column_stack([fields.blob_sum(pts, seed=40 + v, nblobs=5, wmin=4, wmax=15) for v in range(2)])
    g.set_physical(u, slot=1)
    S.spectralTransform_b(g)
    spec = g.get_spectral()
    reg = S.getRegularGridpoints(g)
    got = S.regularGridTransform(g, reg)
    r, lam, _ = S.regular_axes(gp)
    ref = O.regular_grid_transform(gp.to_abi(), spec, r, lam)
    assert got.shape == ref.shape == (len(r) * len(lam), 2, 5)
    err = _slot_err(got, ref, gp)
    print("RL regular %s errors" % precision, err)
    assert np.all(err <= TOL64), err


def test_rlz_regular_grid_matches_oracle():
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=40.0, num_cells=16, kMin=0.0, kMax=20000.0,
                                     kDim=16, vars={"u": 1, "w": 2},
                                     BCB={"default": S.DirichletBC()}, BCT={"u": S.NeumannBC(), "w": S.NaturalBC()})
    g = S.createGrid(gp)
    pts = S.getGridpoints(g)
    g.set_physical(fields.rlz_blob_fields(pts, 2, zmax=20000.0), slot=1)
    S.spectralTransform_b(g)
    spec = g.get_spectral()
    r, lam, z = S.regular_axes(gp)
    got = S.regularGridTransform(g, r, lam, z)
    ref = O.regular_grid_transform(gp.to_abi(), spec, r, lam, z)
    assert got.shape == ref.shape == (len(r) * len(lam) * len(z), 2, 7)
    zi = np.tile(np.arange(len(z)), len(r) * len(lam))
    interior = (zi > 0) & (zi < len(z) - 1)
    err = _slot_err(got, ref, gp, rows=interior)
    print("RLZ regular errors (interior levels)", err)
    assert np.all(err <= TOL64), err
    # the end levels: every slot but ∂zz at 1e-12, ∂zz at 1e-5 (see the module docstring)
    ends = _slot_err(got, ref, gp, rows=~interior)
    print("RLZ regular errors (end levels)", ends)
    assert np.all(ends[:, :6] <= TOL64), ends
    assert np.all(ends[:, 6] <= 1e-5), ends
