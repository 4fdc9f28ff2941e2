"""PERIODIC cubic B-spline BC in the oracle (src/CubicBSpline.jl:395-416, 366-369;
the dense factor of src/banded_cholesky.jl:70, 250-260 chosen by calcPQfactor
:777-781), pinned by the reference's periodic known-answer tests and by an
independent dense solve of the same folded system."""
import math

import numpy as np

import oracle as O
from springsteel_gpu import abi

PER = (abi.SS_SBC_PERIODIC, 0.0, 0.0)


def test_periodic_sa_equals_dense_folded_solve():
    sp = O.OracleSpline(0.0, 2 * math.pi, 17, bcl=PER, bcr=PER)
    G, PQ = sp.gamma(), sp.pq()
    assert G.shape == (17, 20)  # Minterior = Mdim − rankL(1) − rankR(2)
    rng = np.random.default_rng(3)
    b = rng.standard_normal(sp.bDim)
    want = G.T @ np.linalg.solve(G @ PQ @ G.T, G @ b)
    got = sp.sa(b)
    assert np.max(np.abs(got - want)) <= 1e-12 * np.max(np.abs(want))


def test_periodic_derivatives_kat():
    # test/basis.jl:166-215: sin on [0, 2π], 30 cells, PERIODIC both ends
    sp = O.OracleSpline(0.0, 2 * math.pi, 30, bcl=PER, bcr=PER)
    x = sp.mish()
    a = sp.sa(sp.sb(np.sin(x)))
    assert np.max(np.abs(sp.si(a, 1) - np.cos(x))) < 0.01
    assert np.max(np.abs(sp.si(a, 2) + np.sin(x))) < 0.01


def test_periodic_rl_grid_roundtrip():
    # test/grids.jl:60-101 (R geometry, PERIODIC, f = sin(2πr/L), error < 1e-4),
    # here on an RL grid: every wavenumber's radial spline is periodic
    g = O.OracleGrid(abi.make_params(abi.SS_GEOM_RL, 20, 0.0, 10.0, 1, BCL=[PER], BCR=[PER]))
    pts = g.gridpoints()
    ph = np.zeros(g.physical_shape, order="F")
    ph[:, 0, 0] = np.sin(2 * math.pi * pts[:, 0] / 10.0)
    sp = g.spectral_transform(ph)
    assert np.max(np.abs(sp)) > 1e-10
    out = g.grid_transform(sp)
    assert np.max(np.abs(out[:, 0, 0] - ph[:, 0, 0])) < 1e-4
