"""GPU elliptic solve and learned preconditioner against the oracle.

Tolerances: the direct banded LU and the oracle's dense LU solve the same
FP64 systems (condition numbers ≲ 1e5 here), so solutions agree to 1e-10
relative.  GMRES stops at ‖c − Gx‖/‖c‖ ≤ 1e-10 per radial system.  The
network runs in BF16 with FP32 accumulation: forward outputs and gradients
are compared with the numpy oracle (same BF16 rounding points, FP64
accumulation) at 2e-2 relative in the Frobenius norm.
"""
import math

import numpy as np
import pytest

import mlp_oracle as M
import oracle as O
import springsteel_gpu as S
from springsteel_gpu import fields

pytestmark = pytest.mark.gpu

TOL_SOLVE = 1e-10
TOL_BF16 = 2e-2


def _problem(nc=40, R=50.0, seed=3, **kw):
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=R, num_cells=nc)
    g = S.createGrid(gp)
    k2 = fields.k2_profile(fields.radial_mish(gp), seed=seed, rmax=R)
    return gp, g, k2, S.SpringsteelProblem(g, k2, **kw)


def _set_forcing(g, seed, R):
    pts = S.getGridpoints(g)
    f = fields.blob_field(pts, fields.elliptic_blobs(seed, rmax=R))
    g.set_physical(f[:, None], slot=1)
    return f


def test_operator_matches_oracle():
    gp, g, k2, prob = _problem()
    el = O.OracleElliptic(O.OracleGrid(gp.to_abi()), k2)
    for m in (0, 1, 7, prob.K):
        Gg, Go = prob.operator(m), el.operator(m)
        assert Gg.shape == Go.shape
        assert np.max(np.abs(Gg - Go)) <= 1e-14 * np.max(np.abs(Go))


def test_direct_solve_matches_oracle():
    R = 50.0
    gp, g, k2, prob = _problem(R=R, backend="direct")
    f = _set_forcing(g, seed=11, R=R)
    st = S.solve(prob)
    assert st["converged"] == st["systems"] and st["max_rel_residual"] <= TOL_SOLVE
    got = g.get_physical()
    ref, _ = O.OracleElliptic(O.OracleGrid(gp.to_abi()), k2).solve(f[:, None])
    for s in range(5):
        scale = max(np.max(np.abs(ref[:, 0, s])), 1e-300)
        assert np.max(np.abs(got[:, 0, s] - ref[:, 0, s])) <= TOL_SOLVE * scale, s


def test_jacobi_gmres_converges_to_direct():
    R = 50.0
    gp, g, k2, prob = _problem(R=R, backend="krylov", preconditioner="diag", tol=1e-10, restart=40, maxiter=4000)
    _set_forcing(g, seed=12, R=R)
    st = S.solve(prob)
    assert st["converged"] == st["systems"], st
    assert st["max_rel_residual"] <= 1e-10
    it = st["max_iterations"]
    u_gm = g.get_physical()
    _set_forcing(g, seed=12, R=R)
    S.solve(prob, method="direct")
    u_d = g.get_physical()
    assert np.max(np.abs(u_gm[:, 0, 0] - u_d[:, 0, 0])) <= 1e-7 * np.max(np.abs(u_d[:, 0, 0]))
    assert it > 1


def _random_rows(rng, B, n=200):
    x = np.zeros((B, 256), np.float32)
    x[:, :n] = rng.normal(size=(B, n)) / math.sqrt(n)
    x[:, 254] = rng.uniform(size=B)
    x[:, 255] = rng.uniform(size=B)
    return x


def test_mlp_forward_matches_oracle():
    rng = np.random.default_rng(1)
    net = S.MLPPreconditioner(seed=4)
    W = rng.normal(0, math.sqrt(2 / 256), (3, 256, 256)).astype(np.float32)
    b = rng.normal(0, 0.05, (3, 256)).astype(np.float32)
    net.set_params(W, b)
    x = _random_rows(rng, 300)  # not a multiple of 128: padded rows
    got = net.forward(x)
    ref, _ = M.forward(W.astype(np.float64), b.astype(np.float64), x)
    assert np.linalg.norm(got - ref) <= TOL_BF16 * np.linalg.norm(ref)


def test_mlp_gradients_match_oracle():
    rng = np.random.default_rng(2)
    net = S.MLPPreconditioner(seed=5)
    W = rng.normal(0, math.sqrt(2 / 256), (3, 256, 256)).astype(np.float32)
    b = rng.normal(0, 0.05, (3, 256)).astype(np.float32)
    net.set_params(W, b)
    B = 512
    x = _random_rows(rng, B)
    t = rng.normal(size=(B, 256)).astype(np.float32)
    n = rng.integers(150, 255, B).astype(np.int32)
    dW, db, loss = net.gradients(x, t, n)
    L, dWo, dbo = M.loss_and_gradients(W.astype(np.float64), b.astype(np.float64), x, t, n)
    assert abs(loss - L) <= 1e-3 * abs(L)
    for l in range(3):
        assert np.linalg.norm(dW[l] - dWo[l]) <= TOL_BF16 * np.linalg.norm(dWo[l]), l
        assert np.linalg.norm(db[l] - dbo[l]) <= TOL_BF16 * np.linalg.norm(dbo[l]), l


def test_learned_fgmres_solves_and_training_lowers_loss():
    R = 50.0
    gp, g, k2, prob = _problem(R=R, backend="krylov", preconditioner="mlp", tol=1e-10, restart=30, maxiter=600)
    net = S.MLPPreconditioner(seed=7)
    blobs = [fields.elliptic_blobs(s, rmax=R) for s in range(64)]
    prob.collect_training(net, blobs)
    assert net.dataset_rows() == 64 * (1 + 2 * prob.K)
    stats = net.train(epochs=6, batch=1024, lr=1e-3, seed=1)
    assert stats["last_epoch_loss"] < stats["first_epoch_loss"]
    prob.attach(net)
    _set_forcing(g, seed=100001, R=R)
    st = S.solve(prob)
    assert st["converged"] == st["systems"], st
    u = g.get_physical()
    _set_forcing(g, seed=100001, R=R)
    S.solve(prob, method="direct")
    u_d = g.get_physical()
    assert np.max(np.abs(u[:, 0, 0] - u_d[:, 0, 0])) <= 1e-7 * np.max(np.abs(u_d[:, 0, 0]))


def test_trained_network_needs_fewer_iterations_than_jacobi():
    """What the learned preconditioner gains: after training on direct-solve pairs,
    flexible GMRES with the network reaches 1e-10 on held-out forcings in fewer
    iterations (on the slowest radial system and on average) than GMRES with the
    reference's :diag Jacobi preconditioner, and both agree with the direct solve."""
    R = 50.0
    gp, g, k2, prob = _problem(R=R, backend="krylov", preconditioner="mlp", tol=1e-10, restart=30, maxiter=2000)
    net = S.MLPPreconditioner(seed=11)
    prob.collect_training(net, [fields.elliptic_blobs(s, rmax=R) for s in range(256)])
    for s in range(256):
        prob.collect_random(net, 1, seed=s, smooth=s % 5)
    for ep, lr in ((3, 1e-3), (3, 3e-4)):
        net.train(epochs=ep, batch=2048, lr=lr, seed=ep)
    prob.attach(net)
    learned, jacobi = [], []
    for seed in range(10 ** 6, 10 ** 6 + 8):  # held out: training used seeds < 256
        _set_forcing(g, seed=seed, R=R)
        S.solve(prob, method="direct")
        u_d = g.get_physical()[:, 0, 0]
        for method, out in (("mlp", learned), ("diag", jacobi)):
            _set_forcing(g, seed=seed, R=R)
            st = S.solve(prob, method=method)
            assert st["converged"] == st["systems"] and st["fallback_systems"] == 0, (method, st)
            u = g.get_physical()[:, 0, 0]
            assert np.max(np.abs(u - u_d)) <= 1e-7 * np.max(np.abs(u_d)), method
            out.append(st)
    lmax = max(s["max_iterations"] for s in learned)
    jmax = max(s["max_iterations"] for s in jacobi)
    lmean = np.mean([s["mean_iterations"] for s in learned])
    jmean = np.mean([s["mean_iterations"] for s in jacobi])
    print("held-out iterations: learned max %d mean %.1f, Jacobi max %d mean %.1f" % (lmax, lmean, jmax, jmean))
    assert lmax < jmax and lmean < jmean
