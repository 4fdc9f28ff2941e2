"""Elliptic solve on RL grids and the learned preconditioner (host mirror).

``SpringsteelProblem(grid, k2=…, backend=…, preconditioner=…)`` and
``solve(problem)`` follow the reference's Pair constructor and ``solve!``
(src/solver_problem.jl:311-339, :474-529) for the operator
∂rr + (1/r)∂r + (1/r²)∂λλ − k²(r): ``backend="direct"`` is the banded LU,
``backend="krylov"`` is GMRES with ``preconditioner="diag"`` (the reference's
Jacobi, :172-179) or ``preconditioner="mlp"`` (flexible GMRES with the learned
network).  The forcing f is read from physical slot 1 of the grid; u and its
derivatives land in every physical slot, as gridTransform! leaves them.
"""
import ctypes as C

import numpy as np

from . import abi, load_library, _check, getGridpoints

_METHODS = {"direct": abi.SS_SOLVER_DIRECT, "diag": abi.SS_SOLVER_GMRES_JACOBI, "mlp": abi.SS_SOLVER_FGMRES_MLP}


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


class MLPPreconditioner:
    """The per-wavenumber network (3 × 256, BF16 weights, FP32 accumulation)."""

    width = abi.MLP_WIDTH
    layers = abi.MLP_LAYERS

    def __init__(self, seed=0, device=0):
        h = C.c_void_p()
        _check(load_library().ss_mlp_create(int(device), int(seed), C.byref(h)))
        self._h = h

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("network closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            load_library().ss_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_params(self):
        W = np.zeros((self.layers, self.width, self.width), np.float32)
        b = np.zeros((self.layers, self.width), np.float32)
        _check(load_library().ss_mlp_get_params(self.handle, _ptr(W), _ptr(b)))
        return W, b

    def set_params(self, W, b):
        W = np.ascontiguousarray(W, np.float32).reshape(self.layers, self.width, self.width)
        b = np.ascontiguousarray(b, np.float32).reshape(self.layers, self.width)
        _check(load_library().ss_mlp_set_params(self.handle, _ptr(W), _ptr(b)))

    def forward(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros_like(x)
        _check(load_library().ss_mlp_forward(self.handle, _ptr(x), _ptr(out), x.shape[0]))
        return out

    def gradients(self, x, target, n):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(target, np.float32)
        n = np.ascontiguousarray(n, np.int32)
        dW = np.zeros((self.layers, self.width, self.width), np.float32)
        db = np.zeros((self.layers, self.width), np.float32)
        loss = C.c_double()
        _check(load_library().ss_mlp_gradients(self.handle, _ptr(x), _ptr(t), _ptr(n), x.shape[0], _ptr(dW),
                                                _ptr(db), C.byref(loss)))
        return dW, db, loss.value

    def dataset_rows(self):
        r = C.c_int64()
        _check(load_library().ss_mlp_dataset_rows(self.handle, C.byref(r)))
        return r.value

    def clear_dataset(self):
        _check(load_library().ss_mlp_dataset_clear(self.handle))

    def train(self, epochs=4, batch=4096, lr=1e-3, seed=0):
        st = abi.ss_train_stats()
        _check(load_library().ss_mlp_train(self.handle, int(epochs), int(batch), float(lr), int(seed), C.byref(st)))
        return {k: getattr(st, k) for k, _ in st._fields_ if not k.startswith("_")}


class SpringsteelProblem:
    """Radial Galerkin systems of one RL grid, factorised once (``_factorize_operator``)."""

    def __init__(self, grid, k2, backend="krylov", preconditioner="diag", tol=1e-10, maxiter=2000, restart=30,
                 mlp=None, mlp_max_wavenumber=-1):
        self.grid = grid
        k2 = np.ascontiguousarray(k2, np.float64)
        if k2.shape != (grid.dims["iDim"],):
            raise ValueError("k2 must hold one value per radial mish point (%d)" % grid.dims["iDim"])
        h = C.c_void_p()
        _check(load_library().ss_problem_create(grid.handle, _ptr(k2), C.byref(h)))
        self._h = h
        self.backend, self.preconditioner = backend, preconditioner
        self.tol, self.maxiter, self.restart = float(tol), int(maxiter), int(restart)
        self.mlp = None
        if mlp is not None:
            self.attach(mlp, mlp_max_wavenumber)
        nsys, nmax, K, bw = C.c_int32(), C.c_int32(), C.c_int32(), C.c_int32()
        _check(load_library().ss_problem_dims(h, C.byref(nsys), C.byref(nmax), C.byref(K), C.byref(bw)))
        self.nsys, self.nmax, self.K, self.bandwidth = nsys.value, nmax.value, K.value, bw.value

    @property
    def handle(self):
        if self._h is None:
            raise ValueError("problem closed")
        return self._h

    def close(self):
        if getattr(self, "_h", None) is not None:
            load_library().ss_problem_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def attach(self, mlp, max_wavenumber=-1):
        _check(load_library().ss_problem_set_mlp(self.handle, mlp.handle if mlp else None, int(max_wavenumber)))
        self.mlp = mlp

    def method(self):
        return _METHODS["direct"] if self.backend == "direct" else _METHODS[self.preconditioner]

    def operator(self, m):
        """Dense G_m (host copy) for checks."""
        band = np.zeros((self.nmax, self.bandwidth))
        n, kl = C.c_int32(), C.c_int32()
        _check(load_library().ss_problem_operator_band(self.handle, int(m), _ptr(band), C.byref(n), C.byref(kl)))
        n, kl = n.value, kl.value
        G = np.zeros((n, n))
        for i in range(n):
            for t in range(self.bandwidth):
                j = i + t - kl
                if 0 <= j < n:
                    G[i, j] = band[i, t]
        return G

    def export(self):
        rhs = np.zeros((self.nsys, self.nmax))
        x = np.zeros((self.nsys, self.nmax))
        res = np.zeros(self.nsys)
        it = np.zeros(self.nsys, np.int32)
        _check(load_library().ss_problem_export(self.handle, _ptr(rhs), _ptr(x), _ptr(res), _ptr(it)))
        return rhs, x, res, it

    def collect_training(self, mlp, blob_lists, max_wavenumber=-1, points=None):
        """Append the direct solutions of the fields Σ A exp(−|x − x_c|²/w²) (one list of
        (xc, yc, w, A) per field) to the network's training set."""
        offs = np.zeros(len(blob_lists) + 1, np.int32)
        for i, bl in enumerate(blob_lists):
            offs[i + 1] = offs[i] + len(bl)
        blobs = np.ascontiguousarray(np.concatenate([np.asarray(b, np.float64).reshape(-1, 4) for b in blob_lists])
                                     if len(blob_lists) else np.zeros((0, 4)))
        if points is None:
            points = getGridpoints(self.grid)
        pts = np.asfortranarray(points[:, :2], np.float64)
        _check(load_library().ss_problem_collect_training(self.handle, mlp.handle, _ptr(pts), _ptr(blobs), _ptr(offs),
                                                          len(blob_lists), int(max_wavenumber)))

    def collect_random(self, mlp, nsets, seed=0, smooth=0, max_wavenumber=-1):
        """Append direct solutions of seeded random right-hand sides (one per radial system
        per set, smoothed ``smooth`` times) to the network's training set."""
        _check(load_library().ss_problem_collect_random(self.handle, mlp.handle, int(nsets), int(seed), int(smooth),
                                                        int(max_wavenumber)))


def solve(problem, method=None, tol=None, maxiter=None, restart=None, stream=None):
    """solve!(problem): f in physical slot 1 → u (all derivative slots); returns the solve statistics."""
    st = abi.ss_solve_stats()
    m = problem.method() if method is None else _METHODS[method]
    _check(load_library().ss_solve(problem.handle, m, problem.tol if tol is None else float(tol),
                                   problem.maxiter if maxiter is None else int(maxiter),
                                   problem.restart if restart is None else int(restart), C.byref(st), stream))
    return {k: getattr(st, k) for k, _ in st._fields_ if not k.startswith("_")}
