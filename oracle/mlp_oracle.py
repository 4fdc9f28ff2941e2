"""Test infrastructure, not product code: numpy restatement of the learned
preconditioner network, used only by tests/ to check the tensor-core kernels.

The network has no counterpart in the reference (its preconditioners are
:none and :diag, src/solver_problem.jl:128-179).  This oracle computes the
same forward pass, mean-squared loss and gradients as the device kernels, in
FP64 arithmetic, rounding to bfloat16 exactly where the device stores
bfloat16 (inputs, weights, hidden activations, back-propagated gradients), so
the two agree up to FP32-versus-FP64 accumulation and the rare bfloat16
rounding flip that difference causes.  ``exact=True`` skips every rounding,
for finite-difference checks of the formulas themselves.
"""
import numpy as np

WIDTH = 256
LAYERS = 3


def bf16(x):
    """Round float values to bfloat16 (round to nearest, ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = rounded.astype(np.uint32).view(np.float32)
    return out.astype(np.float64)


def _r(x, exact):
    return np.asarray(x, np.float64) if exact else bf16(x)


def forward(W, b, x, exact=False):
    """Rows x (B × 256) → (output, cache).  W[l] is (out × in), b[l] is (out,)."""
    Wb = [_r(W[l], exact) for l in range(LAYERS)]
    X0 = _r(x, exact)
    Z1 = X0 @ Wb[0].T + b[0]
    Y1 = _r(np.maximum(Z1, 0.0), exact)
    Z2 = Y1 @ Wb[1].T + b[1]
    Y2 = _r(np.maximum(Z2, 0.0), exact)
    O = Y2 @ Wb[2].T + b[2]
    return O, (Wb, X0, Z1, Y1, Z2, Y2)


def loss_and_gradients(W, b, x, target, n, exact=False):
    """L = (1/B) Σ_rows Σ_{i<n_row} (O − T)²; returns (L, dW, db)."""
    B = x.shape[0]
    O, (Wb, X0, Z1, Y1, Z2, Y2) = forward(W, b, x, exact)
    T = _r(target, exact)
    mask = np.arange(WIDTH)[None, :] < np.asarray(n)[:, None]
    D = np.where(mask, O - T, 0.0)
    L = float(np.sum(D * D) / B)
    G3 = _r(2.0 * D / B, exact)
    dW = np.zeros((LAYERS, WIDTH, WIDTH))
    db = np.zeros((LAYERS, WIDTH))
    dW[2], db[2] = G3.T @ Y2, G3.sum(axis=0)
    G2 = _r((G3 @ Wb[2]) * (Z2 > 0), exact)
    dW[1], db[1] = G2.T @ Y1, G2.sum(axis=0)
    G1 = _r((G2 @ Wb[1]) * (Z1 > 0), exact)
    dW[0], db[0] = G1.T @ X0, G1.sum(axis=0)
    return L, dW, db
