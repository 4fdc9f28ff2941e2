"""GPU test of ss_spectral_transform_noalloc, the forward RL transform that
allocates nothing (for callers that cannot call cudaMalloc where they
transform: inside an open stream capture, under their own device-memory pool,
or in loops that must stay out of the allocator).

The caller owns the device input and output (here torch CUDA tensors, i.e.
memory allocated before the call by the caller); the ring-coefficient scratch
is the library's static 8 MiB device array.  The result of two calls in a row
(two different fields, so stale scratch from the first call would show) must
match the existing entry point, ss_spectral_transform, within the FP64 parity
tolerance of the other GPU tests.  This file is collected last on purpose.
"""
import ctypes as C

import numpy as np
import pytest

import springsteel_gpu as S
from springsteel_gpu import abi, fields

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _reference_spectral(grid, u):
    grid.set_physical(u, slot=1)
    S.spectralTransform_b(grid)
    return grid.get_spectral()


@pytest.mark.parametrize("precision", ["f64", "f64_fast"])
def test_noalloc_matches_spectral_transform_twice(precision):
    """Both FP64-storage precisions the entry point accepts: binary64 arithmetic
    and the double-float FFT arithmetic of SS_PREC_F64_FAST; the reference
    result is the existing entry point on the same grid, so the same
    tolerance applies to both."""
    import torch

    lib = S.load_library()
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=100.0, num_cells=100, vars={"u": 1, "v": 2},
                                     precision=precision)
    grid = S.createGrid(gp)
    pts = S.getGridpoints(grid)
    d = grid.dims
    fields_ab = []
    for seed in (1, 2):
        u = np.empty((d["n_physical"], 2), order="F")
        u[:, 0] = fields.gaussian_ring_field(pts, seed=seed)
        u[:, 1] = fields.blob_sum(pts, seed=10 + seed, nblobs=6)
        fields_ab.append(u)
    refs = [_reference_spectral(grid, u) for u in fields_ab]

    dev = torch.device("cuda", 0)
    d_in = torch.empty((2, d["n_physical"]), dtype=torch.float64, device=dev)   # column-major (np, nvars)
    d_out = torch.empty((2, d["n_spectral"]), dtype=torch.float64, device=dev)  # column-major (nspec, nvars)
    torch.cuda.synchronize()
    for u, ref in zip(fields_ab, refs):
        d_in.copy_(torch.from_numpy(np.ascontiguousarray(u.T)))
        d_out.fill_(float("nan"))
        torch.cuda.synchronize()
        st = lib.ss_spectral_transform_noalloc(grid.handle, C.c_void_p(d_in.data_ptr()),
                                               C.c_void_p(d_out.data_ptr()), None)
        assert st == abi.SS_OK, lib.ss_last_error_string().decode()
        grid.synchronize()
        got = d_out.cpu().numpy().T
        for v in range(2):
            den = np.max(np.abs(ref[:, v]))
            err = np.max(np.abs(got[:, v] - ref[:, v])) / den
            assert err <= TOL64, (v, err)
    grid.close()


def test_noalloc_rejects_grids_beyond_static_scratch():
    import torch

    lib = S.load_library()
    # 2 vars × Σ(1+2ri) for 250 cells = 1,128,000 > 1,048,576
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=250.0, num_cells=250, vars={"u": 1, "v": 2})
    grid = S.createGrid(gp)
    d = grid.dims
    d_in = torch.zeros((2, d["n_physical"]), dtype=torch.float64, device="cuda")
    d_out = torch.zeros((2, d["n_spectral"]), dtype=torch.float64, device="cuda")
    st = lib.ss_spectral_transform_noalloc(grid.handle, C.c_void_p(d_in.data_ptr()),
                                           C.c_void_p(d_out.data_ptr()), None)
    assert st == abi.SS_BAD_SHAPE
    assert b"static scratch" in lib.ss_last_error_string()
    grid.close()


def test_noalloc_rejects_misaligned_input():
    # the ring kernel reads (2n, 2n+1) point pairs as one 16-byte access: the call
    # checks the caller's pointer before launching anything
    import torch

    lib = S.load_library()
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=20.0, num_cells=20, vars={"u": 1})
    grid = S.createGrid(gp)
    d = grid.dims
    d_in = torch.zeros(d["n_physical"] * d["nvars"] + 2, dtype=torch.float64, device="cuda")
    d_out = torch.zeros(d["n_spectral"] * d["nvars"], dtype=torch.float64, device="cuda")
    st = lib.ss_spectral_transform_noalloc(grid.handle, C.c_void_p(d_in.data_ptr() + 8),
                                           C.c_void_p(d_out.data_ptr()), None)
    assert st == abi.SS_BAD_ARG
    assert b"16-byte aligned" in lib.ss_last_error_string()
    grid.close()
