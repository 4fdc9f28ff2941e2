"""CPU checks of the C-ABI library: it builds for sm_103a, loads, exports every
entry point declared in include/*.h, and fails loudly without a GPU."""
import ctypes as C
import glob
import os
import re

import pytest

import springsteel_gpu as S
from springsteel_gpu import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(ss_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = _declared_symbols()
    assert {"ss_grid_create", "ss_spectral_transform", "ss_grid_transform"} <= names


def test_library_exports_every_declared_symbol():
    lib = S.load_library()
    missing = [n for n in sorted(_declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(abi.EXPORTED) <= _declared_symbols()


def test_struct_layout_matches_header():
    assert C.sizeof(abi.ss_spline_bc) == 24
    assert C.sizeof(abi.ss_grid_params) == 10 * 4 + 4 * 8 + 6 * 8 + 2 * 4
    assert C.sizeof(abi.ss_dims) == 12 * 8


def test_solver_struct_layout_matches_header():
    assert C.sizeof(abi.ss_solve_stats) == 6 * 4 + 3 * 8
    assert C.sizeof(abi.ss_train_stats) == 2 * 4 + 2 * 8 + 3 * 8


def test_solver_null_arguments_rejected():
    lib = S.load_library()
    assert lib.ss_problem_create(None, None, None) == abi.SS_BAD_ARG
    assert lib.ss_solve(None, 0, 1e-10, 10, 10, None, None) == abi.SS_BAD_ARG
    assert lib.ss_mlp_create(0, 0, None) == abi.SS_BAD_ARG
    assert lib.ss_mlp_forward(None, None, None, 0) == abi.SS_BAD_ARG
    assert lib.ss_mlp_train(None, 1, 128, 1e-3, 0, None) == abi.SS_BAD_ARG
    assert lib.ss_problem_destroy(None) == abi.SS_OK
    assert lib.ss_mlp_destroy(None) == abi.SS_OK


def test_mlp_without_gpu_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(S.SpringsteelError) as e:
        S.MLPPreconditioner(seed=0)
    assert e.value.status == abi.SS_NO_DEVICE


def test_version_and_error_string():
    lib = S.load_library()
    assert lib.ss_version() == 2
    assert isinstance(lib.ss_last_error_string(), bytes)


def test_null_arguments_rejected():
    lib = S.load_library()
    assert lib.ss_grid_create(None, None) == abi.SS_BAD_ARG
    assert lib.ss_grid_dims(None, None) == abi.SS_BAD_ARG
    assert lib.ss_spectral_transform(None, None) == abi.SS_BAD_ARG


def test_create_without_gpu_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    gp = S.SpringsteelGridParameters(geometry="RL", num_cells=4, iMin=0.0, iMax=10.0)
    with pytest.raises(S.SpringsteelError) as e:
        S.createGrid(gp)
    assert e.value.status == abi.SS_NO_DEVICE
