"""Golden fixtures of small RL/RLZ round trips (`tests/golden/*.npz`, made by
`tests/golden/make_golden.py` from the FP64 oracle on seeded inputs).

CPU: the oracle reproduces every fixture (a change to the restatement shows up
here).  GPU: the CUDA path through the C ABI matches every fixture per (variable,
slot) at the FP64 bound, without running the oracle."""
import glob
import json
import os

import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from springsteel_gpu.io import _params_from_json

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = sorted(glob.glob(os.path.join(HERE, "*.npz")))
TOL64 = 1e-12


def _load(path):
    z = np.load(path)
    return (_params_from_json(json.loads(str(z["params"]))), np.asfortranarray(z["slot1"]),
            z["spectral"], z["physical"])


def _rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a)))


def test_fixtures_exist():
    names = {os.path.basename(p)[:-4] for p in CASES}
    assert {"rl10_natural", "rl8_two_vars_bcs", "rlz4_k10_dirichlet"} <= names


@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_oracle_reproduces_fixture(path):
    gp, slot1, spec, phys = _load(path)
    o = O.OracleGrid(gp.to_abi())
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, :, 0] = slot1
    spec_o = o.spectral_transform(ph)
    phys_o = o.grid_transform(spec_o)
    o.close()
    assert spec_o.shape == spec.shape and phys_o.shape == phys.shape
    assert _rel(spec_o, spec) <= 1e-14
    for v in range(phys.shape[1]):
        for s in range(phys.shape[2]):
            assert _rel(phys_o[:, v, s], phys[:, v, s]) <= 1e-13, (v, s)


@pytest.mark.gpu
@pytest.mark.parametrize("path", CASES, ids=lambda p: os.path.basename(p)[:-4])
def test_cuda_path_matches_fixture(path):
    from test_gpu_parity import slot_errors

    gp, slot1, spec, phys = _load(path)
    g = S.createGrid(gp)
    g.set_physical(slot1, slot=1)
    S.spectralTransform_b(g)
    spec_g = g.get_spectral()
    S.gridTransform_b(g)
    phys_g = g.get_physical()
    g.close()
    for v in range(spec.shape[1]):
        assert _rel(spec_g[:, v], spec[:, v]) <= TOL64, v
    errs = slot_errors(phys_g, phys, gp)
    assert np.all(errs <= TOL64), errs
