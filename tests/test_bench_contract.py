"""bench.py's host-side contract, on CPU: the reference arm's JSON line, its
behaviour under a two-rank launch (rank 0 alone runs and prints), the
max-over-ranks reduction of the timed region on a world-size-2 gloo group, and the
per-stage byte / flop models the roofline fields use."""
import json
import math
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

REQUIRED = ["metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
            "scaling", "vs_baseline", "dtype", "data", "config"]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _json_lines(text):
    return [json.loads(ln) for ln in text.splitlines() if ln.startswith("{")]


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "rlz100-f64",
                          "--steps", "1", "--warmup", "0"], cwd=ROOT, capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = _json_lines(out.stdout)
    assert len(lines) == 1
    line = lines[0]
    for k in REQUIRED + ["impl", "cpu_baseline", "e2e"]:
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0 and line["higher_is_better"] is True
    assert line["e2e"] == {"value": line["value"], "unit": line["unit"], "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    # the GPU arm's config object for the same workload
    cfg = line["config"]
    assert cfg["workload"].startswith("RLZ 100 cells x 32 Chebyshev levels, 2 vars")
    assert (cfg["iDim"], cfg["b_kDim"], cfg["jDim"]) == (300, 22, 181800)
    assert cfg["parallelism"] == "single"


def test_reference_arm_two_ranks_prints_once():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py", "--impl", "reference",
           "--workload", "rlz100-f64", "--gpus", "2", "--steps", "1", "--warmup", "0"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = _json_lines(out.stdout)
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2


def _rank_main(rank, port, values, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=len(values))
    try:
        q.put((rank, bench._max_over_ranks(values[rank], device="cpu")))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo_world_size_2():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    values = [12.5, 40.25]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, port, values, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == {0: 40.25, 1: 40.25}


def test_max_over_ranks_without_group_is_identity():
    assert bench._max_over_ranks(3.5, device="cpu") == 3.5


def test_stage_models_of_the_default_workload():
    dims = {"iDim": 600, "kDim_wn": 600, "b_kDim": 22, "nvars": 5, "kDim": 32, "jDim": 723600,
            "b_jDim": 360600, "n_physical": 723600 * 32, "n_spectral": 5363666, "nslots": 7}
    # one real DFT per ring, z-mode and variable at 2.5·L·log2 L, L = 4 + 4r
    want = sum(2.5 * (4 + 4 * r) * math.log2(4 + 4 * r) for r in range(1, 601)) * 22 * 5
    assert bench._ring_fft_flops(dims) == pytest.approx(want, rel=1e-12)
    sb = bench._stage_bytes(dims, 8)
    assert sb["ring_inverse"] == 8 * 5 * (3 * 22 * 360600 + 5 * 22 * 723600)
    assert sb["cheb_inverse"] == 8 * 5 * (5 * 22 * 723600 + 7 * 723600 * 32)
    assert bench._bytes_per_roundtrip(dims, 8) == 8 * 5 * (723600 * 32 * 8 + 2 * 5363666)


def test_output_check_tolerances_and_detection():
    import numpy as np

    from springsteel_gpu.io import _params_from_json

    assert set(bench.CHECK_TOLERANCE) == {"f64", "f64_fast", "f32"}
    assert len(bench.CHECK_TOLERANCE["f32"]) == 7
    # the check's per-slot errors on a golden fixture: zero against itself, and a
    # perturbation of one slot (planted in a host copy) is caught by the FP64 bound
    z = np.load(os.path.join(ROOT, "tests", "golden", "rlz4_k10_dirichlet.npz"))
    gp = _params_from_json(json.loads(str(z["params"])))
    phys = z["physical"]
    errs = bench._slot_errors(lambda v, s: phys[:, v, s], phys, gp)
    assert errs.shape == (1, 7) and np.all(errs == 0.0)
    bad = phys.copy()
    bad[17, 0, 5] += 1e-9 * np.max(np.abs(phys[:, 0, 5]))
    errs = bench._slot_errors(lambda v, s: bad[:, v, s], phys, gp)
    tol = np.broadcast_to(np.asarray(bench.CHECK_TOLERANCE["f64"], np.float64), (7,))
    assert errs[0, 5] > tol[5] and np.all(np.delete(errs[0], 5) <= tol[:6])
