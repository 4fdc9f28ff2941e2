#!/usr/bin/env python
"""Benchmark of the GB300 RL/RLZ transform path (one JSON line on rank 0).

Metric: RLZ transforms/s — one transform = one round trip, spectralTransform!
followed by gridTransform!, over every variable of the grid, all 7 derivative
slots.  Default workload: the 5-variable RLZ grid of 200 radial cells, rings
of 4+4r points, 32 Chebyshev levels on z ∈ [0, 20000], FP64 (the reference's
precision).  ``--workload rlz400-f32`` runs the 8-variable 400-cell / 64-level
FP32+refinement grid instead.

  value     round trips/s with inputs resident in HBM (CUDA events on the
            library's stream, max over ranks)
  e2e       round trips/s through the C ABI with pinned host buffers:
            ss_spectral_transform_from_host (physical slot 1 in) and
            ss_grid_transform_to_host (all 7 slots out) per step, the copies of
            each radial chunk overlapping the other chunks' transforms; the
            same with upload → transforms → download in sequence is reported
            beside it
  roofline  the dominant stage, timed live with CUDA events inside the timed
            region (the library's stage instrumentation)
  cpu_baseline  the FP64 oracle (C port of the reference path) on the host
            cores: one whole round trip of every variable of the same grid and
            inputs (the 400-cell FP32 grid: its first variable, host RAM)
  check     the GPU round trip of the same inputs against that oracle output,
            per variable and derivative slot (the run fails above 1e-12 in FP64)
  secondary the default run also measures the 8-variable 400-cell / 64-level
            FP32+refinement grid and nests its line under "secondary"

``--impl reference`` times the reference's CPU path instead: Julia is not
available on either machine, so that arm runs the C port of the reference
algorithm (the oracle) with every host thread.  Multi-GPU: independent
replicas of the grid (no collective on the data path), weak scaling.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (os.path.join(ROOT, "springsteel.jl_gb300"), os.path.join(ROOT, "oracle")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

# Per-slot bound of the output check [f, ∂r, ∂rr, ∂λ, ∂λλ, ∂z, ∂zz], relative to the slot's
# scale: FP64 to round-off; double-float bulk to its 48-bit significand; binary32 storage
# with the FP64-refined spline solve to the binary32 floor of each derivative.
CHECK_TOLERANCE = {
    "f64": 1e-12,
    "f64_fast": 2e-11,
    "f32": [2e-6, 5e-5, 5e-5, 5e-5, 5e-5, 5e-6, 5e-6],
}

WORKLOADS = {
    "rlz200-f64": dict(num_cells=200, kDim=32, nvars=5, precision="f64"),
    "rlz200-f64fast": dict(num_cells=200, kDim=32, nvars=5, precision="f64_fast"),
    "rlz400-f32": dict(num_cells=400, kDim=64, nvars=8, precision="f32", noise=1e-2),
    # small case for profiling captures (same kernels, a few hundred MB)
    "rlz100-f64": dict(num_cells=100, kDim=32, nvars=2, precision="f64"),
    "rlz200-f32": dict(num_cells=200, kDim=64, nvars=2, precision="f32", noise=1e-2),
    # 64 uneven RL grids (50-400 cells, 1-4 variables) as one batch under a CUDA graph
    "batch-rl64": dict(ngrids=64, nc_min=50, nc_max=400, nv_min=1, nv_max=4, precision="f64", seed=3),
    "batch-rl64-f32": dict(ngrids=64, nc_min=50, nc_max=400, nv_min=1, nv_max=4, precision="f32", seed=3),
    # learned-preconditioner elliptic solve on the 200-cell RL grid (separate JSON line)
    "elliptic-rl200": dict(num_cells=200, rmax=100.0, train_fields=20000, train_random=20000, eval_seeds=1000,
                           k2_seed=5, restart=30, tol=1e-10),
}


def run_batch(args):
    """Batched workload of 64 uneven RL grids: one step = spectralTransform! + gridTransform! of
    every grid of the batch (all variables, all 5 slots), replayed as one CUDA graph
    with autotuned ring-kernel CTA sizes.  Also reported: the same grids as
    individual calls (no graph), and e2e with every grid's slot 1 uploaded and all
    slots downloaded per step."""
    import torch

    import springsteel_gpu as S
    from springsteel_gpu import abi, fields

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    w = WORKLOADS[args.workload]
    rng = np.random.default_rng(w["seed"] + rank)
    grids, ups = [], []
    nbytes = 0
    host_dt = np.float32 if w["precision"] == "f32" else np.float64
    for i in range(w["ngrids"]):
        nc = int(rng.integers(w["nc_min"], w["nc_max"] + 1))
        nv = int(rng.integers(w["nv_min"], w["nv_max"] + 1))
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=float(nc), num_cells=nc,
                                         vars={"v%d" % k: k + 1 for k in range(nv)}, precision=w["precision"])
        g = S.createGrid(gp)
        pts = S.getGridpoints(g)
        u = np.empty((pts.shape[0], nv), order="F", dtype=host_dt)
        for v in range(nv):
            u[:, v] = fields.blob_sum(pts, seed=1000 * i + v, nblobs=4)
        g.set_physical(u, slot=1)
        grids.append(g)
        ups.append(u)
        nbytes += g.dims["n_physical"] * nv * (1 + 5) * np.dtype(host_dt).itemsize
    lib = S.load_library()
    batch = S.Batch(grids, autotune=True)
    for _ in range(max(args.warmup, 3)):
        batch.run(what=3, use_graph=True)
    batch.synchronize()

    def timed(fn, steps, on=None):  # wall clock between device-wide synchronisations
        torch.cuda.synchronize()
        for g in grids:
            g.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        (on or batch).synchronize()
        for g in grids:
            g.synchronize()
        return (time.perf_counter() - t0) / steps

    # the same grids with per-grid launch sequences on forked streams (graph)
    seq = S.Batch(grids, autotune=False, fused=False)
    for _ in range(max(args.warmup, 3)):
        seq.run(what=3, use_graph=True)
    seq.synchronize()
    with ClockSampler(local) as clk:
        t_batch = timed(lambda: batch.run(what=3, use_graph=True), args.steps)
        t_seq = timed(lambda: seq.run(what=3, use_graph=True), args.steps, on=seq)

        def singles():
            for g in grids:
                S.spectralTransform_b(g)
                S.gridTransform_b(g)

        t_single = timed(singles, max(1, args.steps // 2))

        pinned = [torch.from_numpy(np.ascontiguousarray(u.T)).pin_memory() for u in ups]
        outs = [torch.empty(g.dims["n_physical"] * g.dims["nvars"] * g.dims["nslots"],
                            dtype=torch.float32 if host_dt == np.float32 else torch.float64).pin_memory()
                for g in grids]
        dt_code = abi.SS_DTYPE_F32 if host_dt == np.float32 else abi.SS_DTYPE_F64

        def e2e():
            for g, h in zip(grids, pinned):
                S._check(lib.ss_upload_physical(g.handle, C.c_void_p(h.data_ptr()), dt_code, 1, None))
            batch.run(what=3, use_graph=True)
            batch.synchronize()
            for g, h in zip(grids, outs):
                S._check(lib.ss_download_physical(g.handle, C.c_void_p(h.data_ptr()), dt_code, 0, None))

        t_e2e = timed(e2e, max(1, min(args.steps, 3)))
    h2d = sum(p.numel() * p.element_size() for p in pinned)
    d2h = sum(o.numel() * o.element_size() for o in outs)
    peak, peak_kind = _peaks()
    fused_launches = batch.fused_launches(3)
    line = {
        "metric": "batched RL transforms/s (64 uneven grids, fused launches under a graph)", "value": 1.0 / t_batch,
        "unit": "batch round trips/s", "n_gpus": ws, "steps": args.steps, "warmup": max(args.warmup, 3),
        "ms_per_step": t_batch * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32" if host_dt == np.float32 else "f64", "data": "synthetic",
        "config": {"workload": args.workload, "grids": len(grids),
                   "cells": [g.params.num_cells for g in grids], "vars": [g.dims["nvars"] for g in grids]},
        "individual_calls_ms": t_single * 1e3, "speedup_vs_individual_calls": t_single / t_batch,
        "per_grid_sequences_graph_ms": t_seq * 1e3, "speedup_vs_per_grid_graph": t_seq / t_batch,
        "fused_launches_per_round_trip": fused_launches,
        "path_gbs": nbytes / t_batch / 1e9, "path_frac": nbytes / t_batch / 1e9 / peak, "peak": peak,
        "peak_source": peak_kind, "clocks": clk.summary(),
        "e2e": {"value": 1.0 / t_e2e, "unit": "batch round trips/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
    }
    batch.close()
    seq.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_elliptic(args):
    """ms per elliptic solve to ‖c − Gx‖/‖c‖ ≤ 1e-10 on every radial system, for the direct
    banded LU, Jacobi-preconditioned GMRES and flexible GMRES with the learned
    preconditioner.  The network is trained first (untimed) on direct solutions of
    `train_fields` forcing fields and `train_random` sets of random right-hand sides;
    the held-out forcing seeds start at 10⁶.  Per solve and method: upload f from
    pinned host memory, ss_solve (transform, radial solves, inverse transform),
    download u (all 5 slots); device time of the radial solve stage from the
    library's events, wall time around the whole call."""
    import torch

    import springsteel_gpu as S
    from springsteel_gpu import abi, fields

    ws, rank, local = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    w = WORKLOADS["elliptic-rl200"]
    n_eval = min(w["eval_seeds"], max(args.steps, 1) * 100) if args.steps < 10 else w["eval_seeds"]
    gp = fields.elliptic_rl200_params(num_cells=w["num_cells"], rmax=w["rmax"])
    grid = S.createGrid(gp)
    k2 = fields.k2_profile(fields.radial_mish(gp), seed=w["k2_seed"], rmax=w["rmax"])
    prob = S.SpringsteelProblem(grid, k2, tol=w["tol"], restart=w["restart"], maxiter=20000)
    pts = S.getGridpoints(grid)
    net = S.MLPPreconditioner(seed=1)
    t0 = time.perf_counter()
    for i in range(0, w["train_fields"], 1000):
        blobs = [fields.elliptic_blobs(s, rmax=w["rmax"]) for s in range(i, min(i + 1000, w["train_fields"]))]
        prob.collect_training(net, blobs, points=pts)
    for s in range(w["train_random"]):
        prob.collect_random(net, 1, seed=s, smooth=s % 5)
    collect_s = time.perf_counter() - t0
    train = []
    for ep, lr in ((2, 1e-3), (2, 3e-4), (2, 1e-4)):
        train.append(net.train(epochs=ep, batch=8192, lr=lr, seed=ep))
    prob.attach(net)
    n = grid.dims["n_physical"]
    h_f = torch.empty(n, dtype=torch.float64).pin_memory()
    h_u = torch.empty(n * 5, dtype=torch.float64).pin_memory()
    lib = S.load_library()

    def one(method):
        grid.synchronize()
        t = time.perf_counter()
        S._check(lib.ss_upload_physical(grid.handle, C.c_void_p(h_f.data_ptr()), abi.SS_DTYPE_F64, 1, None))
        st = S.solve(prob, method=method)
        S._check(lib.ss_download_physical(grid.handle, C.c_void_p(h_u.data_ptr()), abi.SS_DTYPE_F64, 0, None))
        st["wall_ms"] = (time.perf_counter() - t) * 1e3
        return st

    def forcing(seed):
        h_f.numpy()[:] = fields.blob_field(pts, fields.elliptic_blobs(seed, rmax=w["rmax"]))

    methods = {"direct": "direct", "jacobi_gmres": "diag", "learned_fgmres": "mlp"}
    for s in range(max(args.warmup, 3)):
        forcing(10 ** 6 - 1 - s)
        for m in methods.values():
            one(m)
    res, per = {}, {k: [] for k in methods}
    with ClockSampler(local) as clk:
        for s in range(n_eval):
            forcing(10 ** 6 + s)  # host-side field synthesis, outside every timed call
            for name, m in methods.items():
                per[name].append(one(m))
        for name in methods:
            sts = per[name]
            res[name] = {
                "device_ms": statistics.mean(s["ms"] for s in sts),
                "wall_ms": statistics.mean(s["wall_ms"] for s in sts),
                "max_iterations": statistics.mean(s["max_iterations"] for s in sts),
                "mean_iterations": statistics.mean(s["mean_iterations"] for s in sts),
                "all_converged": all(s["converged"] == s["systems"] for s in sts),
                "worst_rel_residual": max(s["max_rel_residual"] for s in sts),
                "fallback_systems": sum(s["fallback_systems"] for s in sts),
            }
    line = {
        "metric": "ms per elliptic solve to 1e-10 (learned FGMRES)", "value": res["learned_fgmres"]["wall_ms"],
        "unit": "ms", "n_gpus": 1, "steps": n_eval, "warmup": max(args.warmup, 3),
        "ms_per_step": res["learned_fgmres"]["wall_ms"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (solve), bf16/fp32 (network)", "data": "synthetic",
        "config": {"workload": "elliptic-rl200", "grid": "RL, 200 cells, r in [0, 100], rings of 4+4r",
                   "radial_systems": prob.nsys, "unknowns_per_system": prob.nmax, "held_out_seeds": n_eval,
                   "train_fields": w["train_fields"], "train_random_sets": w["train_random"],
                   "train_rows": net.dataset_rows(), "restart": w["restart"], "tol": w["tol"]},
        "methods": res, "training": {"collect_s": collect_s, "phases": train},
        "clocks": clk.summary(),
        "e2e": {"value": res["learned_fgmres"]["wall_ms"], "unit": "ms", "h2d_bytes_per_step": n * 8,
                "d2h_bytes_per_step": n * 5 * 8},
    }
    print(json.dumps(line), flush=True)
    return 0


def _params(wl):
    from springsteel_gpu import fields

    w = WORKLOADS[wl]
    if w["precision"] != "f32":
        return fields.rlz_params(precision=w["precision"], num_cells=w["num_cells"], kDim=w["kDim"],
                                     nvars=w["nvars"])
    return fields.rlz400_f32_params(precision="f32", num_cells=w["num_cells"], kDim=w["kDim"], nvars=w["nvars"])


def _config(wl, dims):
    w = WORKLOADS[wl]
    return {
        "workload": "RLZ %d cells x %d Chebyshev levels, %d vars, %s" % (
            w["num_cells"], w["kDim"], w["nvars"],
            {"f64_fast": "FP64 data, double-float FFT/DCT on FP32 pipes", "f64": "FP64 throughout",
             "f32": "FP32+FP64 refinement"}[w["precision"]]),
        "precision": w["precision"],
        "geometry": "RLZ", "num_cells": w["num_cells"], "iDim": dims["iDim"], "kDim": w["kDim"],
        "b_kDim": dims["b_kDim"], "nvars": w["nvars"], "jDim": dims["jDim"],
        "physical_points_per_var": dims["n_physical"], "spectral_per_var": dims["n_spectral"],
        "fields": "seeded Gaussian-blob sums (8 blobs, widths 5-30, z in [0, 20000])" + (
            " plus N(0, %g) noise" % w["noise"] if w.get("noise") else ""),
        "l2": "inputs larger than L2 (physical slot 1 > 129 MB)",
    }


def _bytes_per_roundtrip(dims, w):
    """Algorithmic HBM bytes of one round trip: read slot 1, write every slot,
    write + read spectral (per variable)."""
    return w * dims["nvars"] * (dims["n_physical"] * (1 + dims["nslots"]) + 2 * dims["n_spectral"])


def _ring_fft_flops(dims):
    """Conventional flops of one real DFT per ring, z-mode and variable."""
    pol = dims["kDim_wn"] - dims["iDim"]  # patchOffsetL
    per = sum(2.5 * L * np.log2(L) for L in (4 + 4 * (r + pol) for r in range(1, dims["iDim"] + 1)))
    return per * dims["b_kDim"] * dims["nvars"]


def _matmul_tflops(dtype, n=4096):
    """Dense matmul rate of `dtype` on the current GPU (best of 3, CUDA events)."""
    import torch

    a = torch.randn(n, n, dtype=dtype, device="cuda")
    torch.matmul(a, a)
    best = None
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, a)
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        best = t if best is None else min(best, t)
    return 2.0 * n ** 3 / best / 1e12


def _stage_bytes(dims, w):
    """Compulsory bytes of each stage for one round trip (all variables)."""
    nv, bk, jD, fr = dims["nvars"], dims["b_kDim"], dims["jDim"], dims["b_jDim"]
    npx, ns = dims["n_physical"], dims["n_spectral"]
    rlz = dims["kDim"] > 1
    out = {
        "cheb_forward": w * nv * (npx + bk * jD) if rlz else 0,
        "ring_forward": w * nv * ((bk * jD if rlz else npx) + bk * fr),
        "sb_project": w * nv * (bk * fr + ns),
        "sa_si": w * nv * (ns + 3 * bk * fr),
        "ring_inverse": w * nv * (3 * bk * fr + (5 * bk * jD if rlz else 5 * npx)),
        "cheb_inverse": w * nv * (5 * bk * jD + 7 * npx) if rlz else 0,
    }
    return out


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _max_over_ranks(x, device="cuda"):
    """The largest `x` over all ranks of the process group (x itself on one rank)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _device_inputs(grid, wl, seed):
    """Seeded blob-sum fields (plus the workload's noise) written into physical
    slot 1 on the device; returns a pinned host copy of slot 1, (nvars, n) rows."""
    import torch

    from springsteel_gpu import fields

    w = WORKLOADS[wl]
    fields.fill_rlz_blobs_device(grid, base_seed=seed, zmax=20000.0, noise=w.get("noise", 0.0))
    d = grid.dims
    dt = torch.float32 if w["precision"] == "f32" else torch.float64
    h = torch.empty((d["nvars"], d["n_physical"]), dtype=dt).pin_memory()
    for v in range(d["nvars"]):
        h[v].copy_(grid.device_array("physical", v, slot=1))
    return h


def _slot_errors(planes, phys_o, gp):
    """max|gpu − oracle| / scale per (variable, slot): scale = max(max|oracle slot|,
    max|oracle f|/ℓ^d) for a derivative of order d along a domain of length ℓ (the
    tests' parity norm).  planes(v, s) returns the GPU plane as float64 numpy."""
    lengths = {"r": gp.iMax - gp.iMin, "l": 1.0, "z": (gp.kMax - gp.kMin) or 1.0}
    deriv = [(None, 0), ("r", 1), ("r", 2), ("l", 1), ("l", 2), ("z", 1), ("z", 2)]
    out = np.zeros(phys_o.shape[1:])
    for v in range(phys_o.shape[1]):
        fmax = np.max(np.abs(phys_o[:, v, 0]))
        for s in range(phys_o.shape[2]):
            dirn, d = deriv[s]
            den = max(np.max(np.abs(phys_o[:, v, s])), fmax / lengths[dirn] ** d if dirn else 0.0)
            out[v, s] = np.max(np.abs(planes(v, s) - phys_o[:, v, s])) / den if den > 0 else 0.0
    return out


def _oracle_roundtrip(gp, slot1, threads, var_index=None):
    """spectralTransform! + gridTransform! of the FP64 oracle (the C port of the
    reference path) on host inputs `slot1` (nvars, n); with var_index, only that
    variable, on a one-variable grid of the same shape.  Returns (seconds, physical)."""
    import copy

    import oracle as O

    O.set_threads(threads)
    if var_index is not None:
        g1 = copy.copy(gp)
        g1.vars = {gp.var_names()[0]: 1}
        gp, rows = g1, [var_index]
    else:
        rows = list(range(slot1.shape[0]))
    o = O.OracleGrid(gp.to_abi())
    ph = np.zeros(o.physical_shape, order="F")
    for i, v in enumerate(rows):
        ph[:, i, 0] = slot1[v]
    t0 = time.perf_counter()
    out = o.grid_transform(o.spectral_transform(ph))
    dt = time.perf_counter() - t0
    o.close()
    return dt, out


# Measured DRAM traffic of each stage for one round trip: dram__bytes_read.sum +
# dram__bytes_write.sum summed over the stage's launches (every ring bucket), from
# one ncu capture (1-pass metrics, --clock-control none) of the full-size bench
# workload itself: `bench.py --workload W --steps 1 --warmup 3 --no-cpu-baseline
# --no-secondary` under `ncu --metrics gpu__time_duration.sum,dram__bytes_read.sum,
# dram__bytes_write.sum -k regex:"ring_|cheb_|sa_si|sb_project"`, one warm-up
# round trip's launches.  Bytes per round trip.
MEASURED_TRAFFIC = {
    ("rlz200-f64", "cheb_forward"): 1.539e9,
    ("rlz200-f64", "ring_forward"): 0.863e9,
    ("rlz200-f64", "sb_project"): 0.493e9,
    ("rlz200-f64", "sa_si"): 1.106e9,
    ("rlz200-f64", "ring_inverse"): 3.903e9,
    ("rlz200-f64", "cheb_inverse"): 9.642e9,
    ("rlz400-f32", "cheb_forward"): 9.910e9,
    ("rlz400-f32", "ring_forward"): 6.068e9,
    ("rlz400-f32", "sb_project"): 3.279e9,
    ("rlz400-f32", "sa_si"): 24.037e9,
    ("rlz400-f32", "ring_inverse"): 26.665e9,
    ("rlz400-f32", "cheb_inverse"): 64.088e9,
}


def run_reference(args):
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    from springsteel_gpu import fields

    threads = os.cpu_count() or 1
    wl = args.workload
    w = WORKLOADS[wl]
    gp = _params(wl)
    import oracle as O

    o = O.OracleGrid(gp.to_abi())
    dims = o.dims
    pts = o.gridpoints()
    o.close()
    slot1 = np.stack([fields.blob_sum(pts, seed=2000 + v, zmax=20000.0, noise=w.get("noise", 0.0))
                      for v in range(dims["nvars"])])
    del pts
    one_var = w["precision"] == "f32"  # the 400-cell grid's FP64 oracle exceeds host RAM with all 8 variables
    times = []
    for i in range(args.warmup + args.steps):
        if one_var:
            dt, _ = _oracle_roundtrip(gp, slot1, threads, var_index=i % dims["nvars"])
        else:
            dt, _ = _oracle_roundtrip(gp, slot1, threads)
        if i >= args.warmup:
            times.append(dt)
    per = sum(times) / len(times)
    units = 1.0 / dims["nvars"] if one_var else 1.0  # round trips per step
    val = units / per
    config = dict(_config(wl, dims), parallelism="replicas" if ws > 1 else "single")
    sample = ("every variable of the grid per step (one full round trip, spectralTransform! + "
              "gridTransform!), FP64 C port of the reference path, OpenMP over rings and columns")
    if one_var:
        sample = ("one variable per step (1/%d of a round trip, variables in turn), FP64 C port of the "
                  "reference path; value = round trips per second of measured time" % dims["nvars"])
    line = {
        "impl": "reference", "metric": "RLZ transforms/s", "value": val, "unit": "round trips/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup, "ms_per_step": per * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config,
        "cpu_baseline": {"value": val, "unit": "round trips/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "round trips/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "Julia/FFTW are not installed; the reference arm runs the oracle's C restatement",
    }
    print(json.dumps(line), flush=True)
    return 0


def measure(wl, args, lib, ws, rank, local, cpu_baseline=True):
    """Device-resident and end-to-end round trips of workload `wl`, the live stage
    roofline, the CPU baseline (oracle) and a check of the GPU output against it."""
    import torch

    import springsteel_gpu as S
    from springsteel_gpu import abi

    gp = _params(wl)
    grid = S.createGrid(gp)
    dims = grid.dims
    w = 4 if gp.precision == "f32" else 8
    h_in = _device_inputs(grid, wl, seed=2 + rank)
    n_out = dims["n_physical"] * dims["nvars"] * dims["nslots"]
    h_out = torch.empty(n_out, dtype=torch.float64 if w == 8 else torch.float32).pin_memory()
    dt_code = abi.SS_DTYPE_F64 if w == 8 else abi.SS_DTYPE_F32
    h2d = h_in.numel() * h_in.element_size()
    d2h = h_out.numel() * h_out.element_size()

    def chk(st):
        S._check(st)

    stream = torch.cuda.ExternalStream(grid.stream())

    def step():
        chk(lib.ss_spectral_transform(grid.handle, None))
        chk(lib.ss_grid_transform(grid.handle, None))

    for _ in range(max(args.warmup, 3)):
        step()
    grid.synchronize()

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        grid.synchronize()

    # ---- device-resident timed region (with live stage events)
    chk(lib.ss_grid_profile(grid.handle, 1))
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        ev1.synchronize()
        barrier()
    ms = ev0.elapsed_time(ev1)
    stage_ms = (C.c_double * 6)()
    launches = (C.c_int64 * 6)()
    chk(lib.ss_grid_profile_read(grid.handle, stage_ms, launches))
    chk(lib.ss_grid_profile(grid.handle, 0))
    ms = _max_over_ranks(ms)
    ms_step = ms / args.steps
    value = ws * args.steps / (ms / 1e3)

    # ---- end to end through the C ABI with host buffers: the reference-facing
    # calls spectralTransform!(grid) / gridTransform!(grid) on a host physical
    # array (slot 1 in, every slot out), the copies of each radial chunk
    # overlapping the transforms of the others
    e2e_steps = max(1, min(args.steps, 10))

    def e2e_loop(overlapped):
        phases = []
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            ta = time.perf_counter()
            if overlapped:
                chk(lib.ss_spectral_transform_from_host(grid.handle, C.c_void_p(h_in.data_ptr()), dt_code, None))
                tb = time.perf_counter()
                chk(lib.ss_grid_transform_to_host(grid.handle, C.c_void_p(h_out.data_ptr()), dt_code, None))
            else:  # upload, both transforms, download, one after the other
                chk(lib.ss_upload_physical(grid.handle, C.c_void_p(h_in.data_ptr()), dt_code, 1, None))
                tb = time.perf_counter()
                step()
                chk(lib.ss_download_physical(grid.handle, C.c_void_p(h_out.data_ptr()), dt_code, 0, None))
            tc = time.perf_counter()
            phases.append(((tb - ta) * 1e3, (tc - tb) * 1e3))
        barrier()
        e2e_s = _max_over_ranks(time.perf_counter() - t0)
        return ws * e2e_steps / e2e_s, [round(float(np.median([p[i] for p in phases])), 2) for i in range(2)]

    with ClockSampler(local) as e2e_clk:
        e2e_val, (ph_in, ph_out) = e2e_loop(True)
        seq_val, (sq_up, sq_rest) = e2e_loop(False)
    e2e_phase_ms = {"spectral_from_host": ph_in, "grid_to_host": ph_out}
    # stage events of one overlapped round trip (chunked launches); its output is
    # the one round trip of h_in that the check below compares with the oracle
    chk(lib.ss_grid_profile(grid.handle, 1))
    chk(lib.ss_spectral_transform_from_host(grid.handle, C.c_void_p(h_in.data_ptr()), dt_code, None))
    chk(lib.ss_grid_transform_to_host(grid.handle, C.c_void_p(h_out.data_ptr()), dt_code, None))
    grid.synchronize()
    ov_ms, ov_n = (C.c_double * 6)(), (C.c_int64 * 6)()
    chk(lib.ss_grid_profile_read(grid.handle, ov_ms, ov_n))
    chk(lib.ss_grid_profile(grid.handle, 0))
    e2e_phase_ms["stage_ms"] = {abi.STAGES[i]: round(ov_ms[i], 2) for i in range(6)}
    e2e_phase_ms["launches"] = [int(ov_n[i]) for i in range(6)]
    e2e_sequential = {"value": seq_val, "upload_ms": sq_up, "transforms_and_download_ms": sq_rest}

    # ---- roofline of the dominant stage
    sb = _stage_bytes(dims, w)
    names = abi.STAGES
    per_step_ms = {names[i]: stage_ms[i] / args.steps for i in range(6)}
    dom = max(per_step_ms, key=per_step_ms.get)
    peak, peak_kind = _peaks()
    achieved = sb[dom] / (per_step_ms[dom] * 1e-3) / 1e9
    path_gbs = _bytes_per_roundtrip(dims, w) / (ms_step * 1e-3) / 1e9
    traffic = MEASURED_TRAFFIC.get((wl, dom))
    roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic,
            "traffic_source": ("ncu capture of this full-size workload: dram__bytes_read.sum + "
                               "dram__bytes_write.sum over the stage's launches of one round trip") if traffic else None,
            "traffic_over_algorithmic": traffic / sb[dom] if traffic else None,
            "algorithmic_bytes_per_step": sb[dom],
            "launches_per_step": int(launches[names.index(dom)]) // max(args.steps, 1),
            "stage_ms_per_step": per_step_ms,
            "stage_traffic_per_step": {k: MEASURED_TRAFFIC.get((wl, k)) for k in names},
            "stage_algorithmic_bytes_per_step": sb,
            "path_achieved_gbs": path_gbs, "path_frac": path_gbs / peak}
    gpu_launches = int(sum(launches[i] for i in range(6)))
    # the ring stages are bound by the arithmetic pipe of the compute type, not by
    # HBM: their conventional FFT flops (2.5·L·log2 L per real length-L transform;
    # 5 inverse and 1 forward transform per ring, z-mode and variable) over the live
    # stage time, against a dense matmul of the same type timed here
    pipe_peak = _matmul_tflops(torch.float64 if w == 8 else torch.float32)
    ring_flops = _ring_fft_flops(dims)
    roof["pipe"] = {
        "unit": "TFLOP/s", "peak": pipe_peak,
        "peak_source": "torch.matmul %s 4096^3 on this GPU, best of 3" % ("float64" if w == 8 else "float32"),
        "flop_model": "2.5*L*log2(L) per real ring transform (FFT convention)",
    }
    for st, nt in (("ring_inverse", 5), ("ring_forward", 1)):
        t = per_step_ms[st] * 1e-3
        roof["pipe"][st] = {"achieved": nt * ring_flops / t / 1e12, "frac": nt * ring_flops / t / 1e12 / pipe_peak}

    res = {
        "metric": "RLZ transforms/s", "value": value, "unit": "round trips/s", "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if w == 8 else "f32",
        "data": "synthetic", "config": dict(_config(wl, dims), parallelism="replicas" if ws > 1 else "single"),
        "clocks": clk.summary(),
        "e2e": {"value": e2e_val, "unit": "round trips/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "steps": e2e_steps, "api": "ss_spectral_transform_from_host + ss_grid_transform_to_host",
                "phase_ms": e2e_phase_ms, "sequential_copies": e2e_sequential, "clocks": e2e_clk.summary()},
        "gpu_launches": gpu_launches,
        "roofline": roof,
    }
    if rank == 0 and cpu_baseline:
        threads = os.cpu_count() or 1
        slot1 = h_in.numpy()
        nv = dims["nvars"]
        one_var = w == 4  # the 400-cell grid's FP64 oracle holds ~10 GB per variable
        dt, phys_o = _oracle_roundtrip(gp, slot1.astype(np.float64), threads, var_index=0 if one_var else None)
        out = h_out.numpy().reshape(dims["nslots"], nv, dims["n_physical"])
        errs = _slot_errors(lambda v, s: out[s, v].astype(np.float64), phys_o, gp)
        units = 1.0 / nv if one_var else 1.0
        res["cpu_baseline"] = {
            "value": units / dt, "unit": "round trips/s", "cores": threads, "kind": "port",
            "sample": ("variable 1 of %d of the same grid and inputs (host RAM), forward+inverse, FP64 C port "
                       "(oracle), %.2f s; value = 1/%d round trip over that time" % (nv, dt, nv)) if one_var else
                      ("every variable of the same grid and inputs, one round trip (forward+inverse), FP64 C port "
                       "(oracle), %.2f s" % dt)}
        tol = np.broadcast_to(np.asarray(CHECK_TOLERANCE[gp.precision], np.float64), (dims["nslots"],))
        worst = errs.max(axis=0)
        res["check"] = {
            "against": "FP64 oracle on the same inputs, one round trip",
            "variables": [0] if one_var else list(range(nv)),
            "max_rel_err_per_slot": [float(x) for x in worst],
            "max_rel_err": float(errs.max()), "tolerance_per_slot": [float(x) for x in tol],
            "pass": bool(np.all(worst <= tol))}
    grid.close()
    return res


def run_ours(args):
    import torch

    import springsteel_gpu as S

    ws, rank, local = _dist()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    lib = S.load_library()
    line = measure(args.workload, args, lib, ws, rank, local, cpu_baseline=not args.no_cpu_baseline)
    if args.workload == "rlz200-f64" and not args.no_secondary:
        # the FP32+refinement 400-cell grid, measured in the same run
        sec = measure("rlz400-f32", args, lib, ws, rank, local, cpu_baseline=not args.no_cpu_baseline)
        line["secondary"] = {"rlz400-f32": sec}
    if ws > 1:
        torch.distributed.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    failed = [c for c in [line.get("check")] + [v.get("check") for v in line.get("secondary", {}).values()]
              if c and not c["pass"]]
    return 3 if failed else 0


def run_cufft_comparison(args):
    """Comparison point only, never the product path: the vendor FFT (cuFFT through
    torch.fft) timed on the same ring lengths and batch sizes as the workload's
    ring stages — one batched C2R per ring with the inverse stage's 5 real
    outputs per (variable, Chebyshev mode), one batched R2C per ring for the
    forward stage.  It leaves out what the library's ring kernels also do (the
    phase rotation, the λ-derivative scaling, the packed-row gathers), so it is
    a lower bound on a cuFFT-based ring stage.  Prints one JSON line."""
    import torch

    _, rank, local = _dist()
    if rank != 0:
        return 0
    torch.cuda.set_device(local)
    from springsteel_gpu import abi  # noqa: F401  (same package path as the main arms)

    gp = _params(args.workload)
    w = WORKLOADS[args.workload]
    nrings, pol = gp.num_cells * 3, 0
    items = w["nvars"] * (gp.b_kDim if getattr(gp, "b_kDim", 0) else _bk(w["kDim"]))
    real = torch.float32 if w["precision"] == "f32" else torch.float64
    cplx = torch.complex64 if real == torch.float32 else torch.complex128
    torch.backends.cuda.cufft_plan_cache.max_size = 4096
    out = {}
    for stage, batch, inverse in (("ring_inverse", 5 * items, True), ("ring_forward", items, False)):
        xs = []
        for r in range(1, nrings + 1):
            L = 4 + 4 * (r + pol)
            xs.append((L, torch.randn(batch, L // 2 + 1, dtype=cplx, device="cuda") if inverse
                       else torch.randn(batch, L, dtype=real, device="cuda")))

        def one():
            for L, x in xs:
                torch.fft.irfft(x, n=L) if inverse else torch.fft.rfft(x)

        for _ in range(max(args.warmup, 1)):
            one()
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(max(args.steps, 1)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            one()
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1))
        out[stage] = {"ms": best, "transforms_per_ring": batch, "rings": nrings}
        del xs
        torch.cuda.empty_cache()
    print(json.dumps({"comparison": "cuFFT (torch.fft, %s) on the ring lengths 4+4r, r = 1..%d" % (
        torch.version.cuda, nrings), "workload": args.workload, "dtype": str(real).replace("torch.", ""),
        "stages": out}), flush=True)
    return 0


def _bk(kz):
    """b_kDim of a kz-level Chebyshev column (src/Springsteel.jl:425-465)."""
    return min(kz, (2 * kz - 1) // 3 + 1)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="rlz200-f64", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-secondary", action="store_true", help="skip the FP32 400-cell grid of the default run")
    ap.add_argument("--cufft-comparison", action="store_true",
                    help="time cuFFT on the workload's ring lengths instead (comparison point only)")
    args = ap.parse_args()
    if args.cufft_comparison:
        return run_cufft_comparison(args)
    if args.workload == "elliptic-rl200":
        return run_elliptic(args)
    if args.workload.startswith("batch-"):
        return run_batch(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
