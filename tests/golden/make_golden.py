"""Generate the committed golden fixtures of small RL/RLZ round trips.

The reference (Julia) cannot run on these machines and ships no golden arrays,
so the fixtures are outputs of the FP64 oracle (the C restatement of the
reference path) on seeded inputs, at sizes small enough to commit.  They pin the
oracle itself (a change to the restatement shows up as a fixture mismatch, a
CPU test) and give the CUDA path a fixed target that needs no oracle run (a GPU
test).  Run from the repository root:

    python tests/golden/make_golden.py

Each case stores its grid parameters (JSON), the physical slot-1 input
(n_physical × nvars, column-major as the reference), the spectral array after
spectralTransform! and every physical slot after gridTransform!.
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "springsteel.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
import springsteel_gpu as S  # noqa: E402
from springsteel_gpu import fields  # noqa: E402
from springsteel_gpu.io import _params_json  # noqa: E402


def cases():
    """(name, parameters, input seed, z extent) of every fixture."""
    return [
        ("rl10_natural", S.SpringsteelGridParameters(
            geometry="RL", iMin=0.0, iMax=10.0, num_cells=10, vars={"u": 1},
            BCL={"default": S.NaturalBC()}, BCR={"default": S.NaturalBC()}), 11, None),
        ("rl8_two_vars_bcs", S.SpringsteelGridParameters(
            geometry="RL", iMin=0.0, iMax=16.0, num_cells=8, vars={"u": 1, "v": 2},
            BCL={"u": S.NaturalBC(), "v": S.NaturalBC()},
            BCR={"u": S.DirichletBC(), "v": S.NeumannBC()}), 12, None),
        ("rlz4_k10_dirichlet", S.SpringsteelGridParameters(
            geometry="RLZ", iMin=0.0, iMax=8.0, num_cells=4, kMin=0.0, kMax=100.0, kDim=10, vars={"w": 1},
            BCL={"default": S.NaturalBC()}, BCR={"default": S.NaturalBC()},
            BCB={"default": S.DirichletBC()}, BCT={"default": S.DirichletBC()}), 13, (0.0, 100.0)),
    ]


def compute(gp, seed, zext):
    o = O.OracleGrid(gp.to_abi())
    pts = o.gridpoints()
    nv = o.physical_shape[1]
    ph = np.zeros(o.physical_shape, order="F")
    for v in range(nv):
        kw = dict(zmin=zext[0], zmax=zext[1], vert=0.2) if zext else {}
        ph[:, v, 0] = fields.blob_sum(pts, seed=seed * 100 + v, nblobs=4, wmin=2.0, wmax=6.0, **kw)
    spec = o.spectral_transform(ph)
    phys = o.grid_transform(spec)
    o.close()
    return ph[:, :, 0].copy(order="F"), spec, phys


def main():
    for name, gp, seed, zext in cases():
        slot1, spec, phys = compute(gp, seed, zext)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), params=json.dumps(_params_json(gp)),
                            slot1=slot1, spectral=spec, physical=phys)
        print(name, slot1.shape, spec.shape, phys.shape)


if __name__ == "__main__":
    main()
