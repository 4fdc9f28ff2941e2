"""GPU batches (CUDA graph, autotuner), RL chain coupling and radial tiles."""
import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from springsteel_gpu import fields
from test_gpu_parity import TOL64, slot_errors

pytestmark = pytest.mark.gpu


def _fill(g, seed):
    pts = S.getGridpoints(g)
    nv = g.dims["nvars"]
    u = np.empty((pts.shape[0], nv), order="F")
    for v in range(nv):
        u[:, v] = fields.blob_sum(pts, seed=seed * 10 + v, nblobs=6, wmin=3.0, wmax=12.0,
                                  zmax=max(g.params.kMax, 1.0))
    g.set_physical(u, slot=1)
    return u


def test_rl_chain_40_120_40_parity():
    ps = S.chain_grid_params([0.0, 40.0, 100.0, 140.0], [40, 120, 40], vars={"u": 1, "w": 2})
    gs = [S.createGrid(p) for p in ps]
    os_ = [O.OracleGrid(p.to_abi()) for p in ps]
    specs = []
    for i, (g, o) in enumerate(zip(gs, os_)):
        u = _fill(g, seed=i + 1)
        ph = np.zeros(o.physical_shape, order="F")
        ph[:, :, 0] = u
        specs.append(o.spectral_transform(ph))
        S.spectralTransform_b(g)
    chain = S.PatchChain(gs)
    och = O.OracleChain(os_)
    # two calls in a row: the second sees the shared spline-object ahat state the
    # first left behind, as the reference's reused spline objects do
    for _ in range(2):
        chain.multiGridTransform()
        ref = och.multi_grid_transform(specs)
        for p, g, r in zip(ps, gs, ref):
            errs = slot_errors(g.get_physical(), r, p)
            assert np.all(errs <= TOL64), errs


def test_rlz_chain_parity():
    """RLZ patches coupled per Chebyshev level and wavenumber (_rlz_kernel!,
    src/multipatch.jl:496-571): a 2-patch chain (2:1 at the interface) and the
    3-patch 40/120/40-shaped chain at reduced size, twice in a row."""
    col = dict(kMin=0.0, kMax=20000.0, kDim=16, BCB={"default": S.DirichletBC()}, BCT={"default": S.NeumannBC()})
    for bounds, cells in (([0.0, 20.0, 30.0], [10, 10]), ([0.0, 12.0, 30.0, 42.0], [6, 18, 6])):
        ps = S.chain_grid_params(bounds, cells, vars={"u": 1, "w": 2}, geometry="RLZ", **col)
        gs = [S.createGrid(p) for p in ps]
        os_ = [O.OracleGrid(p.to_abi()) for p in ps]
        specs = []
        for i, (g, o) in enumerate(zip(gs, os_)):
            u = _fill(g, seed=i + 5)
            ph = np.zeros(o.physical_shape, order="F")
            ph[:, :, 0] = u
            specs.append(o.spectral_transform(ph))
            S.spectralTransform_b(g)
        chain = S.PatchChain(gs)
        och = O.OracleChain(os_)
        for _ in range(2):
            chain.multiGridTransform()
            ref = och.multi_grid_transform(specs)
            for p, g, r in zip(ps, gs, ref):
                errs = slot_errors(g.get_physical(), r, p)
                assert np.all(errs <= TOL64), errs


def test_two_patch_chain_linear_exactness():
    gp1 = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=50.0, num_cells=10)
    gp2 = S.SpringsteelGridParameters(geometry="RL", iMin=50.0, iMax=75.0, num_cells=10,
                                      BCL={"u": S.FixedBC()}, BCR={"u": S.NaturalBC()})
    gs = [S.createGrid(gp) for gp in (gp1, gp2)]
    for g in gs:
        pts = S.getGridpoints(g)
        g.set_physical((3 * pts[:, 0] + 7)[:, None], slot=1)
        S.spectralTransform_b(g)
    S.PatchChain(gs).multiGridTransform()
    pts2 = S.getGridpoints(gs[1])
    assert np.max(np.abs(gs[1].get_physical()[:, 0, 0] - (3 * pts2[:, 0] + 7))) < 1e-8


@pytest.mark.parametrize("fused", [False, True])
@pytest.mark.parametrize("use_graph,autotune", [(True, False), (False, True), (True, True)])
def test_batch_matches_single_grid_calls(use_graph, autotune, fused):
    rng = np.random.default_rng(7)
    grids, refs, inputs = [], [], []
    for i in range(6):
        nc = int(rng.integers(8, 30))
        nv = int(rng.integers(1, 4))
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=float(nc), num_cells=nc,
                                         vars={"v%d" % k: k + 1 for k in range(nv)})
        g = S.createGrid(gp)
        inputs.append(_fill(g, seed=i))
        S.spectralTransform_b(g)
        S.gridTransform_b(g)
        refs.append(g.get_physical())
        grids.append(g)
    batch = S.Batch(grids, autotune=autotune, fused=fused)
    for _ in range(2):  # capture, then replay; gridTransform! overwrites the value slot
        for g, u in zip(grids, inputs):
            g.set_physical(u, slot=1)
        batch.run(what=3, use_graph=use_graph)
        batch.synchronize()
    for g, r in zip(grids, refs):
        assert np.array_equal(g.get_physical(), r)
    if autotune:
        assert all(t in (64, 128, 256) for i in range(6) for t in batch.ring_threads(i))


@pytest.mark.parametrize("fused", [False, True])
def test_batch_graph_recaptured_after_filter_and_ahat_changes(fused):
    """A batch graph holds each grid's launch arguments (filter flag, ahat
    pointer); changing them between runs re-captures it, so replays equal fresh
    single-grid calls with the new settings."""
    import ctypes as C

    lib = S.load_library()
    gps = [S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=20.0, num_cells=20),
           S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=20.0, num_cells=12,
                                       BCL={"default": S.FixedBC()})]
    grids = [S.createGrid(gp) for gp in gps]
    inputs = [_fill(g, seed=20 + i) for i, g in enumerate(grids)]
    b1 = grids[1].dims["b_iDim"]
    ahat = np.zeros(b1)
    ahat[:3] = (0.7, -0.2, 0.4)
    batch = S.Batch(grids, fused=fused)

    def run_batch():
        for g, u in zip(grids, inputs):
            g.set_physical(u, slot=1)
        batch.run(what=3, use_graph=True)
        batch.synchronize()
        return [g.get_physical() for g in grids]

    def singles():
        out = []
        for g, u in zip(grids, inputs):
            g.set_physical(u, slot=1)
            S.spectralTransform_b(g)
            S.gridTransform_b(g)
            out.append(g.get_physical())
        return out

    run_batch()  # captured without filter or ahat
    K = grids[0].dims["kDim_wn"]
    fw = np.array([1.0 if k <= 4 else 0.0 for k in range(K + 1)])
    S._check(lib.ss_grid_set_filter(grids[0].handle, 0, fw.ctypes.data_as(C.c_void_p), None))
    grids[1].set_wavenumber_ahat(0, 0, ahat)
    got, ref = run_batch(), singles()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    grids[1].clear_wavenumber_ahat()  # frees the registry the captured graph pointed to
    got, ref = run_batch(), singles()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
    batch.close()


def _sum_spectral_tile(patch_spec, tile_spec, pp, tp):
    """sumSpectralTile! for RLZ (src/tiling.jl:1101-1136) on host arrays."""
    siL = tp.spectralIndexL
    bp, bt, bk = pp.b_iDim, tp.b_iDim, tp.b_kDim
    kp, kt = pp.iDim + pp.patchOffsetL, tp.iDim + tp.patchOffsetL
    sp, st = bp * (1 + 2 * kp), bt * (1 + 2 * kt)
    for zb in range(bk):
        for blk in range(1 + 2 * kt):
            p0 = zb * sp + blk * bp + siL - 1
            t0 = zb * st + blk * bt
            patch_spec[p0:p0 + bt, :] += tile_spec[t0:t0 + bt, :]


def test_rlz_tiles_halo_sum_matches_oracle():
    gp = fields.rlz_params(num_cells=40, nvars=2)
    patch = S.createGrid(gp)
    u = _fill(patch, seed=9)
    S.spectralTransform_b(patch)
    b_patch = patch.get_spectral()  # B-vectors: quadrature sums, so tile halos add up to them
    tps = S.calcTileSizes(gp, 8)
    tiles = [S.createGrid(tp) for tp in tps]
    assert sum(tp.num_cells for tp in tps) == gp.num_cells
    S.zero_spectral(patch)
    for t in tiles:
        S.tile_physical_from_patch(patch, t, slot=1)
        S.spectralTransform_b(t, stream=patch.stream())
        S.sumSpectralTile_b(patch, t, stream=patch.stream())
    patch.synchronize()
    got = patch.get_spectral()
    # oracle: each tile's own spectralTransform! on its rows of the field, summed by the reference's layout
    ref = np.zeros_like(b_patch)
    row0 = 0
    tile_specs = []
    for tp in tps:
        o = O.OracleGrid(tp.to_abi())
        n = o.physical_shape[0]
        ph = np.zeros(o.physical_shape, order="F")
        ph[:, :, 0] = u[row0:row0 + n]
        row0 += n
        tile_specs.append(o.spectral_transform(ph))
        _sum_spectral_tile(ref, tile_specs[-1], gp, tp)
    assert row0 == u.shape[0]
    scale = np.max(np.abs(ref))
    assert np.max(np.abs(got - ref)) <= TOL64 * scale
    assert np.max(np.abs(got - b_patch)) <= TOL64 * scale
    # the halo-summed spectral array evaluates through the patch like any other
    S.gridTransform_b(patch)
    oref = O.OracleGrid(gp.to_abi()).grid_transform(ref)
    errs = slot_errors(patch.get_physical(), oref, gp)
    assert np.all(errs <= TOL64), errs
    # setSpectralTile! zeroes the patch, then writes one tile's blocks
    S.setSpectralTile_b(patch, tiles[0], stream=patch.stream())
    patch.synchronize()
    one = np.zeros_like(ref)
    _sum_spectral_tile(one, tile_specs[0], gp, tps[0])
    assert np.max(np.abs(patch.get_spectral() - one)) <= TOL64 * np.max(np.abs(one))


# binary32 bulk with the FP64-refined spline solve (RL): f near 2e-7 of its scale,
# the derivative slots amplify the binary32 rounding of the ring transforms
F32_RL_BOUNDS = np.array([2e-6, 5e-5, 5e-5, 5e-5, 5e-5])


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_fused_batch_config3_range_matches_oracle(precision):
    """Uneven RL grids of the batched workload's ranges (50-400 cells, 1-4
    variables) in one fused batch, against the oracle grid by grid; then the
    same batch with per-grid launch sequences gives bit-identical results."""
    rng = np.random.default_rng(11)
    grids, oracles, params, inputs = [], [], [], []
    for i in range(8):
        nc = int(rng.integers(50, 401)) if i else 400
        nv = int(rng.integers(1, 5))
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=float(nc), num_cells=nc,
                                         vars={"v%d" % k: k + 1 for k in range(nv)}, precision=precision)
        g = S.createGrid(gp)
        inputs.append(_fill(g, seed=40 + i))
        grids.append(g)
        oracles.append(O.OracleGrid(gp.to_abi()))
        params.append(gp)
    fused = S.Batch(grids, autotune=True, fused=True)  # the autotuner's timed runs overwrite slot 1
    assert fused.fused_launches(3) <= 20  # a few launches per stage for all 8 grids
    for g, u in zip(grids, inputs):
        g.set_physical(u, slot=1)
    fused.run(what=3, use_graph=True)
    fused.synchronize()
    outs = [g.get_physical() for g in grids]
    for g, o, gp, u, out in zip(grids, oracles, params, inputs, outs):
        ph = np.zeros(o.physical_shape, order="F")
        ph[:, :, 0] = u.astype(np.float32).astype(np.float64) if precision == "f32" else u
        ref = o.grid_transform(o.spectral_transform(ph))
        errs = slot_errors(out, ref, gp)
        bound = TOL64 if precision == "f64" else F32_RL_BOUNDS
        assert np.all(errs <= bound), (gp.num_cells, errs.max(axis=0))
    plain = S.Batch(grids, fused=False)
    for g, u in zip(grids, inputs):
        g.set_physical(u, slot=1)
    plain.run(what=3, use_graph=False)
    plain.synchronize()
    for g, out in zip(grids, outs):
        assert np.array_equal(g.get_physical(), out)


def test_embedded_three_level_linear_exactness():
    """PatchEmbedded (src/multipatch.jl:891-925; test/multipatch.jl:1121-1164): radial
    splines nested [0, 30] ⊃ [10, 20] ⊃ [13, 17] (DX 1, 0.5, 0.25), l_q = 0; f = 2r + 1
    is reproduced to 1e-10 on every level, the inner grids through R3X data at both ends."""
    ps = S.embedded_grid_params([(0.0, 30.0), (10.0, 20.0), (13.0, 17.0)], [30, 20, 16], l_q={"default": 0.0},
                                BCL={"default": S.R0}, BCR={"default": S.R0})
    gs = [S.createGrid(p) for p in ps]
    for g in gs:
        pts = S.getGridpoints(g)
        g.set_physical((2 * pts[:, 0] + 1)[:, None], slot=1)
        S.spectralTransform_b(g)
    S.PatchEmbedded(gs).multiGridTransform()
    for g in gs:
        pts = S.getGridpoints(g)
        assert np.max(np.abs(g.get_physical()[:, 0, 0] - (2 * pts[:, 0] + 1))) < 1e-10


@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
def test_embedded_parity(geometry):
    """Embedded multigrid against the oracle's (two levels, two variables), twice in
    a row: the second run sees the spline-object backgrounds the first left."""
    col = {} if geometry == "RL" else dict(kMin=0.0, kMax=2000.0, kDim=12, BCB={"default": S.DirichletBC()},
                                           BCT={"default": S.NeumannBC()})
    ps = S.embedded_grid_params([(0.0, 36.0), (12.0, 24.0), (15.0, 21.0)], [18, 12, 12], vars={"u": 1, "w": 2},
                                geometry=geometry, **col)
    gs = [S.createGrid(p) for p in ps]
    os_ = [O.OracleGrid(p.to_abi()) for p in ps]
    specs = []
    for i, (g, o) in enumerate(zip(gs, os_)):
        u = _fill(g, seed=60 + i)
        ph = np.zeros(o.physical_shape, order="F")
        ph[:, :, 0] = u
        specs.append(o.spectral_transform(ph))
        S.spectralTransform_b(g)
    emb = S.PatchEmbedded(gs)
    och = O.OracleChain(os_, embedded=True)
    for _ in range(2):
        emb.multiGridTransform()
        ref = och.multi_grid_transform(specs)
        for p, g, r in zip(ps, gs, ref):
            errs = slot_errors(g.get_physical(), r, p)
            assert np.all(errs <= TOL64), errs
