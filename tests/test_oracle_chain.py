"""Oracle multipatch chain and tiling host logic (test/multipatch.jl:1258-1340,
src/tiling.jl:185-259)."""
import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from springsteel_gpu import fields


def _two_patch():
    gp1 = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=50.0, num_cells=10)
    gp2 = S.SpringsteelGridParameters(geometry="RL", iMin=50.0, iMax=75.0, num_cells=10,
                                      BCL={"u": S.FixedBC()}, BCR={"u": S.NaturalBC()})
    return [O.OracleGrid(gp.to_abi()) for gp in (gp1, gp2)]


def _chain_out(gs, f):
    sp = []
    for g in gs:
        pts = g.gridpoints()
        ph = np.zeros(g.physical_shape, order="F")
        ph[:, 0, 0] = f(pts)
        sp.append(g.spectral_transform(ph))
    return O.OracleChain(gs).multi_grid_transform(sp)


def test_chain_linear_exactness():
    # test/multipatch.jl:1258-1283: f = 3r + 7 on the secondary within 1e-8
    gs = _two_patch()
    out = _chain_out(gs, lambda p: 3 * p[:, 0] + 7)
    pts2 = gs[1].gridpoints()
    assert np.max(np.abs(out[1][:, 0, 0] - (3 * pts2[:, 0] + 7))) < 1e-8


@pytest.mark.parametrize("trig", [np.cos, np.sin])
def test_chain_wavenumber1_coupling(trig):
    # test/multipatch.jl:1285-1340: r·cos λ and r·sin λ within 0.5
    gs = _two_patch()
    out = _chain_out(gs, lambda p: p[:, 0] * trig(p[:, 1]))
    pts2 = gs[1].gridpoints()
    assert np.max(np.abs(out[1][:, 0, 0] - pts2[:, 0] * trig(pts2[:, 1]))) < 0.5


def test_chain_params_follow_create_chain_rules():
    ps = S.chain_grid_params([0.0, 40.0, 100.0, 140.0], [40, 120, 40])
    assert [p.patchOffsetL for p in ps] == [0, 120, 480]
    assert S._bc_to_spline(ps[1].BCL["default"]) == S.R3X and S._bc_to_spline(ps[1].BCR["default"]) == S.R3X
    assert S._bc_to_spline(ps[0].BCR["default"]) == S.R0 and S._bc_to_spline(ps[2].BCL["default"]) == S.R0
    with pytest.raises(ValueError):
        S.chain_grid_params([0.0, 30.0, 40.0], [10, 30])  # 3:1


def test_chain_rejects_unsupported_ratio():
    gp1 = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=30.0, num_cells=10)
    gp2 = S.SpringsteelGridParameters(geometry="RL", iMin=30.0, iMax=40.0, num_cells=10,
                                      BCL={"u": S.FixedBC()})
    with pytest.raises(O.OracleError):
        O.OracleChain([O.OracleGrid(gp.to_abi()) for gp in (gp1, gp2)])


@pytest.mark.parametrize("ntiles", [1, 2, 5, 8])
def test_calc_tile_sizes_cover_patch(ntiles):
    gp = fields.rlz_params()
    tiles = S.calcTileSizes(gp, ntiles)
    assert sum(t.num_cells for t in tiles) == gp.num_cells
    assert all(t.num_cells >= 3 for t in tiles)
    assert tiles[0].iMin == gp.iMin and tiles[-1].iMax == gp.iMax
    for a, b in zip(tiles, tiles[1:]):
        assert a.iMax == b.iMin and b.spectralIndexL == a.spectralIndexL + a.num_cells
        assert b.patchOffsetL == (b.spectralIndexL - 1) * gp.mubar


def test_calc_tile_sizes_too_many():
    with pytest.raises(ValueError):
        S.calcTileSizes(S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=10.0, num_cells=10), 4)


def test_oracle_tiles_sum_to_patch_spectral():
    # forward transform of tiles + halo sum equals the patch's forward transform
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=40.0, num_cells=20, kMin=0.0, kMax=100.0,
                                     kDim=8)
    og = O.OracleGrid(gp.to_abi())
    pts = og.gridpoints()
    ph = np.zeros(og.physical_shape, order="F")
    ph[:, 0, 0] = fields.blob_sum(pts, seed=3, nblobs=5, wmin=3, wmax=8, zmax=100.0)
    ref = og.spectral_transform(ph)
    acc = np.zeros_like(ref)
    b = og.dims["b_iDim"]
    row = 0
    for tp in S.calcTileSizes(gp, 4):
        ot = O.OracleGrid(tp.to_abi())
        n = ot.dims["n_physical"]
        pt = np.zeros(ot.physical_shape, order="F")
        pt[:, 0, 0] = ph[row:row + n, 0, 0]
        row += n
        st = ot.spectral_transform(pt)
        bt, Kt, Kp = ot.dims["b_iDim"], ot.dims["kDim_wn"], og.dims["kDim_wn"]
        off = tp.spectralIndexL - 1
        for zb in range(og.dims["b_kDim"]):
            for blk in range(1 + 2 * Kt):
                p0 = (zb * (1 + 2 * Kp) + blk) * b + off
                t0 = (zb * (1 + 2 * Kt) + blk) * bt
                acc[p0:p0 + bt, 0] += st[t0:t0 + bt, 0]
    assert row == og.dims["n_physical"]
    assert np.max(np.abs(acc - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_embedded_three_level_linear_exactness():
    # test/multipatch.jl:1121-1164 (R geometry there; radial splines of an RL grid
    # here): outer [0, 30] 30 cells, mid [10, 20] 20 cells, inner [13, 17] 16 cells,
    # l_q = 0, f = 2r + 1 reproduced to 1e-10 on every level
    ps = S.embedded_grid_params([(0.0, 30.0), (10.0, 20.0), (13.0, 17.0)], [30, 20, 16], l_q={"default": 0.0},
                                BCL={"default": S.R0}, BCR={"default": S.R0})
    gs = [O.OracleGrid(p.to_abi()) for p in ps]
    sp = []
    for g in gs:
        pts = g.gridpoints()
        ph = np.zeros(g.physical_shape, order="F")
        ph[:, 0, 0] = 2 * pts[:, 0] + 1
        sp.append(g.spectral_transform(ph))
    out = O.OracleChain(gs, embedded=True).multi_grid_transform(sp)
    for g, o in zip(gs, out):
        pts = g.gridpoints()
        assert np.max(np.abs(o[:, 0, 0] - (2 * pts[:, 0] + 1))) < 1e-10


def test_embedded_rejects_equal_resolution_and_misalignment():
    # test/multipatch.jl:1108-1118, 429-443
    with pytest.raises(ValueError):
        S.embedded_grid_params([(0.0, 30.0), (10.0, 20.0)], [30, 10])
    ps = S.embedded_grid_params([(0.0, 30.0), (10.25, 20.25)], [30, 20])
    with pytest.raises(O.OracleError):
        O.OracleChain([O.OracleGrid(p.to_abi()) for p in ps], embedded=True)
