"""GPU parity: the CUDA path through the C ABI against the FP64 oracle.

Relative error of a (variable, slot) block = max|gpu - oracle| / scale, with
scale = max(max|oracle slot|, max|oracle f| / L^d): the slot's own magnitude,
floored by the field's natural scale for a derivative of order d along a
domain of length L (r: iMax - iMin, λ: 1, z: kMax - kMin).  The floor only
matters for derivative slots that vanish analytically (e.g. ∂rr of a field
linear in r), where both sides are pure round-off.
FP64 path tolerance: 1e-12 (the stated FP64 parity bound).  FP32+refinement: below.
"""
import numpy as np
import pytest

import oracle as O
import springsteel_gpu as S
from springsteel_gpu import fields

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
# SS_PREC_F64_FAST: binary64 data, double-float (48-bit) FFT/DCT arithmetic; the
# derivative slots amplify its 2^-48 rounding (by k ≤ K for ∂λ, by the Chebyshev
# recurrence for ∂z), so its stated bound is 2e-11.
TOL_FAST = 2e-11


def _rel(a, b):
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / den) if den > 0 else float(np.max(np.abs(a)))


def _run_both(gp, phys_slot1, ahats=None):
    g = S.createGrid(gp)
    o = O.OracleGrid(gp.to_abi())
    if ahats:
        for (v, blk, a) in ahats:
            g.set_wavenumber_ahat(v, blk, a)
            o.set_ahat(v, blk, a)
    if gp.fourier_filter or gp.chebyshev_filter:
        K, bk = o.dims["kDim_wn"], o.dims["b_kDim"]
        for v, name in enumerate(gp.var_names()):
            ff = S._per_var(gp.fourier_filter, name, None)
            cf = S._per_var(gp.chebyshev_filter, name, None)
            fw = np.array([S._snap(S.filter_weight(ff, k)) for k in range(K + 1)]) if ff else None
            cw = np.array([S._snap(S.filter_weight(cf, z)) for z in range(bk)]) if cf else None
            o.set_filter(v, fw, cw)
    ph = np.zeros(o.physical_shape, order="F")
    ph[:, :, 0] = phys_slot1
    g.set_physical(ph[:, :, 0], slot=1)
    S.spectralTransform_b(g)
    spec_g = g.get_spectral()
    spec_o = o.spectral_transform(ph)
    S.gridTransform_b(g)
    phys_g = g.get_physical()
    phys_o = o.grid_transform(spec_o)
    return g, o, spec_g, spec_o, phys_g, phys_o


# (direction, order) of each physical slot: f, ∂r, ∂rr, ∂λ, ∂λλ, ∂z, ∂zz
SLOT_DERIV = [(None, 0), ("r", 1), ("r", 2), ("l", 1), ("l", 2), ("z", 1), ("z", 2)]


def slot_errors(phys_g, phys_o, gp):
    """Per (var, slot) error with the scale-aware denominator described above."""
    lengths = {"r": gp.iMax - gp.iMin, "l": 1.0, "z": (gp.kMax - gp.kMin) or 1.0}
    out = np.zeros(phys_o.shape[1:])
    for v in range(phys_o.shape[1]):
        fmax = np.max(np.abs(phys_o[:, v, 0]))
        for s in range(phys_o.shape[2]):
            dirn, d = SLOT_DERIV[s]
            floor = fmax / lengths[dirn] ** d if dirn else 0.0
            den = max(np.max(np.abs(phys_o[:, v, s])), floor)
            out[v, s] = np.max(np.abs(phys_g[:, v, s] - phys_o[:, v, s])) / den if den > 0 else 0.0
    return out


def _assert_parity(spec_g, spec_o, phys_g, phys_o, gp, tol=TOL64):
    nv = spec_o.shape[1]
    espec = [_rel(spec_g[:, v], spec_o[:, v]) for v in range(nv)]
    errs = slot_errors(phys_g, phys_o, gp)
    print("parity %s %s: spectral max %.2e, slots max %s" % (gp.geometry, gp.precision, max(espec),
                                                              np.array2string(errs.max(axis=0), precision=2)))
    for v in range(nv):
        assert espec[v] <= tol, ("spectral", v, espec[v])
    bad = [(v, s + 1, errs[v, s]) for v in range(nv) for s in range(errs.shape[1]) if not errs[v, s] <= tol]
    assert not bad, bad


@pytest.mark.parametrize("precision", ["f64", "f64_fast"])
def test_rl100_one_var_parity(precision):
    gp = fields.rl100_params(precision=precision)
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.gaussian_ring_field(pts, seed=1)
    _, _, sg, so, pg, po = _run_both(gp, u[:, None])
    _assert_parity(sg, so, pg, po, gp, tol=TOL64 if precision == "f64" else TOL_FAST)


def test_rl_gridpoints_match_oracle():
    gp = fields.rl100_params()
    g = S.createGrid(gp)
    o = O.OracleGrid(gp.to_abi())
    assert np.max(np.abs(S.getGridpoints(g) - o.gridpoints())) < 1e-13


def test_rl_multivar_bcs_offset_kmax():
    gp = S.SpringsteelGridParameters(
        geometry="RL", iMin=5.0, iMax=65.0, num_cells=20, vars={"a": 1, "b": 2, "c": 3, "d": 4},
        BCL={"a": S.DirichletBC(), "b": S.NeumannBC(), "c": S.CauchyBC(0.0, 0.0), "d": S.ZerosBC()},
        BCR={"a": S.NaturalBC(), "b": S.SecondDerivativeBC(), "c": S.AntisymmetricBC(), "d": S.RobinBC(1.0, -2.0)},
        l_q={"default": 2.0, "c": 0.5}, max_wavenumber={"default": -1, "b": 7, "d": 0},
        spectralIndexL=2)
    g0 = S.createGrid(gp)
    pts = S.getGridpoints(g0)
    u = np.column_stack([fields.blob_sum(pts, seed=s, nblobs=5, wmin=3, wmax=10) for s in range(4)])
    _, _, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp)


def test_rl_r3x_ahat():
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=10.0, iMax=40.0, num_cells=15,
                                     BCL={"default": S.FixedBC()}, BCR={"default": S.NaturalBC()})
    g0 = S.createGrid(gp)
    pts = S.getGridpoints(g0)
    u = (fields.blob_sum(pts, seed=7, nblobs=4, wmin=2, wmax=8) + 0.5)[:, None]
    b = g0.dims["b_iDim"]
    rng = np.random.default_rng(3)
    ahats = []
    for blk in (0, 1, 2, 5, 6):
        a = np.zeros(b)
        a[:3] = rng.normal(size=3)
        ahats.append((0, blk, a))
    _, _, sg, so, pg, po = _run_both(gp, u, ahats)
    _assert_parity(sg, so, pg, po, gp)


def test_rl_filters():
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=30.0, num_cells=10,
                                     fourier_filter={"default": S.SpectralFilter(low_pass=6, notch=[2], window="hann",
                                                                                 taper_width=3)})
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.blob_sum(pts, seed=11, nblobs=6, wmin=2, wmax=6)[:, None]
    _, _, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp)


@pytest.mark.parametrize("bcb,bct", [(S.DirichletBC(), S.DirichletBC()), (S.NaturalBC(), S.NaturalBC()),
                                     (S.NeumannBC(), S.DirichletBC()), (S.NeumannBC(), S.NeumannBC()),
                                     (S.DirichletBC(), S.NaturalBC())])
def test_rlz_parity_bcs(bcb, bct):
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=40.0, num_cells=20, kMin=0.0,
                                     kMax=20000.0, kDim=16, vars={"u": 1, "w": 2},
                                     BCB={"default": bcb}, BCT={"default": bct})
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.rlz_blob_fields(pts, 2, zmax=20000.0)
    _, _, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp)


@pytest.mark.parametrize("precision", ["f64", "f64_fast"])
def test_rlz_5var_kz32_reduced(precision):
    # the configuration-2 layout (kz = 32, 5 variables, Dirichlet in z) at 40 cells
    gp = fields.rlz_params(num_cells=40, precision=precision)
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.rlz_blob_fields(pts, 5, zmax=20000.0)
    _, _, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp, tol=TOL64 if precision == "f64" else TOL_FAST)


def test_rlz_patch_offset_and_filters():
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=40.0, num_cells=4, spectralIndexL=2,
                                     kMin=0.0, kMax=10.0, kDim=8,
                                     fourier_filter={"default": S.GaussianFilter(sigma=6.0, order=2)},
                                     chebyshev_filter={"default": S.SpectralFilter(low_pass=3)})
    pts = S.getGridpoints(S.createGrid(gp))
    u = (pts[:, 0] * pts[:, 2] + np.cos(3 * pts[:, 1]) * pts[:, 0] / 40.0)[:, None]
    _, _, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp)


def test_rl_linear_field_exact():
    # f = 3r + 7 is reproduced exactly by the cubic B-spline fit (test/multipatch.jl:1258-1283 pattern)
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=120.0, num_cells=60)
    g = S.createGrid(gp)
    pts = S.getGridpoints(g)
    g.set_physical((3 * pts[:, 0] + 7)[:, None], slot=1)
    S.spectralTransform_b(g)
    S.gridTransform_b(g)
    ph = g.get_physical()
    assert np.max(np.abs(ph[:, 0, 0] - (3 * pts[:, 0] + 7))) < 1e-8
    assert np.max(np.abs(ph[:, 0, 1] - 3.0)) < 1e-8
    assert np.max(np.abs(ph[:, 0, 2])) < 1e-8


def test_fp32_refined_error_vs_fp64_oracle():
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=40.0, num_cells=20, kMin=0.0,
                                     kMax=20000.0, kDim=16, vars={"u": 1},
                                     BCB={"default": S.DirichletBC()}, BCT={"default": S.DirichletBC()},
                                     precision="f32")
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.rlz_blob_fields(pts, 1, zmax=20000.0)
    _, o, sg, so, pg, po = _run_both(gp, u)
    errs = slot_errors(pg, po, gp)
    assert np.all(errs < 1e-4), errs


@pytest.mark.parametrize("precision", ["f64", "f64_fast"])
def test_rlz_kz64_parity(precision):
    # the configuration-4 column length (64 levels) in FP64 arithmetic
    gp = fields.rlz400_f32_params(precision=precision, num_cells=12, kDim=64, nvars=2)
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.rlz_blob_fields(pts, 2, zmax=20000.0)
    _, _, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp, tol=TOL64 if precision == "f64" else TOL_FAST)


def test_fp32_kz64_error_vs_fp64_oracle():
    gp = fields.rlz400_f32_params(precision="f32", num_cells=24, kDim=64, nvars=2)
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.rlz_blob_fields(pts, 2, zmax=20000.0)
    _, o, sg, so, pg, po = _run_both(gp, u)
    errs = slot_errors(pg, po, gp)
    print("FP32 kz=64 slot errors", errs)
    # binary32 bulk: f and the first derivatives ~1e-5, second derivatives ~1e-4
    assert np.all(errs < 5e-4), errs


def test_bad_shapes_rejected():
    with pytest.raises(S.SpringsteelError):
        S.createGrid(S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=1.0, num_cells=0))
    with pytest.raises(S.SpringsteelError) as e:  # a periodic spline needs 4 interior coefficients
        S.createGrid(S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=1.0, num_cells=3,
                                                 BCL={"default": S.PeriodicBC()}, BCR={"default": S.PeriodicBC()}))
    assert e.value.status == S.abi.SS_BAD_SHAPE


def _host_case(geometry, precision):
    if geometry == "RLZ":
        gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=60.0, num_cells=30, kMin=0.0,
                                         kMax=20000.0, kDim=16, vars={"u": 1, "w": 2},
                                         BCB={"default": S.DirichletBC()}, BCT={"default": S.NeumannBC()},
                                         precision=precision)
        pts = S.getGridpoints(S.createGrid(gp))
        return gp, fields.rlz_blob_fields(pts, 2, zmax=20000.0)
    gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=100.0, num_cells=50,
                                     vars={"u": 1, "w": 2}, precision=precision)
    pts = S.getGridpoints(S.createGrid(gp))
    u = np.stack([fields.blob_sum(pts, seed=7 + v, nblobs=4) for v in range(2)], axis=1)
    return gp, u


@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
@pytest.mark.parametrize("precision", ["f64", "f32"])
@pytest.mark.parametrize("host", ["numpy", "pinned", "converted"])
def test_host_overlapped_transforms_match(geometry, precision, host):
    """spectralTransform_from_host / gridTransform_to_host (radial chunks, copies on a
    second stream) give the same bits as upload → transforms → download."""
    import torch

    gp, u = _host_case(geometry, precision)
    native = np.float32 if precision == "f32" else np.float64
    hdt = (np.float64 if native == np.float32 else np.float32) if host == "converted" else native
    u = np.asfortranarray(u.astype(hdt))
    ref = S.createGrid(gp)
    ref.set_physical(u, slot=1)
    S.spectralTransform_b(ref)
    spec_ref = ref.get_spectral()
    S.gridTransform_b(ref)
    phys_ref = ref.get_physical(dtype=hdt)

    g = S.createGrid(gp)
    n, nv, ns = g.physical_shape
    if host == "pinned":
        tdt = torch.float32 if hdt == np.float32 else torch.float64
        h_in = torch.from_numpy(np.ascontiguousarray(u.T)).pin_memory()
        h_out = torch.empty((ns, nv, n), dtype=tdt).pin_memory()
        import ctypes as C
        lib = S.load_library()
        code = S.abi.SS_DTYPE_F32 if hdt == np.float32 else S.abi.SS_DTYPE_F64
        for _ in range(2):  # second round trip reuses the copy stream and events
            S._check(lib.ss_spectral_transform_from_host(g.handle, C.c_void_p(h_in.data_ptr()), code, None))
            spec = g.get_spectral()
            S._check(lib.ss_grid_transform_to_host(g.handle, C.c_void_p(h_out.data_ptr()), code, None))
        phys = np.asfortranarray(h_out.numpy().transpose(2, 1, 0))
    else:
        for _ in range(2):
            S.spectralTransform_from_host(g, u)
            spec = g.get_spectral()
            phys = S.gridTransform_to_host(g, dtype=hdt)
    assert np.array_equal(spec, spec_ref)
    assert np.array_equal(phys, phys_ref)


def test_rlz_unequal_max_wavenumber():
    """Variables with different max_wavenumber entries on RLZ: the shared rings take
    the last own entry in vars order (src/factory.jl:730-733) on both sides."""
    gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=40.0, num_cells=20, kMin=0.0,
                                     kMax=20000.0, kDim=16, vars={"w": 3, "u": 1, "v": 2},
                                     max_wavenumber={"default": 9, "w": 4, "u": 6},
                                     BCB={"default": S.DirichletBC()}, BCT={"default": S.NeumannBC()})
    assert gp.shared_ring_kmax() == 6
    pts = S.getGridpoints(S.createGrid(gp))
    u = fields.rlz_blob_fields(pts, 3, zmax=20000.0)
    _, o, sg, so, pg, po = _run_both(gp, u)
    _assert_parity(sg, so, pg, po, gp)


@pytest.mark.parametrize("precision", ["f64", "f64_fast", "f32"])
@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
def test_periodic_spline_bc_parity(geometry, precision):
    """PERIODIC radial splines (DenseSplineFactor, src/banded_cholesky.jl:70, 250-260):
    the wrap-around Γ fold and the dense factor's tail rows against the oracle's
    dense solve; a second variable keeps a banded BC in the same grid."""
    kw = dict(vars={"u": 1, "w": 2}, BCL={"u": S.PeriodicBC(), "w": S.DirichletBC()},
              BCR={"u": S.PeriodicBC(), "w": S.NaturalBC()}, precision=precision)
    if geometry == "RL":
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=30.0, num_cells=15, **kw)
    else:
        gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=24.0, num_cells=12, kMin=0.0, kMax=500.0,
                                         kDim=10, BCB={"default": S.DirichletBC()}, **kw)
    pts = S.getGridpoints(S.createGrid(gp))
    u = np.column_stack([fields.blob_sum(pts, seed=31 + v, nblobs=5, wmin=3.0, wmax=9.0,
                                         zmax=max(gp.kMax, 1.0)) for v in range(2)])
    if precision == "f32":
        u = u.astype(np.float32).astype(np.float64)
    g, o, spec_g, spec_o, phys_g, phys_o = _run_both(gp, u)
    if precision == "f32":
        errs = slot_errors(phys_g, phys_o, gp)
        assert np.all(errs.max(axis=0)[:5] <= [2e-6, 5e-5, 5e-5, 5e-5, 5e-5]), errs
    else:
        _assert_parity(spec_g, spec_o, phys_g, phys_o, gp, TOL64 if precision == "f64" else TOL_FAST)
