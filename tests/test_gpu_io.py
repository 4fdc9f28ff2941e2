"""Grid I/O on the GPU (src/io.jl): save_grid / load_grid archives streamed from
and to the device arrays, write_grid CSV files, read_physical_grid, and the
NetCDF regular-grid output."""
import ctypes as C
import os

import numpy as np
import pytest

import springsteel_gpu as S
from springsteel_gpu import fields
from test_gpu_multi import _fill

pytestmark = pytest.mark.gpu


def _grid(geometry, precision, filtered=False):
    kw = dict(vars={"u": 1, "w": 2}, BCL={"u": S.DirichletBC()}, BCR={"w": S.NeumannBC()}, precision=precision)
    if filtered:
        kw["fourier_filter"] = {"u": S.SpectralFilter(low_pass=10, window="hann", taper_width=3)}
    if geometry == "RL":
        gp = S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=40.0, num_cells=20, **kw)
    else:
        gp = S.SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=30.0, num_cells=12, kMin=0.0,
                                         kMax=1000.0, kDim=10, BCB={"default": S.DirichletBC()}, **kw)
    g = S.createGrid(gp)
    _fill(g, seed=5)
    S.spectralTransform_b(g)
    S.gridTransform_b(g)
    return g


@pytest.mark.parametrize("geometry,precision", [("RL", "f64"), ("RLZ", "f32"), ("RLZ", "f64_fast")])
def test_save_load_roundtrip(tmp_path, geometry, precision):
    g = _grid(geometry, precision, filtered=True)
    path = str(tmp_path / "grid.ssg")
    S.save_grid(path, g)
    g2 = S.load_grid(path)
    assert g2.params.precision == precision and g2.dims == g.dims
    s0 = g.get_spectral()
    assert np.array_equal(g2.get_spectral(g.dtype), g.get_spectral(g.dtype))
    assert np.array_equal(g2.get_physical(0, g.dtype), g.get_physical(0, g.dtype))
    # the filter travels with the parameters: the same forward transform on both
    S.spectralTransform_b(g)
    S.spectralTransform_b(g2)
    assert np.array_equal(g2.get_spectral(g.dtype), g.get_spectral(g.dtype))
    # the C entry point rebuilds the grid from the parameter record alone
    lib = S.load_library()
    h = C.c_void_p()
    S._check(lib.ss_grid_load(os.fsencode(path), C.byref(h), None))
    n = g.dims["n_spectral"] * g.dims["nvars"]
    out = np.empty(n, dtype=np.float64)
    S._check(lib.ss_download_spectral(h, out.ctypes.data_as(C.c_void_p), S.abi.SS_DTYPE_F64, None))
    lib.ss_grid_destroy(h)
    assert np.array_equal(out.reshape(s0.shape, order="F"), s0)
    saved = np.fromfile(path, dtype=np.uint8)
    assert saved[:8].tobytes() == b"SSGRID01"
    g.close()
    g2.close()


def test_load_rejects_other_shapes(tmp_path):
    g = _grid("RL", "f64")
    path = str(tmp_path / "g.ssg")
    S.save_grid(path, g)
    other = S.createGrid(S.SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=40.0, num_cells=21,
                                                     vars={"u": 1, "w": 2}))
    with pytest.raises(S.SpringsteelError) as e:
        S._check(S.load_library().ss_grid_load_arrays(other.handle, os.fsencode(path), None))
    assert e.value.status == S.abi.SS_BAD_SHAPE
    bad = str(tmp_path / "bad.ssg")
    with open(bad, "wb") as f:
        f.write(b"NOTAGRID" + b"\0" * 64)
    with pytest.raises(S.SpringsteelError):
        S.load_grid(bad)


@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
def test_write_grid_csv_and_read_back(tmp_path, geometry):
    g = _grid(geometry, "f64")
    S.write_grid(g, str(tmp_path), "t")
    phys = g.get_physical()
    spec = g.get_spectral()
    d = np.loadtxt(tmp_path / "t_physical.csv", delimiter=",", skiprows=1)
    nc = 2 if geometry == "RL" else 3
    assert np.array_equal(d[:, :nc], S.getGridpoints(g))
    nv, ns = phys.shape[1], phys.shape[2]
    for s in range(ns):
        for v in range(nv):
            assert np.array_equal(d[:, nc + s * nv + v], phys[:, v, s])
    ds = np.loadtxt(tmp_path / "t_spectral.csv", delimiter=",", skiprows=1)
    assert np.array_equal(ds[:, 1:], spec)
    if geometry == "RL":
        dg = np.loadtxt(tmp_path / "t_gridded.csv", delimiter=",", skiprows=1)
        reg = S.regularGridTransform(g, S.getRegularGridpoints(g))
        assert np.array_equal(dg[:, 2], reg[:, 0, 0])
    # read_physical_grid: one column per variable into slot 1
    csv = tmp_path / "in.csv"
    np.savetxt(csv, phys[:, :, 0], delimiter=",", header="u,w", comments="", fmt="%.17g")
    g2 = S.createGrid(g.params)
    S.read_physical_grid(str(csv), g2)
    assert np.array_equal(g2.get_physical(1), phys[:, :, 0])
    g.close()


@pytest.mark.parametrize("geometry", ["RL", "RLZ"])
def test_netcdf_regular_output(tmp_path, geometry):
    g = _grid(geometry, "f64")
    path = str(tmp_path / "out.nc")
    S.write_netcdf(path, g, include_derivatives=True, global_attributes={"institution": "test"}, time=3600.0)
    data = S.read_netcdf(path)
    assert data["attributes"]["Conventions"] == "CF-1.12"
    assert data["attributes"]["institution"] == "test"
    r, lam, z = S.regular_axes(g.params)
    assert np.allclose(data["coordinates"]["radius"], r)
    assert np.allclose(data["coordinates"]["azimuth"], np.degrees(lam))
    reg = S.regularGridTransform(g, r, lam) if z is None else S.regularGridTransform(g, r, lam, z)
    shape = (len(r), len(lam)) if z is None else (len(r), len(lam), len(z))
    sfx = ["", "_r", "_rr", "_az", "_azaz", "_z", "_zz"]
    for v, name in enumerate(["u", "w"]):
        for s in range(reg.shape[2]):
            got = data["variables"][name + sfx[s]]
            assert got.shape == (1,) + shape
            assert np.array_equal(got[0], reg[:, v, s].reshape(shape))
    g.close()
