"""Grid I/O for RL / RLZ grids (src/io.jl), reading back from the device arrays.

  save_grid / load_grid      params + spectral + physical archive (src/io.jl:410-439);
                             the arrays stream between HBM and the file in the
                             library (ss_grid_save / ss_grid_load_arrays)
  write_grid                 CSV files of spectral, physical and the regular grid
                             (src/io.jl:142-216 RL, 274-336 RLZ)
  read_physical_grid         CSV → physical slot 1 (src/io.jl:338-368)
  write_netcdf / read_netcdf CF NetCDF of the regular-grid output (src/io.jl:730-851,
                             979-1078, 1115-1154), NetCDF-3 64-bit-offset files
                             through scipy.io (the reference writes NetCDF-4 through
                             NCDatasets; this image has no netCDF-4/HDF5 library)
"""
import ctypes as C
import json
import os
import time as _time

import numpy as np

from . import (SpectralFilter, GaussianFilter, SpringsteelGridParameters, _check, createGrid, getGridpoints,
               getRegularGridpoints, load_library, regular_axes, regularGridTransform)

ARCHIVE_FORMAT = "1.0"  # the reference's format_version tag


def _vars_sorted(gp):
    """_io_vars_sorted (src/io.jl:41): (name, index) by index."""
    return sorted(gp.vars.items(), key=lambda kv: kv[1])


def _enc_filter(f):
    if f is None:
        return None
    return {"type": type(f).__name__, **f.__dict__}


def _dec_filter(d):
    if d is None:
        return None
    d = dict(d)
    kind = d.pop("type")
    cls = {"SpectralFilter": SpectralFilter, "GaussianFilter": GaussianFilter}[kind]
    obj = cls.__new__(cls)
    obj.__dict__.update(d)
    return obj


def _params_json(gp):
    from . import CHEB_R0, R0, _bc_to_chebyshev, _bc_to_spline, _per_var

    names = gp.var_names()
    out = dict(geometry=gp.geometry, iMin=gp.iMin, iMax=gp.iMax, num_cells=gp.num_cells, mubar=gp.mubar,
               quadrature=gp.quadrature, kMin=gp.kMin, kMax=gp.kMax, kDim=gp.kDim, b_kDim=gp.b_kDim,
               vars=dict(gp.vars), spectralIndexL=gp.spectralIndexL, patchOffsetL=gp.patchOffsetL,
               precision=gp.precision, i_regular_out=gp.i_regular_out, j_regular_out=gp.j_regular_out,
               k_regular_out=gp.k_regular_out,
               l_q={n: float(_per_var(gp.l_q, n, 2.0)) for n in names},
               BCL={n: list(_bc_to_spline(_per_var(gp.BCL, n, R0))) for n in names},
               BCR={n: list(_bc_to_spline(_per_var(gp.BCR, n, R0))) for n in names},
               max_wavenumber={k: int(v) for k, v in gp.max_wavenumber.items()},
               fourier_filter={k: _enc_filter(v) for k, v in gp.fourier_filter.items()},
               chebyshev_filter={k: _enc_filter(v) for k, v in gp.chebyshev_filter.items()})
    if gp.geometry == "RLZ":
        out["BCB"] = {n: int(_bc_to_chebyshev(_per_var(gp.BCB, n, CHEB_R0))) for n in names}
        out["BCT"] = {n: int(_bc_to_chebyshev(_per_var(gp.BCT, n, CHEB_R0))) for n in names}
    return out


def _params_from_json(d):
    d = dict(d)
    for key in ("BCL", "BCR"):
        d[key] = {n: tuple(v) for n, v in d.get(key, {}).items()}
    d["fourier_filter"] = {k: _dec_filter(v) for k, v in d.get("fourier_filter", {}).items()}
    d["chebyshev_filter"] = {k: _dec_filter(v) for k, v in d.get("chebyshev_filter", {}).items()}
    return SpringsteelGridParameters(**d)


def save_grid(filename, grid, stream=None):
    """save_grid(filename, grid) (src/io.jl:410-418): format_version, params,
    spectral and physical, the arrays read back from the device by the library.
    The host mirror's parameters ride in the archive's caller block as JSON."""
    blob = json.dumps({"format_version": ARCHIVE_FORMAT, "params": _params_json(grid.params)}).encode()
    _check(load_library().ss_grid_save(grid.handle, os.fsencode(filename), blob, len(blob), stream))


def load_grid(filename, stream=None):
    """load_grid(filename) (src/io.jl:431-439): createGrid(params), then the
    archived spectral and physical arrays copied into the fresh grid's device
    memory."""
    lib = load_library()
    n = C.c_int64()
    _check(lib.ss_grid_archive_user(os.fsencode(filename), None, 0, C.byref(n)))
    if n.value <= 0:
        raise ValueError("%s carries no host parameter block; load it with ss_grid_load" % filename)
    buf = C.create_string_buffer(n.value)
    _check(lib.ss_grid_archive_user(os.fsencode(filename), buf, n.value, C.byref(n)))
    meta = json.loads(buf.raw[: n.value].decode())
    grid = createGrid(_params_from_json(meta["params"]))
    _check(lib.ss_grid_load_arrays(grid.handle, os.fsencode(filename), stream))
    return grid


def _slot_suffixes(gp):
    return ["", "_r", "_rr", "_l", "_ll"] + (["_z", "_zz"] if gp.geometry == "RLZ" else [])


def _write_csv(path, header, cols):
    data = np.column_stack(cols)
    with open(path, "w") as f:
        f.write(",".join(header) + "\n")
        np.savetxt(f, data, delimiter=",", fmt="%.17g")


def write_grid(grid, output_dir, tag):
    """write_grid(grid, output_dir, tag) (src/io.jl:142-216 RL, 274-336 RLZ):
    `tag`_spectral.csv (idx, one column per variable), `tag`_physical.csv
    (r, l[, z], then every derivative slot of every variable) and, for RL,
    `tag`_gridded.csv on the regular output grid."""
    gp = grid.params
    print("Writing %s to %s" % (tag, output_dir))
    vs = _vars_sorted(gp)
    sfx = _slot_suffixes(gp)
    spec = grid.get_spectral()
    _write_csv(os.path.join(output_dir, "%s_spectral.csv" % tag), ["idx"] + [v for v, _ in vs],
               [np.arange(1, spec.shape[0] + 1)] + [spec[:, i - 1] for _, i in vs])
    pts = getGridpoints(grid)
    phys = grid.get_physical()
    coords = ["r", "l"] + (["z"] if gp.geometry == "RLZ" else [])
    header = coords + [v + sfx[d] for d in range(len(sfx)) for v, _ in vs]
    _write_csv(os.path.join(output_dir, "%s_physical.csv" % tag), header,
               [pts[:, c] for c in range(len(coords))] + [phys[:, i - 1, d] for d in range(len(sfx)) for _, i in vs])
    if gp.geometry == "RL":
        rp = getRegularGridpoints(grid)
        reg = regularGridTransform(grid, rp, stream=None)
        _write_csv(os.path.join(output_dir, "%s_gridded.csv" % tag), header,
                   [rp[:, 0], rp[:, 1]] + [reg[:, i - 1, d] for d in range(len(sfx)) for _, i in vs])


def check_grid_dims(nrows, grid):
    """check_grid_dims (src/io.jl:29-35): the row count must equal size(grid.physical, 1)."""
    expected = grid.dims["n_physical"]
    if expected != nrows:
        raise ValueError("Grid size does not match: expected %d rows, got %d" % (expected, nrows))


def read_physical_grid(file, grid):
    """read_physical_grid(file, grid) (src/io.jl:338-368): one CSV column per
    variable (named by the variable key), one row per physical gridpoint, into
    physical slot 1 of the device grid."""
    with open(file) as f:
        header = f.readline().strip().split(",")
    data = np.loadtxt(file, delimiter=",", skiprows=1, ndmin=2)
    check_grid_dims(data.shape[0], grid)
    gp = grid.params
    for key in gp.vars:
        if key not in header:
            raise ValueError("Grid is missing variable %s" % key)
    u = np.zeros((data.shape[0], len(gp.vars)), order="F")
    for key, v in gp.vars.items():
        u[:, v - 1] = data[:, header.index(key)]
    grid.set_physical(u, slot=1)


# NetCDF coordinate names, units and long names of cylindrical grids
# (_netcdf_coord_info, src/io.jl:637-639) and derivative suffixes (:647)
_COORDS = {"i": ("radius", "1", "radial distance"), "j": ("azimuth", "degrees", "azimuth angle"),
           "k": ("height", "1", "height")}
_NC_SFX = ["", "_r", "_rr", "_az", "_azaz", "_z", "_zz"]


def write_netcdf(filename, grid, include_derivatives=False, global_attributes=None, coordinate_attributes=None,
                 variable_attributes=None, time=None, grid_mapping=None):
    """write_netcdf(filename, grid; include_derivatives, global_attributes, ...)
    (src/io.jl:730-851 RL, 979-1078 RLZ): the regular-grid output of
    regularGridTransform with CF-1.12 attributes — dimensions radius, azimuth
    (degrees, 360(j−1)/n_λ) [, height], one variable per field and, with
    include_derivatives, _r, _rr, _az, _azaz [, _z, _zz] slots; an optional
    leading time dimension and grid_mapping variable."""
    from scipy.io import netcdf_file

    gp = grid.params
    r, lam, z = regular_axes(gp)
    reg = regularGridTransform(grid, r, lam) if z is None else regularGridTransform(grid, r, lam, z)
    n_i, n_j = len(r), len(lam)
    n_k = 1 if z is None else len(z)
    nslots = (5 if z is None else 7) if include_derivatives else 1
    coordinate_attributes = coordinate_attributes or {}
    variable_attributes = variable_attributes or {}
    f = netcdf_file(filename, "w", version=2)
    try:
        f.Conventions = "CF-1.12"
        f.title = "Springsteel.jl regular grid output"
        f.source = "Springsteel.jl"
        f.history = "Created " + _time.strftime("%Y-%m-%d %H:%M:%S")
        for k, v in (global_attributes or {}).items():
            setattr(f, k, v)
        has_time = time is not None
        if has_time:
            f.createDimension("time", 1)
            tv = f.createVariable("time", "d", ("time",))
            tv.units, tv.calendar, tv.long_name = "seconds since 1970-01-01T00:00:00Z", "gregorian", "time"
            tv[:] = [float(time)]
        axes = [("i", np.asarray(r)), ("j", np.array([360.0 * j / n_j for j in range(n_j)]))]
        if z is not None:
            axes.append(("k", np.asarray(z)))
        for key, vals in axes:
            name, units, long_name = _COORDS[key]
            f.createDimension(name, len(vals))
            cv = f.createVariable(name, "d", (name,))
            cv.units, cv.long_name = units, long_name
            for ak, av in coordinate_attributes.get(name, {}).items():
                setattr(cv, ak, av)
            cv[:] = vals
        if grid_mapping is not None:
            gm = f.createVariable(grid_mapping.get("variable_name", "grid_mapping"), "i", ())
            for k, v in grid_mapping.items():
                if k != "variable_name":
                    setattr(gm, k, v)
            gm.assignValue(0)
        dims = tuple(_COORDS[k][0] for k, _ in axes)
        if has_time:
            dims = ("time",) + dims
        shape = (n_i, n_j) if z is None else (n_i, n_j, n_k)
        for name, vi in _vars_sorted(gp):
            for s in range(nslots):
                full = name + _NC_SFX[s]
                vv = f.createVariable(full, "d", dims)
                vv.long_name = full
                vv._FillValue = np.nan
                for ak, av in variable_attributes.get(full, {}).items():
                    setattr(vv, ak, av)
                data = reg[:, vi - 1, s].reshape(shape)  # r outer, λ (then z) inner
                vv[:] = data[None] if has_time else data
    finally:
        f.close()


def read_netcdf(filename):
    """read_netcdf(filename) (src/io.jl:1115-1154): {"dimensions", "coordinates",
    "variables", "attributes"} of a NetCDF file."""
    from scipy.io import netcdf_file

    out = {"dimensions": {}, "coordinates": {}, "variables": {}, "attributes": {}}
    f = netcdf_file(filename, "r", mmap=False)
    try:
        for name, n in f.dimensions.items():
            out["dimensions"][name] = n
        for name, var in f.variables.items():
            arr = np.array(var[:], dtype=np.float64, copy=True)
            if name in f.dimensions:
                out["coordinates"][name] = arr
            else:
                out["variables"][name] = arr
        for k, v in f._attributes.items():
            out["attributes"][k] = v.decode() if isinstance(v, bytes) else v
    finally:
        f.close()
    return out
