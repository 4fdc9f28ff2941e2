"""Host-side mirror of Springsteel.jl's RL/RLZ grid API over the GB300 C ABI.

The reference's Julia entry points map one to one:

=====================================  ==========================================
Springsteel.jl                         here
=====================================  ==========================================
``SpringsteelGridParameters(...)``     :class:`SpringsteelGridParameters`
``createGrid(gp)``                     :func:`createGrid` → :class:`SpringsteelGrid`
``spectralTransform!(grid)``           :func:`spectralTransform_b` (alias ``spectralTransform``)
``gridTransform!(grid)``               :func:`gridTransform_b` (alias ``gridTransform``)
the same on a host physical array      :func:`spectralTransform_from_host`, :func:`gridTransform_to_host`
``getGridpoints(grid)``                :func:`getGridpoints`
``NaturalBC()``, ``DirichletBC()``…    same names (src/Springsteel.jl:68-137)
``SpectralFilter``/``GaussianFilter``  same names (src/filtering.jl:31-127)
=====================================  ==========================================

``grid.physical`` and ``grid.spectral`` live in device memory; reading the
attributes downloads a host copy (``numpy`` arrays in the reference's
column-major shape), assigning them uploads.  The compute path is the CUDA
library only: if it cannot be loaded, calls raise instead of falling back.
"""
import ctypes as C
import math
import os

import numpy as np

from . import abi

_PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
_lib = None


class SpringsteelError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), msg))
        self.status = status


def load_library(build_if_missing=True):
    """Load libspringsteel_gpu.so (building it with nvcc when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    from . import build as _build

    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libspringsteel_gpu.so is missing; run springsteel_gpu.build.build()")
    _lib = abi.bind(C.CDLL(path))
    return _lib


def _check(st):
    if st != abi.SS_OK:
        raise SpringsteelError(st, load_library().ss_last_error_string().decode())


# ----------------------------------------------------------------- BCs
class BoundaryConditions:
    """src/Springsteel.jl:45-63: constraint slots u, du, d2u, robin; periodic."""

    def __init__(self, u=None, du=None, d2u=None, robin=None, periodic=False):
        if robin is not None and any(x is not None for x in (u, du, d2u)):
            raise ValueError("Robin BC is mutually exclusive with u/du/d2u constraint slots")
        if periodic and any(x is not None for x in (u, du, d2u, robin)):
            raise ValueError("PeriodicBC must have all other slots as nothing")
        self.u, self.du, self.d2u, self.robin, self.periodic = u, du, d2u, robin, periodic

    def __repr__(self):
        return "BoundaryConditions(u=%r, du=%r, d2u=%r, robin=%r, periodic=%r)" % (
            self.u, self.du, self.d2u, self.robin, self.periodic)


def NaturalBC():
    return BoundaryConditions()


def DirichletBC(v=0.0):
    return BoundaryConditions(u=float(v))


def NeumannBC(v=0.0):
    return BoundaryConditions(du=float(v))


def SecondDerivativeBC(v=0.0):
    return BoundaryConditions(d2u=float(v))


def RobinBC(alpha, beta, gamma=0.0):
    return BoundaryConditions(robin=(float(alpha), float(beta), float(gamma)))


def PeriodicBC():
    return BoundaryConditions(periodic=True)


def CauchyBC(u, du):
    return BoundaryConditions(u=float(u), du=float(du))


def ExponentialBC(lam):
    return RobinBC(1.0, -float(lam), 0.0)


def SymmetricBC():
    return NeumannBC(0.0)


def AntisymmetricBC():
    return BoundaryConditions(u=0.0, d2u=0.0)


def ZerosBC():
    return BoundaryConditions(u=0.0, du=0.0, d2u=0.0)


def FixedBC(u=None, du=0.0, d2u=0.0):
    if u is None:
        return BoundaryConditions(u=math.nan, du=math.nan, d2u=math.nan)
    return BoundaryConditions(u=float(u), du=float(du), d2u=float(d2u))


def bc_rank(bc):
    """src/Springsteel.jl:147-151."""
    if bc.periodic:
        return 0
    if bc.robin is not None:
        return 1
    return sum(x is not None for x in (bc.u, bc.du, bc.d2u))


def is_inhomogeneous(bc):
    if bc.robin is not None:
        return bc.robin[2] != 0.0
    return any(x is not None and x != 0.0 for x in (bc.u, bc.du, bc.d2u))


# legacy CubicBSpline BC dicts (src/CubicBSpline.jl:41-122) as (kind, α, β)
R0 = (abi.SS_SBC_R0, 0.0, 0.0)
R1T0 = (abi.SS_SBC_RANK1, -4.0, -1.0)
R1T1 = (abi.SS_SBC_RANK1, 0.0, 1.0)
R1T2 = (abi.SS_SBC_RANK1, 2.0, -1.0)
R2T10 = (abi.SS_SBC_RANK2, 1.0, -0.5)
R2T20 = (abi.SS_SBC_RANK2, -1.0, 0.0)
R3 = (abi.SS_SBC_R3, 0.0, 0.0)
R3X = (abi.SS_SBC_R3X, 0.0, 0.0)
PERIODIC = (abi.SS_SBC_PERIODIC, 0.0, 0.0)
# legacy Chebyshev BC dicts (src/Chebyshev.jl) as kinds
CHEB_R0 = abi.SS_CBC_R0
CHEB_R1T0 = abi.SS_CBC_R1T0
CHEB_R1T1 = abi.SS_CBC_R1T1


def _bc_to_spline(bc):
    """_bc_to_spline_dict, src/factory.jl:343-375."""
    if isinstance(bc, tuple):
        return bc
    if bc.periodic:
        return PERIODIC
    r = bc_rank(bc)
    if r == 0:
        return R0
    if r == 1:
        if bc.u is not None:
            return R1T0
        if bc.du is not None:
            return R1T1
        if bc.d2u is not None:
            return R1T2
        a, b, _ = bc.robin
        lam = -b / a
        return (abi.SS_SBC_RANK1, -4.0 / (3 * lam + 1), (3 * lam - 1) / (3 * lam + 1))
    if r == 2:
        if bc.u is not None and bc.du is not None:
            return R2T10
        if bc.u is not None and bc.d2u is not None:
            return R2T20
        raise ValueError("Unsupported rank-2 BC combination for CubicBSpline: du + d2u without u is not defined")
    return R3X if is_inhomogeneous(bc) or any(x is not None and math.isnan(x) for x in (bc.u, bc.du, bc.d2u)) else R3


def _bc_to_chebyshev(bc):
    """_bc_to_chebyshev_dict + _bc_type, src/factory.jl:378-396, src/Chebyshev.jl:949-963."""
    if isinstance(bc, int):
        return bc
    if bc.periodic:
        raise ValueError("PeriodicBC is not supported for Chebyshev basis")
    if bc.robin is not None:
        raise ValueError("RobinBC is not supported for Chebyshev basis")
    r = bc_rank(bc)
    if r == 0:
        return abi.SS_CBC_R0
    if r == 1:
        if bc.u is not None:
            return abi.SS_CBC_R1T0
        if bc.du is not None:
            return abi.SS_CBC_R1T1
        raise ValueError("Chebyshev BC R1T2 is not supported by calcGammaBC")
    raise ValueError("Rank-%d BCs are not yet implemented for Chebyshev basis" % r)


# ----------------------------------------------------------------- filters
class SpectralFilter:
    """src/filtering.jl:58-64."""

    def __init__(self, low_pass=-1, high_pass=0, notch=(), window="boxcar", taper_width=0):
        self.low_pass, self.high_pass = int(low_pass), int(high_pass)
        self.notch = [int(n) for n in notch]
        self.window, self.taper_width = window, int(taper_width)


class GaussianFilter:
    """src/filtering.jl:87-90."""

    def __init__(self, sigma, order=1):
        self.sigma, self.order = float(sigma), int(order)


def _window_weight(window, t):
    """src/filtering.jl:110-127."""
    t = min(max(t, 0.0), 1.0)
    if window == "boxcar":
        return 1.0 if t < 1.0 else 0.0
    if window == "hann":
        return 0.5 * (1.0 + math.cos(math.pi * t))
    if window == "lanczos":
        # t ≈ 0 with isapprox's default atol = 0 holds only for t == 0
        return 1.0 if t == 0.0 else math.sin(math.pi * t) / (math.pi * t)
    if window == "exponential":
        return math.exp(-t * t * 4.0)
    raise ValueError("Unknown window function: %s" % window)


def filter_weight(f, k):
    """_filter_weight, src/filtering.jl:145-194."""
    if isinstance(f, GaussianFilter):
        return math.exp(-(float(k) / f.sigma) ** (2 * f.order))
    if k in f.notch:
        return 0.0
    d = f.taper_width
    if f.high_pass > 0 and k < f.high_pass:
        if d > 0:
            dist = f.high_pass - k
            return 0.0 if dist > d else _window_weight(f.window, dist / d)
        return 0.0
    if f.low_pass >= 0 and k > f.low_pass:
        if d > 0:
            dist = k - f.low_pass
            return 0.0 if dist > d else _window_weight(f.window, dist / d)
        return 0.0
    return 1.0


def _snap(w):
    # the reference skips blocks with w ≈ 1 (isapprox, rtol = √eps) and zeroes w ≈ 0
    if abs(w - 1.0) <= 1.4901161193847656e-08 * max(abs(w), 1.0):
        return 1.0
    return w


# ----------------------------------------------------------------- params
def _per_var(d, key, default):
    if not isinstance(d, dict):
        return d
    if key in d:
        return d[key]
    return d.get("default", default)


class SpringsteelGridParameters:
    """src/Springsteel.jl:425-465 (RL / RLZ fields), plus ``precision``."""

    def __init__(self, geometry="RL", iMin=0.0, iMax=0.0, num_cells=0, mubar=3, quadrature="gauss",
                 l_q=None, BCL=None, BCR=None, kMin=0.0, kMax=0.0, kDim=0, b_kDim=None, BCB=None, BCT=None,
                 vars=None, max_wavenumber=None, fourier_filter=None, chebyshev_filter=None,
                 spectralIndexL=1, patchOffsetL=None, precision="f64", i_regular_out=None, j_regular_out=None,
                 k_regular_out=None, **derived):
        geom = {"RL": "RL", "Spline1D_Fourier": "RL", "RLZ": "RLZ"}.get(geometry, geometry)
        if geom not in ("RL", "RLZ"):
            raise ValueError("only RL and RLZ geometries run on the GPU path (got %r)" % geometry)
        self.geometry = geom
        self.iMin, self.iMax, self.num_cells, self.mubar = float(iMin), float(iMax), int(num_cells), int(mubar)
        self.quadrature = quadrature
        self.iDim = self.num_cells * self.mubar
        self.b_iDim = self.num_cells + 3
        self.l_q = l_q if l_q is not None else {"default": 2.0}
        self.BCL = BCL if BCL is not None else {"default": R0}
        self.BCR = BCR if BCR is not None else {"default": R0}
        self.kMin, self.kMax, self.kDim = float(kMin), float(kMax), int(kDim)
        self.b_kDim = (min(self.kDim, (2 * self.kDim - 1) // 3 + 1) if b_kDim is None else int(b_kDim))
        self.BCB = BCB if BCB is not None else {"default": CHEB_R0}
        self.BCT = BCT if BCT is not None else {"default": CHEB_R0}
        self.vars = vars if vars is not None else {"u": 1}
        self.max_wavenumber = max_wavenumber if max_wavenumber is not None else {"default": -1}
        self.fourier_filter = fourier_filter or {}
        self.chebyshev_filter = chebyshev_filter or {}
        self.spectralIndexL = int(spectralIndexL)
        self.patchOffsetL = (self.spectralIndexL - 1) * self.mubar if patchOffsetL is None else int(patchOffsetL)
        self.precision = precision
        # regular output sizes, src/Springsteel.jl:461-464 defaults
        self.i_regular_out = self.num_cells + 1 if i_regular_out is None else int(i_regular_out)
        self.j_regular_out = self.iDim * 2 + 1 if j_regular_out is None else int(j_regular_out)
        self.k_regular_out = self.kDim + 1 if k_regular_out is None else int(k_regular_out)

    def var_names(self):
        names = [None] * len(self.vars)
        for k, v in self.vars.items():
            names[v - 1] = k
        return names

    def shared_ring_kmax(self):
        """kmax cap of the RLZ rings, which every variable shares: the "default"
        entry, overridden by each variable's own entry in the order ``vars``
        iterates (src/factory.jl:730-733).  The reference's vars is a Julia Dict
        (hash order); here it is a Python dict (insertion order), and a Julia
        caller computes the same value with the same loop over its own Dict."""
        km = int(self.max_wavenumber.get("default", -1))
        for key in self.vars:
            if key in self.max_wavenumber:
                km = int(self.max_wavenumber[key])
        return km

    def to_abi(self):
        names = self.var_names()
        nv = len(names)
        quad = {"gauss": abi.SS_QUAD_GAUSS, "regular": abi.SS_QUAD_REGULAR}[self.quadrature]
        prec = {"f64": abi.SS_PREC_F64, "f32": abi.SS_PREC_F32_REFINED,
                "f32_refined": abi.SS_PREC_F32_REFINED, "f64_fast": abi.SS_PREC_F64_FAST}[self.precision]
        geom = abi.SS_GEOM_RL if self.geometry == "RL" else abi.SS_GEOM_RLZ
        kw = dict(
            mubar=self.mubar, quadrature=quad, precision=prec, patchOffsetL=self.patchOffsetL,
            l_q=[float(_per_var(self.l_q, n, 2.0)) for n in names],
            BCL=[_bc_to_spline(_per_var(self.BCL, n, R0)) for n in names],
            BCR=[_bc_to_spline(_per_var(self.BCR, n, R0)) for n in names],
            max_wavenumber=[int(_per_var(self.max_wavenumber, n, -1)) for n in names],
        )
        if self.geometry == "RLZ":
            kw["ring_kmax"] = self.shared_ring_kmax()
            kw.update(kDim=self.kDim, b_kDim=self.b_kDim, kMin=self.kMin, kMax=self.kMax,
                      BCB=[_bc_to_chebyshev(_per_var(self.BCB, n, CHEB_R0)) for n in names],
                      BCT=[_bc_to_chebyshev(_per_var(self.BCT, n, CHEB_R0)) for n in names])
        return abi.make_params(geom, self.num_cells, self.iMin, self.iMax, nv, **kw)


# ----------------------------------------------------------------- grid
_DTYPES = {np.dtype(np.float64): abi.SS_DTYPE_F64, np.dtype(np.float32): abi.SS_DTYPE_F32}


class SpringsteelGrid:
    """Device-resident RL/RLZ grid (the GPU counterpart of SpringsteelGrid, src/types.jl:249-256)."""

    def __init__(self, gp):
        self.params = gp
        self._bundle = gp.to_abi()
        lib = load_library()
        h = C.c_void_p()
        _check(lib.ss_grid_create(self._bundle.ref, C.byref(h)))
        self._h = h
        d = abi.ss_dims()
        _check(lib.ss_grid_dims(h, C.byref(d)))
        self.dims = d.as_dict()
        self.dtype = np.float32 if gp.precision in ("f32", "f32_refined") else np.float64
        self._apply_filters()

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            load_library().ss_grid_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    @property
    def physical_shape(self):
        d = self.dims
        return (d["n_physical"], d["nvars"], d["nslots"])

    @property
    def spectral_shape(self):
        return (self.dims["n_spectral"], self.dims["nvars"])

    def stream(self):
        s = C.c_void_p()
        _check(load_library().ss_grid_stream(self._h, C.byref(s)))
        return s.value

    # -- host copies
    def get_physical(self, slot=0, dtype=np.float64):
        n, nv, ns = self.physical_shape
        out = np.empty((n, nv, ns) if slot == 0 else (n, nv), dtype=dtype, order="F")
        _check(load_library().ss_download_physical(self._h, out.ctypes.data_as(C.c_void_p),
                                                   _DTYPES[np.dtype(dtype)], int(slot), None))
        return out

    def device_array(self, which, var, slot=1):
        """One variable's column of grid.physical (slot 1-based) or grid.spectral
        as a torch CUDA tensor viewing the grid's own device memory (no copy),
        for checks that must not download every variable of a large grid."""
        import torch

        d = self.dims
        n = d["n_physical"] if which == "physical" else d["n_spectral"]
        p = C.c_void_p()
        fn = load_library().ss_grid_device_physical if which == "physical" else load_library().ss_grid_device_spectral
        _check(fn(self._h, C.byref(p)))
        esz = 4 if self.params.precision == "f32" else 8
        plane = ((slot - 1) * d["nvars"] + var) if which == "physical" else var
        self.synchronize()

        class _View:
            __cuda_array_interface__ = {
                "shape": (n,), "typestr": "<f4" if esz == 4 else "<f8",
                "data": (p.value + plane * n * esz, False), "version": 3, "strides": None}

        return torch.as_tensor(_View(), device="cuda")

    def set_physical(self, arr, slot=1):
        n, nv, ns = self.physical_shape
        a = np.asfortranarray(arr)
        if a.dtype not in _DTYPES:
            a = a.astype(np.float64, order="F")
        want = (n, nv, ns) if slot == 0 else (n, nv)
        if a.ndim == 3 and slot != 0:
            a = np.asfortranarray(a[:, :, slot - 1])
        if a.shape != want and a.size == int(np.prod(want)):
            a = np.asfortranarray(a.reshape(want, order="F"))
        if a.shape != want:
            raise ValueError("physical shape %s, expected %s" % (a.shape, want))
        _check(load_library().ss_upload_physical(self._h, a.ctypes.data_as(C.c_void_p), _DTYPES[a.dtype],
                                                 int(slot), None))

    def get_spectral(self, dtype=np.float64):
        out = np.empty(self.spectral_shape, dtype=dtype, order="F")
        _check(load_library().ss_download_spectral(self._h, out.ctypes.data_as(C.c_void_p),
                                                   _DTYPES[np.dtype(dtype)], None))
        return out

    def set_spectral(self, arr):
        a = np.asfortranarray(arr)
        if a.dtype not in _DTYPES:
            a = a.astype(np.float64, order="F")
        if a.shape != self.spectral_shape:
            raise ValueError("spectral shape %s, expected %s" % (a.shape, self.spectral_shape))
        _check(load_library().ss_upload_spectral(self._h, a.ctypes.data_as(C.c_void_p), _DTYPES[a.dtype], None))

    physical = property(lambda self: self.get_physical(), lambda self, a: self.set_physical(a, 0))
    spectral = property(lambda self: self.get_spectral(), lambda self, a: self.set_spectral(a))

    # -- registry hooks
    def set_wavenumber_ahat(self, var, block, ahat):
        """_set_wavenumber_ahat! (src/multipatch_registry.jl:45-62); `block` is the spectral block index."""
        a = np.ascontiguousarray(ahat, dtype=np.float64)
        if a.size != self.dims["b_iDim"]:
            raise ValueError("ahat needs b_iDim entries")
        _check(load_library().ss_grid_set_ahat(self._h, int(var), int(block), a.ctypes.data_as(C.c_void_p)))

    def clear_wavenumber_ahat(self):
        _check(load_library().ss_grid_clear_ahat(self._h))

    def _apply_filters(self):
        gp = self.params
        if not gp.fourier_filter and not gp.chebyshev_filter:
            return
        K, bk = self.dims["kDim_wn"], self.dims["b_kDim"]
        for v, name in enumerate(gp.var_names()):
            ff = _per_var(gp.fourier_filter, name, None)
            cf_ = _per_var(gp.chebyshev_filter, name, None) if gp.geometry == "RLZ" else None
            fw = cw = None
            if ff is not None:
                fw = np.array([_snap(filter_weight(ff, k)) for k in range(K + 1)])
            if cf_ is not None:
                cw = np.array([_snap(filter_weight(cf_, z)) for z in range(bk)])
            if fw is None and cw is None:
                continue
            _check(load_library().ss_grid_set_filter(
                self._h, v, fw.ctypes.data_as(C.c_void_p) if fw is not None else None,
                cw.ctypes.data_as(C.c_void_p) if cw is not None else None))

    def synchronize(self):
        _check(load_library().ss_grid_synchronize(self._h))


def createGrid(gp):
    """createGrid (src/factory.jl:1104-1143) for RL / RLZ geometries."""
    return SpringsteelGrid(gp)


def spectralTransform_b(grid, stream=None):
    """spectralTransform!(grid): physical slot 1 → spectral, then applyFilter! (asynchronous)."""
    _check(load_library().ss_spectral_transform(grid.handle, stream))
    return grid


def gridTransform_b(grid, stream=None):
    """gridTransform!(grid): spectral → every physical derivative slot (asynchronous)."""
    _check(load_library().ss_grid_transform(grid.handle, stream))
    return grid


spectralTransform = spectralTransform_b
gridTransform = gridTransform_b


def spectralTransform_from_host(grid, physical, stream=None):
    """spectralTransform!(grid) reading physical slot 1 from a host array: an
    (n × nvars) array, or the whole (n × nvars × nslots) physical array of the
    reference's layout (column-major).  The upload of each radial chunk overlaps
    the transform of the previous one; returns once the array may be reused."""
    n, nv, ns = grid.physical_shape
    a = np.asarray(physical)
    if a.ndim == 3:
        a = a[:, :, 0]
    a = np.asfortranarray(a)
    if a.dtype not in _DTYPES:
        a = a.astype(np.float64, order="F")
    if a.shape != (n, nv):
        raise ValueError("physical slot 1 shape %s, expected %s" % (a.shape, (n, nv)))
    _check(load_library().ss_spectral_transform_from_host(grid.handle, a.ctypes.data_as(C.c_void_p),
                                                          _DTYPES[a.dtype], stream))
    return grid


def gridTransform_to_host(grid, out=None, dtype=np.float64, stream=None):
    """gridTransform!(grid) into a host array (n × nvars × nslots, column-major):
    the download of each radial chunk overlaps the transform of the next.
    Returns `out` (allocated when None)."""
    n, nv, ns = grid.physical_shape
    if out is None:
        out = np.empty((n, nv, ns), dtype=dtype, order="F")
    if out.shape != (n, nv, ns) or not out.flags.f_contiguous or out.dtype not in _DTYPES:
        raise ValueError("output must be a column-major %s float32/float64 array" % ((n, nv, ns),))
    _check(load_library().ss_grid_transform_to_host(grid.handle, out.ctypes.data_as(C.c_void_p),
                                                    _DTYPES[out.dtype], stream))
    return out


def getGridpoints(grid):
    """getGridpoints (src/transforms_cylindrical.jl:75-90, 454-476)."""
    gp = grid.params
    d = grid.dims
    nc, mb = gp.num_cells, gp.mubar
    DX = (gp.iMax - gp.iMin) / nc
    if gp.quadrature == "gauss":
        nodes = np.polynomial.legendre.leggauss(mb)[0] if mb != 3 else np.array([-math.sqrt(0.6), 0.0, math.sqrt(0.6)])
        q = (nodes + 1.0) / 2.0
    else:
        q = (2 * np.arange(1, mb + 1) - 1) / (2 * mb)
    rmish = np.array([gp.iMin + mc * DX + q[mu] * DX for mc in range(nc) for mu in range(mb)])
    pts = []
    kz = d["kDim"]
    if gp.geometry == "RLZ":
        N = gp.kDim
        scale, offset = -0.5 * (gp.kMax - gp.kMin), 0.5 * (gp.kMin + gp.kMax)
        zm = np.cos(np.arange(N) * math.pi / (N - 1)) * scale + offset
    for r in range(1, d["iDim"] + 1):
        ri = r + gp.patchOffsetL
        L = 4 + 4 * ri
        ymin = 0.5 * (2 * math.pi / L) * (ri - 1)
        lam = ymin + 2 * math.pi * np.arange(L) / L
        if gp.geometry == "RL":
            pts.append(np.column_stack([np.full(L, rmish[r - 1]), lam]))
        else:
            rr = np.full(L * kz, rmish[r - 1])
            ll = np.repeat(lam, kz)
            zz = np.tile(zm, L)
            pts.append(np.column_stack([rr, ll, zz]))
    return np.asfortranarray(np.vstack(pts))


# ----------------------------------------------------------------- batches
class Batch:
    """Many grids transformed together (optionally replayed as a CUDA graph).
    fused=True (default): the RL grids' stages run as a few launches over all
    grids (one launch per ring shared-memory class, one SB and one SA launch);
    fused=False: every grid's own launch sequence on forked streams.
    autotune=True times tile shapes (ring CTA size, items per ring CTA) on the
    grids' own data at creation."""

    def __init__(self, grids, autotune=False, fused=True):
        self.grids = list(grids)
        lib = load_library()
        arr = (C.c_void_p * len(self.grids))(*[g.handle for g in self.grids])
        h = C.c_void_p()
        flags = (abi.SS_BATCH_AUTOTUNE if autotune else 0) | (abi.SS_BATCH_FUSED if fused else 0)
        _check(lib.ss_batch_create(arr, len(self.grids), flags, C.byref(h)))
        self._h = h
        self.fused = fused

    def run(self, what=3, use_graph=True, stream=None):
        """what: 1 spectralTransform!, 2 gridTransform!, 3 both."""
        _check(load_library().ss_batch_run(self._h, int(what), 1 if use_graph else 0, stream))

    def synchronize(self):
        _check(load_library().ss_batch_synchronize(self._h))

    def fused_launches(self, what=3):
        """Kernel launches the fused batch enqueues for `what` (RL grids)."""
        n = C.c_int32()
        _check(load_library().ss_batch_fused_launches(self._h, int(what), C.byref(n)))
        return n.value

    def ring_threads(self, i):
        f, v = C.c_int32(), C.c_int32()
        _check(load_library().ss_batch_ring_threads(self._h, int(i), C.byref(f), C.byref(v)))
        return f.value, v.value

    def close(self):
        if getattr(self, "_h", None):
            load_library().ss_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ----------------------------------------------------------------- multipatch
class PatchChain:
    """PatchChain(grids) (src/multipatch.jl:825-848) on the device."""

    def __init__(self, grids):
        self.patches = list(grids)
        lib = load_library()
        arr = (C.c_void_p * len(self.patches))(*[g.handle for g in self.patches])
        h = C.c_void_p()
        _check(lib.ss_chain_create(arr, len(self.patches), C.byref(h)))
        self._h = h

    def multiGridTransform(self, stream=None):
        """multiGridTransform! (src/multipatch.jl:769-786)."""
        _check(load_library().ss_multi_grid_transform(self._h, stream))

    def close(self):
        if getattr(self, "_h", None):
            load_library().ss_chain_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PatchEmbedded(PatchChain):
    """PatchEmbedded(grids) (src/multipatch.jl:891-925) on the device: grids nested
    outermost first; each inner grid receives R3X data from its parent at both ends."""

    def __init__(self, grids):
        self.patches = list(grids)
        lib = load_library()
        arr = (C.c_void_p * len(self.patches))(*[g.handle for g in self.patches])
        h = C.c_void_p()
        _check(lib.ss_chain_create_embedded(arr, len(self.patches), C.byref(h)))
        self._h = h


def embedded_grid_params(domains, cells, vars=None, BCL=None, BCR=None, mubar=3, l_q=None, precision="f64",
                         geometry="RL", **column):
    """Per-grid parameters of an embedded multigrid (_create_embedded,
    src/multipatch.jl:1113-1190): domains outermost first, each contained in its
    parent and strictly finer; the outer grid keeps BCL/BCR, inner grids get
    FixedBC (R3X) at both ends; patch offsets from the domain starts."""
    n = len(domains)
    cells = [cells] * n if isinstance(cells, int) else list(cells)
    vars = vars or {"u": 1}
    for k in range(1, n):
        if not (domains[k][0] >= domains[k - 1][0] and domains[k][1] <= domains[k - 1][1]):
            raise ValueError("Domain %d %s not contained in domain %d %s" % (k + 1, domains[k], k, domains[k - 1]))
    dx = [(domains[k][1] - domains[k][0]) / cells[k] for k in range(n)]
    for k in range(1, n):
        if abs(dx[k - 1] / dx[k] - 1.0) < 1e-10 * max(dx[k - 1], dx[k]):
            raise ValueError("Embedded requires strict refinement. Domains %d and %d have same DX=%g" % (k, k + 1, dx[k]))
    offs = compute_patch_offsets([d[0] for d in domains] + [domains[-1][1]], cells, mubar)
    out = []
    for k in range(n):
        bl = (BCL or {"default": NaturalBC()}) if k == 0 else {"default": FixedBC()}
        br = (BCR or {"default": NaturalBC()}) if k == 0 else {"default": FixedBC()}
        out.append(SpringsteelGridParameters(geometry=geometry, iMin=domains[k][0], iMax=domains[k][1],
                                             num_cells=cells[k], mubar=mubar, vars=vars, BCL=bl, BCR=br, l_q=l_q,
                                             patchOffsetL=offs[k], precision=precision, **column))
    return out


def compute_patch_offsets(boundaries, cells, mubar=3):
    """_compute_patch_offsets (src/multipatch.jl:998-1014) for cylindrical grids."""
    offsets, cumulative = [], 0
    if boundaries[0] > 0:
        dx_first = (boundaries[1] - boundaries[0]) / cells[0]
        cumulative = int(round(boundaries[0] / dx_first)) * mubar
    for c in cells:
        offsets.append(cumulative)
        cumulative += c * mubar
    return offsets


def chain_grid_params(boundaries, cells, vars=None, BCL=None, BCR=None, mubar=3, l_q=None, precision="f64",
                      geometry="RL", **column):
    """Per-patch parameters of a chain (_create_chain, src/multipatch.jl:1018-1111):
    at each interface the finer side gets FixedBC (R3X), the coarser NaturalBC;
    patch offsets follow _compute_patch_offsets.  geometry="RLZ" chains take the
    shared column parameters (kMin, kMax, kDim, BCB, BCT) as keywords."""
    n = len(boundaries) - 1
    cells = [cells] * n if isinstance(cells, int) else list(cells)
    vars = vars or {"u": 1}
    dx = [(boundaries[k + 1] - boundaries[k]) / cells[k] for k in range(n)]
    for k in range(n - 1):
        ratio = max(dx[k], dx[k + 1]) / min(dx[k], dx[k + 1])
        tol = 1e-10 * max(dx[k], dx[k + 1])
        if not (abs(ratio - 1.0) < tol or abs(ratio - 2.0) < tol):
            raise ValueError("Adjacent DX ratio between patches %d and %d is %.4g:1, must be 1:1 or 2:1" %
                             (k + 1, k + 2, ratio))
    bl = [{"default": NaturalBC()} for _ in range(n)]
    br = [{"default": NaturalBC()} for _ in range(n)]
    for k in range(n - 1):
        if dx[k] >= dx[k + 1]:
            bl[k + 1] = {"default": FixedBC()}
        else:
            br[k] = {"default": FixedBC()}
    bl[0] = BCL or {"default": NaturalBC()}
    br[-1] = BCR or {"default": NaturalBC()}
    offs = compute_patch_offsets(boundaries, cells, mubar)
    return [SpringsteelGridParameters(geometry=geometry, iMin=boundaries[k], iMax=boundaries[k + 1],
                                      num_cells=cells[k], mubar=mubar, vars=vars, BCL=bl[k], BCR=br[k], l_q=l_q,
                                      patchOffsetL=offs[k], precision=precision, **column) for k in range(n)]


# ----------------------------------------------------------------- tiles
def calcTileSizes(gp, num_tiles):
    """calcTileSizes for cylindrical grids (src/tiling.jl:185-259): tile parameters
    balanced by ring points, at least 3 cells per tile."""
    if gp.num_cells / num_tiles < 3.0:
        raise ValueError("Too many tiles for this grid (need at least 3 cells per tile)")
    DX = (gp.iMax - gp.iMin) / gp.num_cells
    iMins, iMaxs = [0.0] * num_tiles, [0.0] * num_tiles
    nc, siL = [0] * num_tiles, [1] * num_tiles
    if num_tiles == 1:
        iMins[0], iMaxs[0], nc[0] = gp.iMin, gp.iMax, gp.num_cells
    else:
        lpoints = [4 + 4 * (r + gp.patchOffsetL) for r in range(1, gp.iDim + 1)]
        jDim = sum(lpoints)
        q, r_rem = divmod(jDim, num_tiles)
        targets = [q + 1 if i < r_rem else q for i in range(num_tiles)]
        target = 1.0
        nc = [0] * num_tiles
        while any(c < 3 for c in nc) and target > 0.1:
            t = num_tiles - 1
            cell_count = 0
            target -= 0.1
            tile_count = [0] * num_tiles
            nc = [0] * num_tiles
            tile_min = int(target * targets[0])
            for ri in range(gp.iDim, 0, -1):
                tile_count[t] += lpoints[ri - 1]
                if ri % 3 == 0:
                    cell_count += 1
                    if cell_count >= 3 and tile_count[t] >= tile_min:
                        nc[t] = cell_count
                        cell_count = 0
                        t -= 1
                if t < 0:
                    break
            nc[0] = gp.num_cells - sum(nc[1:])
        if any(c < 3 for c in nc):
            raise ValueError("Too many tiles for this grid (need at least 3 cells per tile)")
        iMins[0] = gp.iMin
        iMaxs[0] = nc[0] * DX + iMins[0]
        for i in range(1, num_tiles - 1):
            iMins[i] = iMaxs[i - 1]
            iMaxs[i] = nc[i] * DX + iMins[i]
            siL[i] = nc[i - 1] + siL[i - 1]
        iMins[-1] = iMaxs[-2]
        iMaxs[-1] = gp.iMax
        siL[-1] = nc[-2] + siL[-2]
        nc[-1] = gp.num_cells - sum(nc[:-1])
    tiles = []
    for i in range(num_tiles):
        kw = dict(gp.__dict__)
        for k in ("iDim", "b_iDim", "patchOffsetL"):
            kw.pop(k, None)
        kw.update(iMin=iMins[i], iMax=iMaxs[i], num_cells=nc[i], spectralIndexL=siL[i])
        tiles.append(SpringsteelGridParameters(**kw))
    return tiles


def sumSpectralTile_b(patch, tile, stream=None):
    """sumSpectralTile!(patch, tile) (src/tiling.jl:1048-1136) on the device."""
    _check(load_library().ss_tile_sum_spectral(patch.handle, tile.handle, 0, stream))


def setSpectralTile_b(patch, tile, stream=None):
    """setSpectralTile!: zero the patch spectral, then write the tile's blocks."""
    _check(load_library().ss_grid_zero_spectral(patch.handle, stream))
    _check(load_library().ss_tile_sum_spectral(patch.handle, tile.handle, 1, stream))


def tile_physical_from_patch(patch, tile, slot=1, stream=None):
    _check(load_library().ss_tile_copy_physical(patch.handle, tile.handle, int(slot), 0, stream))


def tile_physical_to_patch(patch, tile, slot=0, stream=None):
    _check(load_library().ss_tile_copy_physical(patch.handle, tile.handle, int(slot), 1, stream))


def splineTransform_b(shared, tile, stream=None):
    """splineTransform!(sharedSpectral, tile) (src/tiling.jl:1490-1516 RL, 1862-1892 RLZ):
    SAtransform(spline, b) of every wavenumber (and Chebyshev-mode) block of
    `shared` — a grid whose device spectral array holds B-vectors in the tile's
    spectral layout and precision, or None for the tile's own spectral array —
    written as spline coefficients a into the tile's spectral array.  As in the
    reference, the two-argument SAtransform adds no R3X background."""
    lib = load_library()
    ptr = None
    if shared is not None:
        if shared.spectral_shape != tile.spectral_shape or \
                (shared.params.precision == "f32") != (tile.params.precision == "f32"):
            raise ValueError("shared spectral array must match the tile's spectral shape and storage type")
        p = C.c_void_p()
        _check(lib.ss_grid_device_spectral(shared.handle, C.byref(p)))
        shared.synchronize()
        ptr = p
    _check(lib.ss_spline_transform(tile.handle, ptr, stream))


def tileTransform_b(shared, tile, stream=None):
    """tileTransform!(sharedSpectral, tile, physical, spectral) (src/tiling.jl:1540-1660 RL,
    1915-2046 RLZ): the tile's spectral array holds spline coefficients a (from
    splineTransform_b); every physical slot is evaluated from them — SI / SIx /
    SIxx, the ring inverse with ∂λ, ∂λλ and, for RLZ, the Chebyshev inverse with
    ∂z, ∂zz — gridTransform! without its SAtransform!.  `shared` is unused, as in
    the reference (kept for the same call shape)."""
    _check(load_library().ss_tile_transform(tile.handle, stream))


def zero_spectral(grid, stream=None):
    _check(load_library().ss_grid_zero_spectral(grid.handle, stream))


# ----------------------------------------------------------------- elliptic solve
from .solver import MLPPreconditioner, SpringsteelProblem, solve  # noqa: E402


# ----------------------------------------------------------------- regular-grid output
def _lin_range(a, b, n):
    """Julia's LinRange(a, b, n) points, (1 − t)·a + t·b with t = j/(n − 1)."""
    if n == 1:
        return np.array([float(a)])
    t = np.arange(n, dtype=np.float64) / float(n - 1)
    return (1.0 - t) * a + t * b


def regular_axes(gp):
    """(r, λ, z) axes of getRegularGridpoints (src/transforms_cylindrical.jl:878-898,
    1117-1138): i_regular_out radii on [iMin, iMax], j_regular_out angles 2π(j−1)/n_λ,
    k_regular_out levels on [kMin, kMax] (RLZ; None for RL)."""
    r = _lin_range(gp.iMin, gp.iMax, gp.i_regular_out)
    n_l = gp.j_regular_out
    lam = np.array([2 * math.pi * j / n_l for j in range(n_l)])
    z = _lin_range(gp.kMin, gp.kMax, gp.k_regular_out) if gp.geometry == "RLZ" else None
    return r, lam, z


def getRegularGridpoints(grid_or_params):
    """getRegularGridpoints: (n_r·n_λ[·n_z], 2|3) points, r outer, λ (then z) inner."""
    gp = getattr(grid_or_params, "params", grid_or_params)
    r, lam, z = regular_axes(gp)
    axes = (r, lam) if z is None else (r, lam, z)
    mesh = np.meshgrid(*axes, indexing="ij")
    return np.column_stack([m.reshape(-1) for m in mesh])


def regularGridTransform(grid, *points, stream=None):
    """regularGridTransform(grid, r_pts, λ_pts[, z_pts]) or regularGridTransform(grid,
    gridpoints) (src/transforms_cylindrical.jl:929-1020 RL, 1168-1287 RLZ) from the
    device-resident spectral array: returns (n_r·n_λ[·n_z], nvars, 5|7) FP64, slots
    f, ∂r, ∂rr, ∂λ, ∂λλ (, ∂z, ∂zz).  A single points matrix is split as the
    reference does: sorted unique r (and z); λ the first n_λ rows (RL) or sorted
    unique (RLZ)."""
    gp = grid.params
    if len(points) == 1:
        pts = np.asarray(points[0], np.float64)
        r = np.unique(pts[:, 0])
        if gp.geometry == "RL":
            lam = pts[: pts.shape[0] // len(r), 1]
            z = None
        else:
            lam, z = np.unique(pts[:, 1]), np.unique(pts[:, 2])
    else:
        r, lam = np.asarray(points[0], np.float64), np.asarray(points[1], np.float64)
        z = np.asarray(points[2], np.float64) if len(points) > 2 else None
    if (gp.geometry == "RLZ") != (z is not None):
        raise ValueError("RLZ grids take r, λ and z points; RL grids r and λ")
    nz = 1 if z is None else len(z)
    d = grid.dims
    out = np.empty((len(r) * len(lam) * nz, d["nvars"], d["nslots"]), order="F")
    rp, lp = np.ascontiguousarray(r), np.ascontiguousarray(lam)
    zp = np.ascontiguousarray(z) if z is not None else None
    _check(load_library().ss_regular_grid_transform(
        grid.handle, rp.ctypes.data_as(C.c_void_p), len(r), lp.ctypes.data_as(C.c_void_p), len(lam),
        zp.ctypes.data_as(C.c_void_p) if zp is not None else None, nz, out.ctypes.data_as(C.c_void_p), stream))
    return out


# ----------------------------------------------------------------- I/O (src/io.jl)
from .io import (check_grid_dims, load_grid, read_netcdf, read_physical_grid, save_grid,  # noqa: E402,F401
                 write_grid, write_netcdf)


# ----------------------------------------------------------------- unstructured points, relocation
def evaluate_unstructured(source, pts, vars=None, out_of_bounds="nan", stream=None):
    """evaluate_unstructured(source, pts; vars, out_of_bounds) (src/interpolation.jl:1735-1850)
    from the device-resident spectral array: pts (N, 2) (r, λ) for RL or (N, 3)
    (r, λ, z) for RLZ; returns (N, nvars) values, NaN for variables not in `vars`.
    out_of_bounds: "nan", "error" (raises), or a number to fill."""
    p = np.asfortranarray(np.asarray(pts, np.float64))
    d = source.dims
    if p.ndim != 2 or p.shape[1] != (3 if source.params.geometry == "RLZ" else 2):
        raise ValueError("pts must be (N, 2) for RL and (N, 3) for RLZ grids")
    mode, fill = (0, 0.0) if out_of_bounds == "nan" else ((1, 0.0) if out_of_bounds == "error"
                                                          else (2, float(out_of_bounds)))
    out = np.empty((p.shape[0], d["nvars"]), order="F")
    st = load_library().ss_evaluate_unstructured(source.handle, p.ctypes.data_as(C.c_void_p), p.shape[0],
                                                 out.ctypes.data_as(C.c_void_p), mode, fill, stream)
    if st == abi.SS_BAD_ARG and mode == 1:
        raise ValueError(load_library().ss_last_error_string().decode())
    _check(st)
    if vars is not None:
        keep = {source.params.vars[v] - 1 for v in vars if v in source.params.vars}
        for j in range(d["nvars"]):
            if j not in keep:
                out[:, j] = np.nan
    return out


_BOUNDARY = {"nan": 0, "nearest": 1, "azimuthal_mean": 2}


def grid_center(grid):
    """grid_center (src/relocation.jl:25-27): cumulative shift of relocate_grid_b calls
    (kept on the grid object)."""
    return getattr(grid, "_center", (0.0, 0.0))


def _relocate(target, source, new_center, boundary, taper_width, stream):
    if boundary not in _BOUNDARY:
        raise ValueError("Unknown boundary strategy: %s. Fast path supports nan, nearest, azimuthal_mean." % boundary)
    dx, dy = float(new_center[0]), float(new_center[1])
    _check(load_library().ss_relocate_grid(target.handle, source.handle, dx, dy, _BOUNDARY[boundary],
                                           int(taper_width), stream))


def relocate_grid(grid, new_center, boundary="azimuthal_mean", taper_width=0, stream=None):
    """relocate_grid(grid, (dx, dy); boundary, taper_width) (src/relocation.jl:56-98): a new
    grid whose fields are the source's reprojected to the shifted center."""
    new = createGrid(grid.params)
    grid.synchronize()
    _relocate(new, grid, new_center, boundary, taper_width, stream)
    return new


def relocate_grid_b(grid, new_center, boundary="azimuthal_mean", taper_width=0, stream=None):
    """relocate_grid!(grid, (dx, dy); ...) (src/relocation.jl:99-128): in place, and the
    grid's cumulative center moves by (dx, dy)."""
    _relocate(grid, grid, new_center, boundary, taper_width, stream)
    old = grid_center(grid)
    grid._center = (old[0] + float(new_center[0]), old[1] + float(new_center[1]))
    return grid
