"""ctypes wrapper of the FP64 CPU oracle (test infrastructure only).

The oracle restates Springsteel.jl's RL/RLZ transform path in C (see
``ss_oracle.c`` for the file:line of each restated function).  Only the test
suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it.
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
_PKG = os.path.join(ROOT, "springsteel.jl_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)

from springsteel_gpu import abi  # noqa: E402

sys.path.insert(0, HERE)
import build as _oracle_build  # noqa: E402

sys.path.remove(HERE)

_lib = None
_dp = C.POINTER(C.c_double)


def lib():
    global _lib
    if _lib is None:
        path = _oracle_build.build()
        L = C.CDLL(path)
        vp, i32, d = C.c_void_p, C.c_int32, C.c_double
        sig = {
            "or_last_error": ([], C.c_char_p),
            "or_set_threads": ([C.c_int], None),
            "or_grid_create": ([C.POINTER(abi.ss_grid_params), C.POINTER(vp)], i32),
            "or_grid_destroy": ([vp], None),
            "or_grid_dims": ([vp, C.POINTER(abi.ss_dims)], i32),
            "or_spectral_transform": ([vp, vp, vp], i32),
            "or_grid_transform": ([vp, vp, vp], i32),
            "or_grid_set_ahat": ([vp, i32, i32, vp], i32),
            "or_grid_set_filter": ([vp, i32, vp, vp], i32),
            "or_grid_points": ([vp, vp], i32),
            "or_grid_radial_points": ([vp, vp], i32),
            "or_grid_ring_points": ([vp, i32, vp], i32),
            "or_grid_column_points": ([vp, vp], i32),
            "or_grid_factor": ([vp, i32, vp, C.POINTER(i32)], i32),
            "or_grid_spline_transform": ([vp, vp, vp], i32),
            "or_grid_transform_coeffs": ([vp, vp, vp], i32),
            "or_spline_create": ([d, d, i32, i32, i32, d, C.POINTER(abi.ss_spline_bc),
                                  C.POINTER(abi.ss_spline_bc), C.POINTER(vp)], i32),
            "or_spline_destroy": ([vp], None),
            "or_spline_info": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], i32),
            "or_basis": ([vp, i32, d, i32], d),
            "or_spline_mish": ([vp, vp], i32),
            "or_spline_sb": ([vp, vp, vp], i32),
            "or_spline_sa": ([vp, vp, vp, vp], i32),
            "or_spline_si": ([vp, vp, i32, vp], i32),
            "or_spline_si_points": ([vp, vp, vp, i32, i32, vp], i32),
            "or_spline_gamma_dense": ([vp, vp], i32),
            "or_spline_pq_dense": ([vp, vp], i32),
            "or_spline_set_ahat_r3x": ([vp, d, d, d, i32, vp], i32),
            "or_band_chol": ([vp, i32, vp], i32),
            "or_band_solve": ([vp, i32, vp, vp], i32),
            "or_r2hc": ([vp, i32, vp], i32),
            "or_hc2r": ([vp, i32, vp], i32),
            "or_fourier_fb": ([i32, i32, i32, d, vp, vp], i32),
            "or_fourier_fa": ([i32, i32, i32, d, vp, vp], i32),
            "or_fourier_fi": ([i32, i32, vp, i32, vp], i32),
            "or_redft00": ([vp, i32, vp], i32),
            "or_cheb_cb": ([i32, i32, vp, vp], i32),
            "or_cheb_gamma": ([i32, i32, i32, vp, C.POINTER(i32)], i32),
            "or_cheb_ca": ([i32, i32, i32, i32, vp, vp], i32),
            "or_cheb_ci": ([i32, d, d, vp, i32, vp], i32),
            "or_cheb_mish": ([i32, d, d, vp], i32),
        }
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


class OracleError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (abi.STATUS_NAMES.get(status, status), msg))
        self.status = status


def _check(st):
    if st != 0:
        raise OracleError(st, lib().or_last_error().decode())


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def set_threads(n):
    lib().or_set_threads(int(n))


class OracleGrid:
    """FP64 CPU grid with the reference's physical/spectral layouts."""

    def __init__(self, bundle):
        self._bundle = bundle
        h = C.c_void_p()
        _check(lib().or_grid_create(bundle.ref, C.byref(h)))
        self.h = h
        d = abi.ss_dims()
        _check(lib().or_grid_dims(h, C.byref(d)))
        self.dims = d.as_dict()

    def close(self):
        if self.h:
            lib().or_grid_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def physical_shape(self):
        d = self.dims
        return (d["n_physical"], d["nvars"], d["nslots"])

    @property
    def spectral_shape(self):
        d = self.dims
        return (d["n_spectral"], d["nvars"])

    def spectral_transform(self, physical):
        """physical: array (n_physical, nvars[, nslots]) in column-major meaning
        (numpy order='F'); only slot 1 is read.  Returns spectral (n_spectral, nvars)."""
        ph = np.asfortranarray(physical, dtype=np.float64)
        spec = np.zeros(self.spectral_shape, dtype=np.float64, order="F")
        _check(lib().or_spectral_transform(self.h, _ptr(ph), _ptr(spec)))
        return spec

    def grid_transform(self, spectral):
        sp = np.asfortranarray(spectral, dtype=np.float64)
        ph = np.zeros(self.physical_shape, dtype=np.float64, order="F")
        _check(lib().or_grid_transform(self.h, _ptr(sp), _ptr(ph)))
        return ph

    def spline_transform(self, shared):
        """splineTransform!(sharedSpectral, tile) (src/tiling.jl:1490-1516, 1862-1892):
        spline coefficients a of every block of `shared` (the grid's spectral layout)."""
        sp = np.asfortranarray(shared, dtype=np.float64)
        a = np.zeros(self.spectral_shape, dtype=np.float64, order="F")
        _check(lib().or_grid_spline_transform(self.h, _ptr(sp), _ptr(a)))
        return a

    def tile_transform(self, acoef):
        """tileTransform!(sharedSpectral, tile, physical, spectral) (src/tiling.jl:1540-1660,
        1915-2046): every physical slot from spline coefficients a (no SAtransform!)."""
        a = np.asfortranarray(acoef, dtype=np.float64)
        ph = np.zeros(self.physical_shape, dtype=np.float64, order="F")
        _check(lib().or_grid_transform_coeffs(self.h, _ptr(a), _ptr(ph)))
        return ph

    def set_ahat(self, var, block, ahat):
        a = _f64(ahat)
        _check(lib().or_grid_set_ahat(self.h, int(var), int(block), _ptr(a)))

    def set_filter(self, var, fourier_w=None, chebyshev_w=None):
        fw = _f64(fourier_w) if fourier_w is not None else None
        cw = _f64(chebyshev_w) if chebyshev_w is not None else None
        _check(lib().or_grid_set_filter(self.h, int(var), _ptr(fw) if fw is not None else None,
                                        _ptr(cw) if cw is not None else None))

    def gridpoints(self):
        ncol = 3 if self.dims["b_kDim"] > 1 or self.dims["kDim"] > 1 else 2
        out = np.zeros((self.dims["n_physical"], ncol), order="F")
        _check(lib().or_grid_points(self.h, _ptr(out)))
        return out

    def radial_points(self):
        out = np.zeros(self.dims["iDim"])
        _check(lib().or_grid_radial_points(self.h, _ptr(out)))
        return out

    def ring_points(self, r):
        out = np.zeros(4 + 4 * (r + self._bundle.params.patchOffsetL))
        _check(lib().or_grid_ring_points(self.h, int(r), _ptr(out)))
        return out

    def column_points(self):
        out = np.zeros(self.dims["kDim"])
        _check(lib().or_grid_column_points(self.h, _ptr(out)))
        return out

    def factor(self, var=0):
        n = C.c_int32()
        out = np.zeros(4 * (self.dims["b_iDim"]))
        _check(lib().or_grid_factor(self.h, int(var), _ptr(out), C.byref(n)))
        return out[: 4 * n.value].reshape(n.value, 4)


class OracleSpline:
    """1-D cubic B-spline (Spline1D) for the basis KATs."""

    def __init__(self, xmin, xmax, num_cells, mubar=3, quadrature=0, l_q=2.0,
                 bcl=(0, 0.0, 0.0), bcr=(0, 0.0, 0.0)):
        L, R = abi.ss_spline_bc(), abi.ss_spline_bc()
        L.kind, L.alpha, L.beta = bcl
        R.kind, R.alpha, R.beta = bcr
        h = C.c_void_p()
        _check(lib().or_spline_create(xmin, xmax, num_cells, mubar, quadrature, l_q,
                                      C.byref(L), C.byref(R), C.byref(h)))
        self.h = h
        b, m, n = C.c_int32(), C.c_int32(), C.c_int32()
        lib().or_spline_info(h, C.byref(b), C.byref(m), C.byref(n))
        self.bDim, self.mishDim, self.Minterior = b.value, m.value, n.value

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_spline_destroy(self.h)
            self.h = None

    def basis(self, m, x, d=0):
        return lib().or_basis(self.h, int(m), float(x), int(d))

    def mish(self):
        x = np.zeros(self.mishDim)
        lib().or_spline_mish(self.h, _ptr(x))
        return x

    def sb(self, u):
        u = _f64(u)
        b = np.zeros(self.bDim)
        _check(lib().or_spline_sb(self.h, _ptr(u), _ptr(b)))
        return b

    def sa(self, b, ahat=None):
        b = _f64(b)
        a = np.zeros(self.bDim)
        ah = _f64(ahat) if ahat is not None else None
        _check(lib().or_spline_sa(self.h, _ptr(b), _ptr(ah) if ah is not None else None, _ptr(a)))
        return a

    def si(self, a, d=0, points=None):
        a = _f64(a)
        if points is None:
            u = np.zeros(self.mishDim)
            _check(lib().or_spline_si(self.h, _ptr(a), int(d), _ptr(u)))
        else:
            p = _f64(points)
            u = np.zeros(len(p))
            _check(lib().or_spline_si_points(self.h, _ptr(a), _ptr(p), len(p), int(d), _ptr(u)))
        return u

    def gamma(self):
        G = np.zeros((self.Minterior, self.bDim), order="F")
        lib().or_spline_gamma_dense(self.h, _ptr(G))
        return G

    def pq(self):
        P = np.zeros((self.bDim, self.bDim), order="F")
        lib().or_spline_pq_dense(self.h, _ptr(P))
        return P

    def ahat_r3x(self, u0, u1, u2, side, ahat=None):
        ah = np.zeros(self.bDim) if ahat is None else _f64(ahat).copy()
        lib().or_spline_set_ahat_r3x(self.h, u0, u1, u2, 0 if side == "left" else 1, _ptr(ah))
        return ah


def band_chol(A):
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    L4 = np.zeros(4 * n)
    _check(lib().or_band_chol(_ptr(A), n, _ptr(L4)))
    return L4


def band_solve(L4, b):
    b = _f64(b)
    x = np.zeros_like(b)
    _check(lib().or_band_solve(_ptr(_f64(L4)), len(b), _ptr(b), _ptr(x)))
    return x


def r2hc(x):
    x = _f64(x)
    out = np.zeros_like(x)
    _check(lib().or_r2hc(_ptr(x), len(x), _ptr(out)))
    return out


def hc2r(x):
    x = _f64(x)
    out = np.zeros_like(x)
    _check(lib().or_hc2r(_ptr(x), len(x), _ptr(out)))
    return out


def redft00(x):
    x = _f64(x)
    out = np.zeros_like(x)
    _check(lib().or_redft00(_ptr(x), len(x), _ptr(out)))
    return out


def fourier_fb(u, kmax, bDim, ymin):
    u = _f64(u)
    b = np.zeros(bDim)
    _check(lib().or_fourier_fb(len(u), kmax, bDim, ymin, _ptr(u), _ptr(b)))
    return b


def fourier_fa(b, yDim, kmax, ymin):
    b = _f64(b)
    a = np.zeros(yDim)
    _check(lib().or_fourier_fa(yDim, kmax, len(b), ymin, _ptr(b), _ptr(a)))
    return a


def fourier_fi(a, kmax, d=0):
    a = _f64(a)
    u = np.zeros_like(a)
    _check(lib().or_fourier_fi(len(a), kmax, _ptr(a), int(d), _ptr(u)))
    return u


def cheb_cb(u, bDim):
    u = _f64(u)
    b = np.zeros(bDim)
    _check(lib().or_cheb_cb(len(u), bDim, _ptr(u), _ptr(b)))
    return b


def cheb_gamma(zDim, bcb, bct):
    G = np.zeros(zDim * zDim)
    ism = C.c_int32()
    _check(lib().or_cheb_gamma(zDim, bcb, bct, _ptr(G), C.byref(ism)))
    return G.reshape(zDim, zDim, order="F") if ism.value else G[:zDim].copy()


def cheb_ca(b, zDim, bcb=0, bct=0):
    b = _f64(b)
    a = np.zeros(zDim)
    _check(lib().or_cheb_ca(zDim, len(b), bcb, bct, _ptr(b), _ptr(a)))
    return a


def cheb_ci(a, zmin, zmax, d=0):
    a = _f64(a)
    u = np.zeros_like(a)
    _check(lib().or_cheb_ci(len(a), zmin, zmax, _ptr(a), int(d), _ptr(u)))
    return u


def cheb_mish(zDim, zmin, zmax):
    z = np.zeros(zDim)
    _check(lib().or_cheb_mish(zDim, zmin, zmax, _ptr(z)))
    return z


class OracleChain:
    """PatchChain + multiGridTransform! on the oracle (src/multipatch.jl)."""

    def __init__(self, grids, embedded=False):
        """embedded=True: PatchEmbedded (src/multipatch.jl:891-925), grids outermost first."""
        L = lib()
        for fn in (L.or_chain_create, L.or_chain_create_embedded):
            fn.argtypes = [C.c_void_p, C.c_int32, C.POINTER(C.c_void_p)]
            fn.restype = C.c_int32
        L.or_chain_destroy.argtypes = [C.c_void_p]
        L.or_chain_destroy.restype = None
        L.or_multi_grid_transform.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.or_multi_grid_transform.restype = C.c_int32
        self.grids = list(grids)
        arr = (C.c_void_p * len(self.grids))(*[g.h.value for g in self.grids])
        h = C.c_void_p()
        _check((L.or_chain_create_embedded if embedded else L.or_chain_create)(arr, len(self.grids), C.byref(h)))
        self.h = h

    def multi_grid_transform(self, spectrals):
        sp = [np.asfortranarray(s, dtype=np.float64) for s in spectrals]
        ph = [np.zeros(g.physical_shape, order="F") for g in self.grids]
        sarr = (C.c_void_p * len(sp))(*[s.ctypes.data for s in sp])
        parr = (C.c_void_p * len(ph))(*[p.ctypes.data for p in ph])
        _check(lib().or_multi_grid_transform(self.h, sarr, parr))
        return ph

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_chain_destroy(self.h)
            self.h = None


class OracleElliptic:
    """Per-wavenumber elliptic solve on an RL oracle grid (see ss_oracle.c)."""

    def __init__(self, grid, k2):
        L = lib()
        for name, args in (("or_elliptic_create", [C.c_void_p, C.c_void_p, C.POINTER(C.c_void_p)]),
                           ("or_elliptic_operator", [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_int32)]),
                           ("or_elliptic_solve_spectral", [C.c_void_p, C.c_void_p]),
                           ("or_grid_transform_coeffs", [C.c_void_p, C.c_void_p, C.c_void_p])):
            getattr(L, name).argtypes = args
            getattr(L, name).restype = C.c_int32
        L.or_elliptic_destroy.argtypes = [C.c_void_p]
        L.or_elliptic_destroy.restype = None
        self.grid = grid
        self._k2 = _f64(k2)
        h = C.c_void_p()
        _check(L.or_elliptic_create(grid.h.value, _ptr(self._k2), C.byref(h)))
        self.h = h

    def operator(self, m):
        b = self.grid.dims["b_iDim"]
        G = np.zeros(b * b)
        n = C.c_int32()
        _check(lib().or_elliptic_operator(self.h, int(m), _ptr(G), C.byref(n)))
        return G[: n.value * n.value].reshape(n.value, n.value, order="F")

    def solve(self, f_phys):
        """f at the gridpoints (n_physical, nvars) → physical (n_physical, nvars, 5) of u."""
        g = self.grid
        ph = np.zeros(g.physical_shape, order="F")
        ph[:, :, 0] = np.asarray(f_phys).reshape(ph.shape[0], -1)
        spec = np.asfortranarray(g.spectral_transform(ph))
        _check(lib().or_elliptic_solve_spectral(self.h, _ptr(spec)))
        out = np.zeros(g.physical_shape, order="F")
        _check(lib().or_grid_transform_coeffs(g.h, _ptr(spec), _ptr(out)))
        return out, spec

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_elliptic_destroy(self.h)
            self.h = None


# ---------------------------------------------------------------- regular-grid output
def _bc_tuple(arr, v):
    if not arr:
        return (0, 0.0, 0.0)
    return (int(arr[v].kind), float(arr[v].alpha), float(arr[v].beta))


def _grid_splines(p):
    """One Spline1D per variable, the grid's radial template (src/factory.jl:667-680)."""
    out = []
    for v in range(p.nvars):
        lq = float(p.l_q[v]) if p.l_q else 2.0
        out.append(OracleSpline(p.iMin, p.iMax, p.num_cells, p.mubar, p.quadrature, lq,
                                _bc_tuple(p.BCL, v), _bc_tuple(p.BCR, v)))
    return out


def _fourier_sums(sv, lam, kdim):
    """Σ over wavenumbers at arbitrary λ of coefficient rows sv[..., 2K+1]
    (slot 0: k = 0, 2k−1: cos k, 2k: sin k) with the R2HC half-amplitude factor 2
    (src/transforms_cylindrical.jl:978-1005): returns f, ∂λ f, ∂λλ f."""
    k = np.arange(1, kdim + 1, dtype=np.float64)
    ang = np.outer(lam, k)  # k·λ
    c, s = np.cos(ang), np.sin(ang)
    rc, rs = sv[..., 1::2], sv[..., 2::2]
    f = sv[..., :1] + 2.0 * (rc @ c.T + rs @ s.T)
    fl = 2.0 * ((-rc * k) @ s.T + (rs * k) @ c.T)
    fll = -2.0 * ((rc * k * k) @ c.T + (rs * k * k) @ s.T)
    return f, fl, fll


def _cheb_point_matrices(N, zmin, zmax, z):
    """Value, ∂z and ∂zz of the DCT-I series at arbitrary z as matrices acting on the
    Chebyshev A-coefficients (_cheb_eval_pts!, _cheb_dz_pts!, _cheb_dzz_pts!,
    src/transforms_cylindrical.jl:1030-1094), clamps included."""
    scale, offset = -0.5 * (zmax - zmin), 0.5 * (zmin + zmax)
    m = np.arange(N, dtype=np.float64)
    xi0 = np.clip((z - offset) / scale, -1.0 + 1e-14, 1.0 - 1e-14)
    t0 = np.arccos(xi0)
    E = 2.0 * np.cos(np.outer(t0, m))
    E[:, 0] = 1.0
    E[:, N - 1] = np.cos((N - 1) * t0)
    xi = np.clip((z - offset) / scale, -1.0 + 1e-10, 1.0 - 1e-10)
    t = np.arccos(xi)
    st, ct = np.sin(t), np.cos(t)
    D1 = -2.0 * m * np.sin(np.outer(t, m))          # df/dt coefficients
    D1[:, 0] = 0.0
    D1[:, N - 1] = -(N - 1) * np.sin((N - 1) * t)
    D2 = -2.0 * m * m * np.cos(np.outer(t, m))      # d²f/dt² coefficients
    D2[:, 0] = 0.0
    D2[:, N - 1] = -(N - 1) ** 2 * np.cos((N - 1) * t)
    Dz = D1 / (-scale * st)[:, None]
    Dzz = (D2 * st[:, None] - D1 * ct[:, None]) / (scale ** 2 * st ** 3)[:, None]
    return E, Dz, Dzz


def regular_grid_transform(params, spectral, r_pts, lam_pts, z_pts=None):
    """regularGridTransform (src/transforms_cylindrical.jl:929-1020 RL, 1168-1287 RLZ):
    per wavenumber (and Chebyshev mode) SAtransform! of the spectral block, SI / SIx /
    SIxx at r_pts, the Fourier series at lam_pts, and for RLZ CAtransform! plus the
    Chebyshev series at z_pts.  Rows: r outer, λ (then z) inner; slots f, ∂r, ∂rr,
    ∂λ, ∂λλ (, ∂z, ∂zz).  `params` is an abi.ParamBundle."""
    p = params.params
    r = np.asarray(r_pts, np.float64)
    lam = np.asarray(lam_pts, np.float64)
    nc, mubar = p.num_cells, p.mubar
    b = nc + 3
    kdim = nc * mubar + p.patchOffsetL
    nslot = 1 + 2 * kdim
    splines = _grid_splines(p)
    spec = np.asarray(spectral, np.float64)
    if p.geometry == abi.SS_GEOM_RL:
        out = np.zeros((len(r) * len(lam), p.nvars, 5))
        for v, sp in enumerate(splines):
            sv = np.zeros((3, len(r), nslot))
            for q in range(nslot):  # blocks: k0, then cos k / sin k at 2k−1, 2k
                a = sp.sa(spec[q * b:(q + 1) * b, v])
                for d in range(3):
                    sv[d, :, q] = sp.si(a, d, r)
            f, fl, fll = _fourier_sums(sv[0], lam, kdim)
            fr = _fourier_sums(sv[1], lam, kdim)[0]
            frr = _fourier_sums(sv[2], lam, kdim)[0]
            for s, arr in enumerate((f, fr, frr, fl, fll)):
                out[:, v, s] = arr.reshape(-1)
        return out
    z = np.asarray(z_pts, np.float64)
    N = p.kDim
    bk = p.b_kDim if p.b_kDim > 0 else min(N, (2 * N - 1) // 3 + 1)
    out = np.zeros((len(r) * len(lam) * len(z), p.nvars, 7))
    E, Dz, Dzz = _cheb_point_matrices(N, p.kMin, p.kMax, z)
    for v, sp in enumerate(splines):
        bcb = int(p.BCB[v]) if p.BCB else 0
        bct = int(p.BCT[v]) if p.BCT else 0
        CA = np.column_stack([cheb_ca(np.eye(bk)[i], N, bcb, bct) for i in range(bk)])  # N × bk
        sv = np.zeros((3, len(r), bk, nslot))
        for zb in range(bk):
            base = zb * b * nslot
            for q in range(nslot):
                a = sp.sa(spec[base + q * b:base + (q + 1) * b, v])
                for d in range(3):
                    sv[d, :, zb, q] = sp.si(a, d, r)
        f, fl, fll = _fourier_sums(sv[0], lam, kdim)       # (n_r, bk, n_λ)
        fr = _fourier_sums(sv[1], lam, kdim)[0]
        frr = _fourier_sums(sv[2], lam, kdim)[0]
        for slot, arr, mats in ((0, f, (E, Dz, Dzz)), (1, fr, (E,)), (2, frr, (E,)), (3, fl, (E,)), (4, fll, (E,))):
            coef = np.einsum("nk,rkl->rln", CA, arr)         # CAtransform! per (r, λ) column
            for i, M in enumerate(mats):
                s = slot if i == 0 else 4 + i
                out[:, v, s] = np.einsum("zn,rln->rlz", M, coef).reshape(-1)
    return out


# ---------------------------------------------------------------- unstructured points, relocation
def _cheb_value_rows(N, zmin, zmax, z):
    """_cheb_eval_single (src/interpolation.jl:1271-1285): weights of the A-coefficients
    for the value at z, ξ clamped to [−1, 1]."""
    scale, offset = -0.5 * (zmax - zmin), 0.5 * (zmin + zmax)
    t = np.arccos(np.clip((np.asarray(z, np.float64) - offset) / scale, -1.0, 1.0))
    E = 2.0 * np.cos(np.outer(t, np.arange(N, dtype=np.float64)))
    E[:, 0] = 1.0
    E[:, N - 1] = np.cos((N - 1) * t)
    return E


def _point_values(p, sp, spec_v, r, lam, mean_only=None):
    """Per Chebyshev mode, the Fourier series of the SI values at each point's own
    (r, λ) (src/interpolation.jl:1628-1656, 1670-1702): (n_pts, bk) values; rows
    flagged in mean_only keep the k = 0 term."""
    nc, mubar = p.num_cells, p.mubar
    b = nc + 3
    kdim = nc * mubar + p.patchOffsetL
    nslot = 1 + 2 * kdim
    bk = 1 if p.geometry == abi.SS_GEOM_RL else (p.b_kDim if p.b_kDim > 0 else min(p.kDim, (2 * p.kDim - 1) // 3 + 1))
    k = np.arange(1, kdim + 1, dtype=np.float64)
    c, s = np.cos(np.outer(lam, k)), np.sin(np.outer(lam, k))
    out = np.zeros((len(r), bk))
    for zb in range(bk):
        sv = np.zeros((len(r), nslot))
        for q in range(nslot):
            a = sp.sa(spec_v[(zb * nslot + q) * b:(zb * nslot + q + 1) * b])
            sv[:, q] = sp.si(a, 0, r)
        full = sv[:, 0] + 2.0 * np.sum(sv[:, 1::2] * c + sv[:, 2::2] * s, axis=1)
        out[:, zb] = np.where(mean_only, sv[:, 0], full) if mean_only is not None else full
    return out


def evaluate_unstructured(params, spectral, pts, out_of_bounds="nan"):
    """evaluate_unstructured (src/interpolation.jl:1735-1850) for RL / RLZ grids: (N, nvars)."""
    p = params.params
    pts = np.asarray(pts, np.float64)
    spec = np.asarray(spectral, np.float64)
    mask = (pts[:, 0] >= p.iMin) & (pts[:, 0] <= p.iMax)
    if p.geometry == abi.SS_GEOM_RLZ:
        mask &= (pts[:, 2] >= p.kMin) & (pts[:, 2] <= p.kMax)
    if out_of_bounds == "error" and not mask.all():
        raise ValueError("%d points are outside the source domain" % int((~mask).sum()))
    out = np.full((pts.shape[0], p.nvars), np.nan)
    ib = np.nonzero(mask)[0]
    for v, sp in enumerate(_grid_splines(p)):
        if len(ib):
            f = _point_values(p, sp, spec[:, v], pts[ib, 0], pts[ib, 1])
            if p.geometry == abi.SS_GEOM_RL:
                out[ib, v] = f[:, 0]
            else:
                N = p.kDim
                bk = f.shape[1]
                CA = np.column_stack([cheb_ca(np.eye(bk)[i], N, int(p.BCB[v]) if p.BCB else 0,
                                              int(p.BCT[v]) if p.BCT else 0) for i in range(bk)])
                A = f @ CA.T  # (n, N) A-coefficients per point
                out[ib, v] = np.sum(_cheb_value_rows(N, p.kMin, p.kMax, pts[ib, 2]) * A, axis=1)
        if out_of_bounds not in ("nan", "error"):
            out[~mask, v] = float(out_of_bounds)
    return out


def relocated_slot1(params, spectral, gridpoints, dx, dy, boundary="azimuthal_mean", taper_width=0):
    """Physical slot 1 of the relocated grid before its transforms (_relocate_rl_fast! /
    _relocate_rlz_fast!, src/relocation.jl:144-439): each gridpoint takes the source's
    value at (r cos λ + dx, r sin λ + dy); out-of-range radii per `boundary`
    ("nan", "nearest", "azimuthal_mean"), cosine taper toward the mean over the last
    `taper_width` cells."""
    p = params.params
    spec = np.asarray(spectral, np.float64)
    gp = np.asarray(gridpoints, np.float64)
    rlz = p.geometry == abi.SS_GEOM_RLZ
    kz = p.kDim if rlz else 1
    ring = gp[::kz]  # one row per ring point
    xo = ring[:, 0] * np.cos(ring[:, 1]) + dx
    yo = ring[:, 0] * np.sin(ring[:, 1]) + dy
    ro = np.hypot(xo, yo)
    lo = np.arctan2(yo, xo)
    oob = (ro > p.iMax) | (ro < p.iMin)
    rs = np.where(oob, np.clip(ro, p.iMin + 1e-10, p.iMax - 1e-10), ro)
    DX = (p.iMax - p.iMin) / p.num_cells
    start = p.iMax - taper_width * DX if taper_width > 0 else p.iMax
    w = np.ones(len(rs))
    tap = (~oob) & (taper_width > 0) & (rs > start)
    w[tap] = 0.5 * (1.0 + np.cos(np.pi * (rs[tap] - start) / (p.iMax - start)))
    out = np.zeros((gp.shape[0], p.nvars))
    for v, sp in enumerate(_grid_splines(p)):
        full = _point_values(p, sp, spec[:, v], rs, lo, mean_only=oob & (boundary == "azimuthal_mean"))
        mean = _point_values(p, sp, spec[:, v], rs, lo, mean_only=np.ones(len(rs), bool))
        if not rlz:
            val = w * full[:, 0] + (1.0 - w) * mean[:, 0]
            val[oob] = full[oob, 0]
            if boundary == "nan":
                val[oob] = np.nan
            out[:, v] = val
            continue
        N, bk = p.kDim, full.shape[1]
        CA = np.column_stack([cheb_ca(np.eye(bk)[i], N, int(p.BCB[v]) if p.BCB else 0,
                                      int(p.BCT[v]) if p.BCT else 0) for i in range(bk)])
        E = _cheb_value_rows(N, p.kMin, p.kMax, gp[:kz, 2])  # (kz, N): the column's levels
        vf = (full @ CA.T) @ E.T  # (n_ring, kz)
        vm = (mean @ CA.T) @ E.T
        val = np.where(tap[:, None], w[:, None] * vf + (1.0 - w[:, None]) * vm, vf)
        if boundary == "nan":
            val[oob] = np.nan
        out[:, v] = val.reshape(-1)
    return out
