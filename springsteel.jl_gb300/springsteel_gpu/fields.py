"""Seeded synthetic fields of the benchmark shapes (no public dataset is involved).

All generators use numpy's PCG64 (``numpy.random.default_rng(seed)``), which is
bit-reproducible across platforms.
"""
import numpy as np

from . import SpringsteelGridParameters, DirichletBC, NaturalBC


def gaussian_ring_field(points, seed=1, noise=1e-3):
    """u = exp(-(r/20)²)(1 + 0.1 cos 2λ) + N(0, noise) at the gridpoints (RL shape)."""
    r, lam = points[:, 0], points[:, 1]
    rng = np.random.default_rng(seed)
    return np.exp(-((r / 20.0) ** 2)) * (1.0 + 0.1 * np.cos(2.0 * lam)) + rng.normal(0.0, noise, r.shape)


def blob_sum(points, seed, nblobs=8, rmax=None, zmin=0.0, zmax=1.0, wmin=5.0, wmax=30.0, vert=100.0,
             noise=0.0):
    """Σ A exp(-[(x-xc)²+(y-yc)²]/w² - (z-zc)²/(vert·w)²), x = r cos λ, y = r sin λ.

    Centres are uniform in the disc of radius rmax (and in [zmin, zmax]),
    widths w ~ U[wmin, wmax], amplitudes A ~ N(0, 1).  ``points`` has columns
    (r, λ[, z]); a 2-column input drops the z factor."""
    rng = np.random.default_rng(seed)
    r, lam = points[:, 0], points[:, 1]
    x, y = r * np.cos(lam), r * np.sin(lam)
    if rmax is None:
        rmax = float(r.max())
    has_z = points.shape[1] > 2
    z = points[:, 2] if has_z else None
    out = np.zeros(r.shape)
    for _ in range(nblobs):
        rc = rmax * np.sqrt(rng.uniform())
        tc = rng.uniform(0.0, 2 * np.pi)
        xc, yc = rc * np.cos(tc), rc * np.sin(tc)
        zc = rng.uniform(zmin, zmax)
        w = rng.uniform(wmin, wmax)
        A = rng.normal()
        e = ((x - xc) ** 2 + (y - yc) ** 2) / (w * w)
        if has_z:
            e = e + ((z - zc) / (vert * w)) ** 2
        out += A * np.exp(-e)
    if noise:
        out += rng.normal(0.0, noise, out.shape)
    return out


# ---------------------------------------------------------------- benchmark shapes
def rl100_params(precision="f64"):
    """RL, radius 0-100, 100 cells × 3 Gauss points, rings of 4+4r, one variable.
    NaturalBC at both ends (the reference has no RL axis-regularity BC)."""
    return SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=100.0, num_cells=100,
                                     BCL={"default": NaturalBC()}, BCR={"default": NaturalBC()},
                                     vars={"u": 1}, precision=precision)


def rlz_params(precision="f64", num_cells=200, kDim=32, nvars=5):
    """RLZ, 200 cells on r ∈ [0, 200] (DX = 1), 32 Chebyshev levels on z ∈ [0, 20000],
    5 variables, Dirichlet in z (Chebyshev R1T0 both ends)."""
    vars_ = {"v%d" % i: i for i in range(1, nvars + 1)}
    return SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=float(num_cells), num_cells=num_cells,
                                     kMin=0.0, kMax=20000.0, kDim=kDim, vars=vars_,
                                     BCB={"default": DirichletBC()}, BCT={"default": DirichletBC()},
                                     precision=precision)


def rlz400_f32_params(precision="f32", num_cells=400, kDim=64, nvars=8):
    """RLZ, 400 cells (r ∈ [0, 400]), 64 Chebyshev levels on z ∈ [0, 20000], 8 variables."""
    vars_ = {"v%d" % i: i for i in range(1, nvars + 1)}
    return SpringsteelGridParameters(geometry="RLZ", iMin=0.0, iMax=float(num_cells), num_cells=num_cells,
                                     kMin=0.0, kMax=20000.0, kDim=kDim, vars=vars_,
                                     BCB={"default": DirichletBC()}, BCT={"default": DirichletBC()},
                                     precision=precision)


def rlz_blob_fields(points, nvars, base_seed=2, zmax=20000.0, noise=0.0):
    """(n_physical, nvars) Fortran-ordered array of per-variable blob sums."""
    out = np.empty((points.shape[0], nvars), order="F")
    for v in range(nvars):
        out[:, v] = blob_sum(points, seed=base_seed * 1000 + v, zmax=zmax, noise=noise)
    return out


# ----------------------------------------------------------------- elliptic solve
def elliptic_rl200_params(num_cells=200, rmax=100.0):
    """RL, 200 cells on r ∈ [0, 100], rings of 4+4r, one variable, native FP64."""
    return SpringsteelGridParameters(geometry="RL", iMin=0.0, iMax=float(rmax), num_cells=num_cells,
                                     BCL={"default": NaturalBC()}, BCR={"default": NaturalBC()},
                                     vars={"u": 1}, precision="f64")


def k2_profile(r, seed, rmax=None):
    """k²(r) = Σ_{i<3} a_i exp(−(r − c_i)²/s_i²) > 0: a ~ U[0.002, 0.02], c ~ U[0, rmax],
    s ~ U[rmax/10, rmax/3]."""
    r = np.asarray(r, np.float64)
    rmax = float(r.max()) if rmax is None else float(rmax)
    rng = np.random.default_rng(seed)
    out = np.zeros_like(r)
    for _ in range(3):
        a = rng.uniform(0.002, 0.02)
        c = rng.uniform(0.0, rmax)
        s = rng.uniform(rmax / 10.0, rmax / 3.0)
        out += a * np.exp(-((r - c) / s) ** 2)
    return out


def elliptic_blobs(seed, rmax=100.0, nmin=1, nmax=12, wmin=5.0, wmax=30.0):
    """Forcing of one elliptic sample: 1–12 blobs (xc, yc, w, A), centres uniform in the
    disc, widths U[wmin, wmax], amplitudes N(0, 1)."""
    rng = np.random.default_rng(seed)
    nb = int(rng.integers(nmin, nmax + 1))
    out = np.empty((nb, 4))
    for i in range(nb):
        rc = rmax * np.sqrt(rng.uniform())
        tc = rng.uniform(0.0, 2 * np.pi)
        out[i] = (rc * np.cos(tc), rc * np.sin(tc), rng.uniform(wmin, wmax), rng.normal())
    return out


def blob_field(points, blobs):
    """Σ A exp(−[(x − xc)² + (y − yc)²]/w²) at (r, λ) points."""
    r, lam = points[:, 0], points[:, 1]
    x, y = r * np.cos(lam), r * np.sin(lam)
    out = np.zeros(r.shape)
    for xc, yc, w, A in np.asarray(blobs).reshape(-1, 4):
        out += A * np.exp(-((x - xc) ** 2 + (y - yc) ** 2) / (w * w))
    return out


def radial_mish(gp):
    """The iDim radial Gauss points x = iMin + (mc + q_μ) DX (src/CubicBSpline.jl:887-897)."""
    nc, mb = gp.num_cells, gp.mubar
    DX = (gp.iMax - gp.iMin) / nc
    if gp.quadrature == "gauss":
        nodes = np.polynomial.legendre.leggauss(mb)[0] if mb != 3 else np.array([-np.sqrt(0.6), 0.0, np.sqrt(0.6)])
        q = (nodes + 1.0) / 2.0
    else:
        q = (2 * np.arange(1, mb + 1) - 1) / (2 * mb)
    return np.array([gp.iMin + mc * DX + q[mu] * DX for mc in range(nc) for mu in range(mb)])


# ------------------------------------------------------------ device-side fields
def column_coordinates_device(grid):
    """(r, λ) of every ring point in jDim order and the Chebyshev levels z (for RLZ),
    as torch CUDA float64 tensors: the getGridpoints coordinates without building
    the (n_physical, 3) host array."""
    import math

    import torch

    gp, d = grid.params, grid.dims
    rmish = torch.tensor(radial_mish(gp), dtype=torch.float64, device="cuda")
    ri = torch.arange(1, d["iDim"] + 1, device="cuda", dtype=torch.int64) + gp.patchOffsetL
    L = 4 + 4 * ri
    ring = torch.repeat_interleave(torch.arange(d["iDim"], device="cuda"), L)
    start = torch.cumsum(L, 0) - L
    j = torch.arange(int(L.sum().item()), device="cuda") - start[ring]
    Lr = L[ring].to(torch.float64)
    lam = 0.5 * (2 * math.pi / Lr) * (ri[ring].to(torch.float64) - 1) + 2 * math.pi * j.to(torch.float64) / Lr
    r = rmish[ring]
    z = None
    if gp.geometry == "RLZ":
        N = gp.kDim
        scale, offset = -0.5 * (gp.kMax - gp.kMin), 0.5 * (gp.kMin + gp.kMax)
        z = torch.cos(torch.arange(N, device="cuda", dtype=torch.float64) * math.pi / (N - 1)) * scale + offset
    return r, lam, z


def blob_sum_device(coords, seed, nblobs=8, rmax=None, zmin=0.0, zmax=1.0, wmin=5.0, wmax=30.0, vert=100.0,
                    noise=0.0):
    """blob_sum evaluated on the GPU (float64) from column_coordinates_device output:
    the same random draws in the same order, so the field equals blob_sum's to
    rounding; the optional N(0, noise) term comes from a seeded torch CUDA
    generator.  Returns a flat tensor in physical-row order (z fastest for RLZ)."""
    import torch

    r, lam, z = coords
    rng = np.random.default_rng(seed)
    x, y = r * torch.cos(lam), r * torch.sin(lam)
    if rmax is None:
        rmax = float(r.max().item())
    kz = 1 if z is None else z.numel()
    out = torch.zeros((r.numel(), kz), dtype=torch.float64, device="cuda")
    for _ in range(nblobs):
        rc = rmax * np.sqrt(rng.uniform())
        tc = rng.uniform(0.0, 2 * np.pi)
        xc, yc = rc * np.cos(tc), rc * np.sin(tc)
        zc = rng.uniform(zmin, zmax)
        w = rng.uniform(wmin, wmax)
        A = rng.normal()
        e = (((x - xc) ** 2 + (y - yc) ** 2) / (w * w))[:, None]
        if z is not None:
            e = e + (((z - zc) / (vert * w)) ** 2)[None, :]
        out += A * torch.exp(-e)
    out = out.reshape(-1)
    if noise:
        g = torch.Generator(device="cuda")
        g.manual_seed(int(seed))
        out += noise * torch.randn(out.shape, dtype=torch.float64, device="cuda", generator=g)
    return out


def fill_rlz_blobs_device(grid, base_seed=2, zmax=20000.0, noise=0.0, variables=None):
    """Write seeded blob-sum fields into physical slot 1 of `grid` on the device
    (variables not listed are zeroed); returns {var: float64 tensor of the field}."""
    coords = column_coordinates_device(grid)
    out = {}
    nv = grid.dims["nvars"]
    for v in range(nv):
        dst = grid.device_array("physical", v, slot=1)
        if variables is not None and v not in variables:
            dst.zero_()
            continue
        f = blob_sum_device(coords, seed=base_seed * 1000 + v, zmax=zmax, noise=noise)
        dst.copy_(f)
        out[v] = f
    import torch

    torch.cuda.synchronize()
    return out
