"""Host side of the grid archive (src/io.jl:410-439): the parameters written
into an archive's caller block rebuild the same C-ABI grid parameters."""
import ctypes as C

import springsteel_gpu as S
from springsteel_gpu import io as sio


def _abi_bytes(gp):
    bundle = gp.to_abi()
    p = bundle.ref._obj if hasattr(bundle.ref, "_obj") else bundle.ref
    out = [bytes(C.string_at(C.addressof(p), C.sizeof(p)))]
    nv = p.nvars
    for name in ("BCL", "BCR"):
        arr = getattr(p, name)
        out.append(bytes(C.string_at(C.cast(arr, C.c_void_p).value, nv * C.sizeof(S.abi.ss_spline_bc))))
    for name in ("l_q",):
        out.append(bytes(C.string_at(C.cast(getattr(p, name), C.c_void_p).value, nv * 8)))
    for name in ("max_wavenumber", "BCB", "BCT"):
        ptr = getattr(p, name)
        if ptr:
            out.append(bytes(C.string_at(C.cast(ptr, C.c_void_p).value, nv * 4)))
    # pointer fields differ between bundles; compare the scalar prefix only
    scal = [f for f, _ in S.abi.ss_grid_params._fields_ if not f[0].isupper() and f not in ("l_q", "max_wavenumber")]
    vals = tuple(getattr(p, f) for f in scal)
    return vals, out[1:]


def test_rl_params_roundtrip_through_archive_block():
    gp = S.SpringsteelGridParameters(
        geometry="RL", iMin=0.0, iMax=50.0, num_cells=25, vars={"u": 1, "w": 2},
        BCL={"u": S.DirichletBC(), "w": S.R1T1}, BCR={"default": S.RobinBC(1.0, -2.0)},
        l_q={"u": 3.0}, max_wavenumber={"default": -1, "w": 12}, spectralIndexL=3,
        fourier_filter={"u": S.SpectralFilter(low_pass=20, window="hann", taper_width=4)}, precision="f32")
    gp2 = sio._params_from_json(sio._params_json(gp))
    assert _abi_bytes(gp) == _abi_bytes(gp2)
    assert gp2.fourier_filter["u"].__dict__ == gp.fourier_filter["u"].__dict__
    assert (gp2.i_regular_out, gp2.j_regular_out) == (gp.i_regular_out, gp.j_regular_out)


def test_rlz_params_roundtrip_through_archive_block():
    gp = S.SpringsteelGridParameters(
        geometry="RLZ", iMin=0.0, iMax=60.0, num_cells=20, kMin=0.0, kMax=1e4, kDim=24,
        vars={"a": 1, "b": 2, "c": 3}, BCB={"default": S.DirichletBC()}, BCT={"b": S.NeumannBC()},
        chebyshev_filter={"default": S.GaussianFilter(sigma=0.3)}, max_wavenumber={"a": 30, "c": 40})
    gp2 = sio._params_from_json(sio._params_json(gp))
    assert _abi_bytes(gp) == _abi_bytes(gp2)
    assert gp2.shared_ring_kmax() == gp.shared_ring_kmax()
