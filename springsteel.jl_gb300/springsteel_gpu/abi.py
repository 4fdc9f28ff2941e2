"""ctypes mirror of ``include/springsteel_gpu.h``.

Every structure and constant here matches the C header field for field; the
host-side Python mirror of the reference API (``springsteel_gpu``) and the
tests build ``ss_grid_params`` through :func:`make_params`.
"""
import ctypes as C

SS_OK = 0
SS_BAD_ARG = 1
SS_BAD_SHAPE = 2
SS_NOT_SPD = 3
SS_UNSUPPORTED_BC = 4
SS_CUDA_ERROR = 5
SS_DEVICE_TIMEOUT = 6
SS_NAN_DETECTED = 7
SS_NOT_CONVERGED = 8
SS_OUT_OF_MEMORY = 9
SS_NO_DEVICE = 10

STATUS_NAMES = {
    0: "OK", 1: "BAD_ARG", 2: "BAD_SHAPE", 3: "NOT_SPD", 4: "UNSUPPORTED_BC",
    5: "CUDA_ERROR", 6: "DEVICE_TIMEOUT", 7: "NAN_DETECTED", 8: "NOT_CONVERGED",
    9: "OUT_OF_MEMORY", 10: "NO_DEVICE",
}

SS_GEOM_RL = 1
SS_GEOM_RLZ = 2
SS_PREC_F64 = 0
SS_PREC_F32_REFINED = 1
SS_PREC_F64_FAST = 2
SS_DTYPE_F64 = 0
SS_DTYPE_F32 = 1
SS_QUAD_GAUSS = 0
SS_QUAD_REGULAR = 1

SS_SBC_R0 = 0
SS_SBC_RANK1 = 1
SS_SBC_RANK2 = 2
SS_SBC_PERIODIC = 3
SS_SBC_R3 = 4
SS_SBC_R3X = 5

SS_BATCH_AUTOTUNE = 1
SS_BATCH_FUSED = 2

SS_CBC_R0 = 0
SS_CBC_R1T0 = 1
SS_CBC_R1T1 = 2


class ss_spline_bc(C.Structure):
    _fields_ = [("kind", C.c_int32), ("_pad", C.c_int32), ("alpha", C.c_double), ("beta", C.c_double)]


class ss_grid_params(C.Structure):
    _fields_ = [
        ("geometry", C.c_int32),
        ("precision", C.c_int32),
        ("num_cells", C.c_int32),
        ("mubar", C.c_int32),
        ("quadrature", C.c_int32),
        ("nvars", C.c_int32),
        ("kDim", C.c_int32),
        ("b_kDim", C.c_int32),
        ("patchOffsetL", C.c_int32),
        ("_pad0", C.c_int32),
        ("iMin", C.c_double),
        ("iMax", C.c_double),
        ("kMin", C.c_double),
        ("kMax", C.c_double),
        ("l_q", C.POINTER(C.c_double)),
        ("BCL", C.POINTER(ss_spline_bc)),
        ("BCR", C.POINTER(ss_spline_bc)),
        ("BCB", C.POINTER(C.c_int32)),
        ("BCT", C.POINTER(C.c_int32)),
        ("max_wavenumber", C.POINTER(C.c_int32)),
        ("ring_kmax_set", C.c_int32),
        ("ring_kmax", C.c_int32),
    ]


class ss_dims(C.Structure):
    _fields_ = [(n, C.c_int64) for n in (
        "iDim", "b_iDim", "jDim", "b_jDim", "kDim", "b_kDim", "kDim_wn", "nvars",
        "nslots", "n_physical", "n_spectral", "n_blocks")]

    def as_dict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class ParamBundle:
    """Keeps the per-variable arrays alive as long as the params struct."""

    def __init__(self, params, keep):
        self.params = params
        self._keep = keep

    @property
    def ref(self):
        return C.byref(self.params)


def make_params(geometry, num_cells, iMin, iMax, nvars, *, mubar=3, quadrature=SS_QUAD_GAUSS,
                kDim=0, b_kDim=0, kMin=0.0, kMax=0.0, patchOffsetL=0, precision=SS_PREC_F64,
                l_q=None, BCL=None, BCR=None, BCB=None, BCT=None, max_wavenumber=None, ring_kmax=None):
    """Build an ``ss_grid_params``.  Per-variable entries are sequences of
    length ``nvars``: l_q floats, BCL/BCR ``(kind, alpha, beta)`` tuples,
    BCB/BCT Chebyshev kinds, max_wavenumber ints (-1 = ring kmax).
    ``ring_kmax`` (RLZ) is the kmax cap of the rings every variable shares;
    None leaves it to the library (the last variable's entry)."""
    keep = []

    def arr(ctype, vals):
        a = (ctype * nvars)(*vals)
        keep.append(a)
        return C.cast(a, C.POINTER(ctype))

    def bcarr(vals):
        a = (ss_spline_bc * nvars)()
        for i, (k, al, be) in enumerate(vals):
            a[i].kind, a[i].alpha, a[i].beta = int(k), float(al), float(be)
        keep.append(a)
        return C.cast(a, C.POINTER(ss_spline_bc))

    p = ss_grid_params()
    p.geometry = int(geometry)
    p.precision = int(precision)
    p.num_cells = int(num_cells)
    p.mubar = int(mubar)
    p.quadrature = int(quadrature)
    p.nvars = int(nvars)
    p.kDim = int(kDim)
    p.b_kDim = int(b_kDim)
    p.patchOffsetL = int(patchOffsetL)
    p.iMin, p.iMax, p.kMin, p.kMax = float(iMin), float(iMax), float(kMin), float(kMax)
    if l_q is not None:
        p.l_q = arr(C.c_double, [float(x) for x in l_q])
    if BCL is not None:
        p.BCL = bcarr(BCL)
    if BCR is not None:
        p.BCR = bcarr(BCR)
    if BCB is not None:
        p.BCB = arr(C.c_int32, [int(x) for x in BCB])
    if BCT is not None:
        p.BCT = arr(C.c_int32, [int(x) for x in BCT])
    if max_wavenumber is not None:
        p.max_wavenumber = arr(C.c_int32, [int(x) for x in max_wavenumber])
    if ring_kmax is not None:
        p.ring_kmax_set, p.ring_kmax = 1, int(ring_kmax)
    return ParamBundle(p, keep)


# --- library binding ----------------------------------------------------------

EXPORTED = [
    "ss_version", "ss_last_error_string", "ss_grid_create", "ss_grid_destroy", "ss_grid_dims",
    "ss_grid_stream", "ss_grid_device_physical", "ss_grid_device_spectral",
    "ss_upload_physical", "ss_download_physical", "ss_upload_spectral", "ss_download_spectral",
    "ss_spectral_transform", "ss_grid_transform", "ss_spectral_transform_from_host",
    "ss_grid_transform_to_host", "ss_grid_set_filter", "ss_grid_set_ahat",
    "ss_grid_clear_ahat", "ss_grid_synchronize", "ss_grid_profile", "ss_grid_profile_read", "ss_fft_plan",
    "ss_spectral_transform_noalloc", "ss_regular_grid_transform", "ss_evaluate_unstructured", "ss_relocate_grid", "ss_spline_transform", "ss_tile_transform",
    "ss_grid_save", "ss_grid_load", "ss_grid_load_arrays", "ss_grid_archive_user",
    "ss_batch_create", "ss_batch_destroy", "ss_batch_run", "ss_batch_synchronize", "ss_batch_ring_threads", "ss_batch_fused_launches",
    "ss_chain_create", "ss_chain_create_embedded", "ss_chain_destroy", "ss_multi_grid_transform",
    "ss_tile_sum_spectral", "ss_tile_copy_physical", "ss_grid_zero_spectral",
    "ss_problem_create", "ss_problem_destroy", "ss_problem_dims", "ss_problem_operator_band",
    "ss_problem_set_mlp", "ss_solve", "ss_problem_export", "ss_problem_collect_training",
    "ss_problem_collect_random",
    "ss_mlp_create", "ss_mlp_destroy", "ss_mlp_set_params", "ss_mlp_get_params", "ss_mlp_forward",
    "ss_mlp_gradients", "ss_mlp_dataset_rows", "ss_mlp_dataset_clear", "ss_mlp_train",
]

SS_SOLVER_DIRECT = 0
SS_SOLVER_GMRES_JACOBI = 1
SS_SOLVER_FGMRES_MLP = 2
MLP_WIDTH = 256
MLP_LAYERS = 3


class ss_solve_stats(C.Structure):
    _fields_ = [("method", C.c_int32), ("systems", C.c_int32), ("converged", C.c_int32),
                ("max_iterations", C.c_int32), ("fallback_systems", C.c_int32), ("_pad", C.c_int32),
                ("mean_iterations", C.c_double), ("max_rel_residual", C.c_double), ("ms", C.c_double)]


class ss_train_stats(C.Structure):
    _fields_ = [("epochs", C.c_int32), ("_pad", C.c_int32), ("steps", C.c_int64), ("rows", C.c_int64),
                ("first_epoch_loss", C.c_double), ("last_epoch_loss", C.c_double), ("ms", C.c_double)]


class ss_fft_plan_info(C.Structure):
    _fields_ = [("n", C.c_int32), ("kind", C.c_int32), ("nrad", C.c_int32), ("rad", C.c_int32 * 24),
                ("rader_p", C.c_int32), ("rader_inner", C.c_int32), ("inner_nrad", C.c_int32),
                ("inner_rad", C.c_int32 * 24), ("bluestein_m", C.c_int32), ("max_prime", C.c_int32),
                ("pad_prime", C.c_int32), ("_pad", C.c_int32)]


FFT_DIRECT, FFT_RADER, FFT_BLUESTEIN = 0, 1, 2

STAGES = ["cheb_forward", "ring_forward", "sb_project", "sa_si", "ring_inverse", "cheb_inverse"]


def bind(lib):
    """Attach argtypes/restypes of every entry point of the C ABI to ``lib``."""
    vp = C.c_void_p
    i32 = C.c_int32
    sig = {
        "ss_version": ([], i32),
        "ss_last_error_string": ([], C.c_char_p),
        "ss_grid_create": ([C.POINTER(ss_grid_params), C.POINTER(vp)], i32),
        "ss_grid_destroy": ([vp], i32),
        "ss_grid_dims": ([vp, C.POINTER(ss_dims)], i32),
        "ss_grid_stream": ([vp, C.POINTER(vp)], i32),
        "ss_grid_device_physical": ([vp, C.POINTER(vp)], i32),
        "ss_grid_device_spectral": ([vp, C.POINTER(vp)], i32),
        "ss_upload_physical": ([vp, vp, i32, i32, vp], i32),
        "ss_download_physical": ([vp, vp, i32, i32, vp], i32),
        "ss_upload_spectral": ([vp, vp, i32, vp], i32),
        "ss_download_spectral": ([vp, vp, i32, vp], i32),
        "ss_spectral_transform": ([vp, vp], i32),
        "ss_grid_transform": ([vp, vp], i32),
        "ss_spectral_transform_from_host": ([vp, vp, i32, vp], i32),
        "ss_grid_transform_to_host": ([vp, vp, i32, vp], i32),
        "ss_grid_set_filter": ([vp, i32, vp, vp], i32),
        "ss_grid_set_ahat": ([vp, i32, i32, vp], i32),
        "ss_grid_clear_ahat": ([vp], i32),
        "ss_grid_synchronize": ([vp], i32),
        "ss_grid_profile": ([vp, i32], i32),
        "ss_grid_profile_read": ([vp, C.POINTER(C.c_double), C.POINTER(C.c_int64)], i32),
        "ss_fft_plan": ([i32, i32, C.POINTER(ss_fft_plan_info)], i32),
        "ss_spectral_transform_noalloc": ([vp, vp, vp, vp], i32),
        "ss_regular_grid_transform": ([vp, vp, i32, vp, i32, vp, i32, vp, vp], i32),
        "ss_spline_transform": ([vp, vp, vp], i32),
        "ss_evaluate_unstructured": ([vp, vp, C.c_int64, vp, i32, C.c_double, vp], i32),
        "ss_relocate_grid": ([vp, vp, C.c_double, C.c_double, i32, i32, vp], i32),
        "ss_tile_transform": ([vp, vp], i32),
        "ss_grid_save": ([vp, C.c_char_p, vp, C.c_int64, vp], i32),
        "ss_grid_load": ([C.c_char_p, C.POINTER(vp), vp], i32),
        "ss_grid_load_arrays": ([vp, C.c_char_p, vp], i32),
        "ss_grid_archive_user": ([C.c_char_p, vp, C.c_int64, C.POINTER(C.c_int64)], i32),
        "ss_batch_create": ([vp, i32, i32, C.POINTER(vp)], i32),
        "ss_batch_destroy": ([vp], i32),
        "ss_batch_run": ([vp, i32, i32, vp], i32),
        "ss_batch_fused_launches": ([vp, i32, C.POINTER(i32)], i32),
        "ss_batch_synchronize": ([vp], i32),
        "ss_batch_ring_threads": ([vp, i32, C.POINTER(i32), C.POINTER(i32)], i32),
        "ss_chain_create": ([vp, i32, C.POINTER(vp)], i32),
        "ss_chain_create_embedded": ([vp, i32, C.POINTER(vp)], i32),
        "ss_chain_destroy": ([vp], i32),
        "ss_multi_grid_transform": ([vp, vp], i32),
        "ss_tile_sum_spectral": ([vp, vp, i32, vp], i32),
        "ss_tile_copy_physical": ([vp, vp, i32, i32, vp], i32),
        "ss_grid_zero_spectral": ([vp, vp], i32),
        "ss_problem_create": ([vp, vp, C.POINTER(vp)], i32),
        "ss_problem_destroy": ([vp], i32),
        "ss_problem_dims": ([vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)], i32),
        "ss_problem_operator_band": ([vp, i32, vp, C.POINTER(i32), C.POINTER(i32)], i32),
        "ss_problem_set_mlp": ([vp, vp, i32], i32),
        "ss_solve": ([vp, i32, C.c_double, i32, i32, C.POINTER(ss_solve_stats), vp], i32),
        "ss_problem_export": ([vp, vp, vp, vp, vp], i32),
        "ss_problem_collect_training": ([vp, vp, vp, vp, vp, i32, i32], i32),
        "ss_problem_collect_random": ([vp, vp, i32, C.c_uint64, i32, i32], i32),
        "ss_mlp_create": ([i32, C.c_uint64, C.POINTER(vp)], i32),
        "ss_mlp_destroy": ([vp], i32),
        "ss_mlp_set_params": ([vp, vp, vp], i32),
        "ss_mlp_get_params": ([vp, vp, vp], i32),
        "ss_mlp_forward": ([vp, vp, vp, C.c_int64], i32),
        "ss_mlp_gradients": ([vp, vp, vp, vp, C.c_int64, vp, vp, C.POINTER(C.c_double)], i32),
        "ss_mlp_dataset_rows": ([vp, C.POINTER(C.c_int64)], i32),
        "ss_mlp_dataset_clear": ([vp], i32),
        "ss_mlp_train": ([vp, i32, i32, C.c_float, C.c_uint64, C.POINTER(ss_train_stats)], i32),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib
