"""ctypes binding of ``libpyranda_gpu.so`` (the C ABI in include/pyranda_gpu.h).

The library is built in-tree by ``pyranda_gb300.build``.  There is no CPU
fallback: if the library cannot be loaded, every operator raises.
"""
import ctypes
import os

from . import build as _build

PG_OK, PG_EBADSHAPE, PG_ENULLOP, PG_ECUDA, PG_ENAN, PG_ETIMEOUT, PG_EINVAL, PG_ENOMEM = range(8)
PG_FP64, PG_FP32, PG_DENSE, PG_AUTO = 0, 1, 2, 3
_PRECISIONS = {"fp64": PG_FP64, "fp32": PG_FP32, "dense": PG_DENSE, "auto": PG_AUTO}


def precision_code(name):
    """'fp64' (reference arithmetic), 'fp32' (FP32 banded sweeps), 'dense' (split-TF32 tensor-core operators)
    or 'auto' (per operator and direction the faster of dense and FP32 banded, timed on the grid)."""
    try:
        return _PRECISIONS[name]
    except KeyError:
        raise ValueError("precision must be one of %s, not %r" % (sorted(_PRECISIONS), name)) from None


PG_SPECTRAL, PG_GAUSSIAN = 0, 1
PG_DIR_ALL = 3

_STATUS = {0: "PG_OK", 1: "PG_EBADSHAPE", 2: "PG_ENULLOP", 3: "PG_ECUDA", 4: "PG_ENAN",
           5: "PG_ETIMEOUT", 6: "PG_EINVAL", 7: "PG_ENOMEM"}


class PgError(RuntimeError):
    """A C-ABI call returned a non-zero pg_status."""

    def __init__(self, status, what, detail=""):
        self.status = status
        super().__init__("%s failed: %s %s" % (what, _STATUS.get(status, status), detail))


class pg_grid(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int * 3), ("periodic", ctypes.c_int * 3),
                ("x1", ctypes.c_double * 3), ("xn", ctypes.c_double * 3),
                ("precision", ctypes.c_int), ("bc", (ctypes.c_int * 2) * 3), ("coordsys", ctypes.c_int)]


PG_BC_NONE, PG_BC_SYMM, PG_BC_XTND = 0, 1, 2
PG_CARTESIAN, PG_CYLINDRICAL, PG_SPHERICAL, PG_CURVILINEAR, PG_SPHERICAL_RATIO = 0, 1, 2, 3, 4


PG_LAD_IN, PG_LAD_K, PG_LAD_HIDDEN, PG_LAD_OUT = 55, 64, 64, 2
PG_LAD_NWEIGHT = 3 * 64 * 64 + 2 * 64
PG_LAD_NPARAM = PG_LAD_NWEIGHT + 3 * 64 + 2


class pg_lad_model(ctypes.Structure):
    _fields_ = [("wbf16", ctypes.c_void_p), ("params", ctypes.c_void_p), ("xmean", ctypes.c_void_p),
                ("xinvstd", ctypes.c_void_p), ("ym", ctypes.c_float * 2), ("ys", ctypes.c_float * 2),
                ("ylo", ctypes.c_float * 2), ("yhi", ctypes.c_float * 2)]


_lib = None

# (name, restype, argtypes) of every exported entry point
P = ctypes.c_void_p
D = ctypes.c_void_p  # device pointers are passed as integers
I = ctypes.c_int
SIGNATURES = [
    ("pg_create", I, [ctypes.POINTER(pg_grid), ctypes.POINTER(P)]),
    ("pg_destroy", I, [P]),
    ("pg_set_precision", I, [P, I]),
    ("pg_device_status", I, [P, ctypes.POINTER(ctypes.c_int)]),
    ("pg_get_spacing", I, [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_dense_plan", I, [P, ctypes.POINTER(ctypes.c_int)]),
    ("pg_set_line_split", I, [P, I]),
    ("pg_sweep_plan", I, [P, ctypes.POINTER(ctypes.c_int)]),
    ("pg_set_sweep_plan", I, [P, ctypes.POINTER(ctypes.c_int)]),
    ("pg_wait_selftest", I, [P, ctypes.c_uint, P]),
    ("pg_last_error", ctypes.c_char_p, []),
    ("pg_version", ctypes.c_char_p, []),
    ("pg_d1", I, [P, I, D, D, P]),
    ("pg_d8", I, [P, I, D, D, P]),
    ("pg_d2", I, [P, I, D, D, P]),
    ("pg_d4", I, [P, I, D, D, P]),
    ("pg_laplacian", I, [P, D, D, P]),
    ("pg_filter", I, [P, I, I, D, D, P]),
    ("pg_ring", I, [P, D, D, P]),
    ("pg_d1_sym", I, [P, I, I, D, D, P]),
    ("pg_d8_sym", I, [P, I, I, D, D, P]),
    ("pg_filter_sym", I, [P, I, I, ctypes.POINTER(ctypes.c_int), D, D, P]),
    ("pg_ringv", I, [P, D, D, D, D, P]),
    ("pg_grad", I, [P, D, D, D, D, P]),
    ("pg_div", I, [P, D, D, D, D, P]),
    ("pg_divt", I, [P, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p), P]),
    ("pg_mesh", I, [P, I, D, P]),
    ("pg_set_mesh_coords", I, [P, D, D, D, I, P]),
    ("pg_rk_stage", I, [P, I, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                        ctypes.POINTER(ctypes.c_void_p), D, ctypes.c_double, ctypes.c_double, P]),
    ("pg_courant", I, [P, D, D, D, D, ctypes.c_double, ctypes.c_double, D, P]),
    ("pg_diff", I, [P, D, D, D, P]),
    ("pg_reduce", I, [P, I, D, ctypes.c_int64, D, P]),
    ("pg_check_finite", I, [D, ctypes.c_int64, D, P]),
    ("pg_d1_host", I, [P, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_d8_host", I, [P, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_d2_host", I, [P, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_d4_host", I, [P, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_laplacian_host", I, [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_filter_host", I, [P, I, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_ring_host", I, [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_launch_count", ctypes.c_uint64, []),
    ("pg_ens_create", I, [I, ctypes.POINTER(pg_grid), ctypes.POINTER(P)]),
    ("pg_ens_destroy", I, [P]),
    ("pg_ens_points", ctypes.c_int64, [P, ctypes.POINTER(ctypes.c_int64)]),
    ("pg_ens_set_precision", I, [P, I]),
    ("pg_ens_set_line_split", I, [P, I]),
    ("pg_ens_spacing", I, [P, I, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("pg_ens_d1", I, [P, I, D, D, P]),
    ("pg_ens_d8", I, [P, I, D, D, P]),
    ("pg_ens_d2", I, [P, I, D, D, P]),
    ("pg_ens_d4", I, [P, I, D, D, P]),
    ("pg_ens_laplacian", I, [P, D, D, P]),
    ("pg_ens_filter", I, [P, I, I, D, D, P]),
    ("pg_ens_ring", I, [P, D, D, P]),
    ("pg_ens_ringv", I, [P, D, D, D, D, P]),
    ("pg_ens_grad", I, [P, D, D, D, D, P]),
    ("pg_ens_div", I, [P, D, D, D, D, P]),
    ("pg_ens_mesh", I, [P, I, D, P]),
    ("pg_ens_rk_stage", I, [P, I, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                            ctypes.POINTER(ctypes.c_void_p), D, ctypes.c_double, ctypes.c_double, P]),
    ("pg_ens_courant", I, [P, D, D, D, D, ctypes.c_double, ctypes.c_double, D, P]),
    ("pg_ens_diff", I, [P, D, D, D, P]),
    ("pg_ens_reduce", I, [P, I, D, D, D, P]),
    ("pg_ens_device_status", I, [P, ctypes.POINTER(ctypes.c_int)]),
    ("pg_lad_closure", I, [P, ctypes.POINTER(pg_lad_model), D, D, D, D, ctypes.c_double, D, D, D, P]),
    ("pg_lad_features", I, [P, D, D, D, ctypes.c_int64, D, P]),
    ("pg_lad_grad_magnitude", I, [P, D, D, P]),
    ("pg_lad_normalize", I, [D, ctypes.c_int64, D, D, D, P]),
    ("pg_lad_train_step", I, [ctypes.POINTER(pg_lad_model), D, D, ctypes.c_int64, ctypes.c_float, D, D, D, P]),
    ("pg_lad_adam", I, [D, D, D, D, I, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, I, D, I, P]),
]


def lib_path():
    return _build.LIB


def load(build_if_missing=True):
    """Load (and if needed build) the CUDA library; raises if that fails."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not os.path.exists(path) or _build._needs_build():
        if not build_if_missing:
            raise RuntimeError("libpyranda_gpu.so is not built (run pyranda_gb300.build)")
        _build.build()
    L = ctypes.CDLL(path)
    for name, res, args in SIGNATURES:
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def check(rc, what):
    if rc != PG_OK:
        detail = ""
        try:
            detail = load().pg_last_error().decode()
        except Exception:
            pass
        raise PgError(rc, what, detail)


def launch_count():
    return int(load().pg_launch_count())
