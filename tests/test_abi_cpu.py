"""The C ABI library builds, loads without a GPU and exports every entry point
that include/pyranda_gpu.h declares; the Python binding covers them all."""
import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "pyranda_gpu.h")


def declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared()
    for must in ("pg_create", "pg_destroy", "pg_d1", "pg_d8", "pg_filter", "pg_ring", "pg_ringv", "pg_grad",
                 "pg_div", "pg_rk_stage", "pg_courant", "pg_diff", "pg_reduce", "pg_reduce_noalloc"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from pyranda_gb300 import build
    path = build.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_header():
    from pyranda_gb300 import _lib
    bound = {name for name, _, _ in _lib.SIGNATURES}
    # the allocation-free reduction is bound by its own callers
    assert set(declared()) - bound <= {"pg_reduce_noalloc"}


def test_calls_without_gpu_fail_cleanly():
    """Host-side argument checks run before any CUDA call."""
    from pyranda_gb300 import _lib
    lib = _lib.load()
    assert lib.pg_d1(None, 0, None, None, None) == _lib.PG_EINVAL
    assert lib.pg_create(None, None) == _lib.PG_EINVAL
    assert b"NULL" in lib.pg_last_error()
    assert lib.pg_version().startswith(b"pyranda_gb300")


def test_grid_codes_checked_before_any_cuda_call():
    """pg_create validates the boundary codes, the coordinate system and the
    extents on the host, before it touches the device: bad values return
    PG_EINVAL / PG_EBADSHAPE with a message, with or without a GPU."""
    import ctypes
    from pyranda_gb300 import _lib
    lib = _lib.load()

    def grid(**kw):
        g = _lib.pg_grid()
        for d in range(3):
            g.n[d] = 16
            g.periodic[d] = 0
            g.x1[d], g.xn[d] = 0.0, 1.0
        for k, v in kw.items():
            if k == "bc":
                d, e, b = v
                g.bc[d][e] = b
            elif k == "n0":
                g.n[0] = v
            else:
                setattr(g, k, v)
        return g

    h = ctypes.c_void_p()
    assert lib.pg_create(ctypes.byref(grid(bc=(1, 0, 7))), ctypes.byref(h)) == _lib.PG_EINVAL
    assert b"pg_bc" in lib.pg_last_error()
    assert lib.pg_create(ctypes.byref(grid(coordsys=2)), ctypes.byref(h)) == _lib.PG_EINVAL
    assert b"coordsys" in lib.pg_last_error()
    assert lib.pg_create(ctypes.byref(grid(n0=0)), ctypes.byref(h)) == _lib.PG_EBADSHAPE
    assert lib.pg_create(ctypes.byref(grid(precision=9)), ctypes.byref(h)) == _lib.PG_EINVAL
