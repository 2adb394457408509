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
    assert lib.pg_create(ctypes.byref(grid(coordsys=5)), ctypes.byref(h)) == _lib.PG_EINVAL
    assert b"coordsys" in lib.pg_last_error()
    assert lib.pg_create(ctypes.byref(grid(n0=0)), ctypes.byref(h)) == _lib.PG_EBADSHAPE
    assert lib.pg_create(ctypes.byref(grid(precision=9)), ctypes.byref(h)) == _lib.PG_EINVAL


def test_plan_cache_round_trip(tmp_path):
    """The autotuner's plan cache: a stored plan is read back under its key,
    other keys miss, malformed entries and files are ignored."""
    import json
    from pyranda_gb300 import grid
    path = str(tmp_path / "plans.json")
    assert grid._plan_cache_get("a", path) is None
    plan = [2] * 12 + [0] * 6
    grid._plan_cache_put("a", plan, path)
    grid._plan_cache_put("b", [1] * 18, path)
    assert grid._plan_cache_get("a", path) == plan
    assert grid._plan_cache_get("b", path) == [1] * 18
    assert grid._plan_cache_get("c", path) is None
    with open(path) as f:
        data = json.load(f)
    data["a"] = [7] * 18
    with open(path, "w") as f:
        json.dump(data, f)
    assert grid._plan_cache_get("a", path) is None
    with open(path, "w") as f:
        f.write("not json")
    assert grid._plan_cache_get("b", path) is None
    grid._plan_cache_put("b", [1] * 18, path)
    assert grid._plan_cache_get("b", path) == [1] * 18
