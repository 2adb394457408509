"""pg_reduce_noalloc: the reduction for callers that cannot allocate device memory.

Some callers cannot call cudaMalloc (their host framework owns all device
memory, or they never create a pg_handle and so own no workspace).  The
allocation-free entry point keeps its scratch in a static device array; this
test calls it through the C ABI and checks it against pg_reduce, twice in a
row so the second call starts from the scratch the first one left behind, and
both of them against numpy's sum / max / min of the host copy, including
inputs that hold infinities and NaN.
It lives in its own file, collected last, and needs nothing from other tests.
"""
import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _lib():
    from pyranda_gb300 import _lib as L
    lib = L.load()
    f = lib.pg_reduce_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p]
    return L, lib


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def test_noalloc_matches_pg_reduce_twice():
    L, lib = _lib()
    from pyranda_gb300.grid import Grid
    g = Grid((256, 128, 96), (True, True, True), (0, 0, 0), (1, 1, 1))  # the existing pg_reduce needs a handle
    gen = torch.Generator(device="cuda").manual_seed(7)
    calls = [torch.randn(256 * 128 * 96, dtype=torch.float64, device="cuda", generator=gen),
             torch.rand(1000, dtype=torch.float64, device="cuda", generator=gen) - 0.25]
    for x in calls:  # two calls in a row per op; the second has fewer blocks than the first
        for op in (0, 1, 2):
            out = torch.empty((), dtype=torch.float64, device="cuda")
            rc = lib.pg_reduce_noalloc(op, ctypes.c_void_p(x.data_ptr()), x.numel(),
                                       ctypes.c_void_p(out.data_ptr()), _stream())
            L.check(rc, "pg_reduce_noalloc")
            ref = g.reduce(op, x)
            torch.cuda.synchronize()
            a, b = float(out), float(ref)
            if op == 0:
                assert abs(a - b) <= 1e-13 * float(x.abs().sum()), (op, a, b)
            else:
                assert a == b, (op, a, b)


def test_noalloc_rejects_oversize():
    L, lib = _lib()
    limit = 8192 * 4096
    x = torch.zeros(limit + 1, dtype=torch.float64, device="cuda")  # real buffer: no read can leave it
    out = torch.empty((), dtype=torch.float64, device="cuda")
    rc = lib.pg_reduce_noalloc(0, ctypes.c_void_p(x.data_ptr()), limit + 1, ctypes.c_void_p(out.data_ptr()),
                               _stream())
    assert rc == L.PG_EBADSHAPE
    assert b"static scratch limit" in lib.pg_last_error()
    rc = lib.pg_reduce_noalloc(1, ctypes.c_void_p(x.data_ptr()), limit, ctypes.c_void_p(out.data_ptr()), _stream())
    L.check(rc, "pg_reduce_noalloc")
    assert float(out) == 0.0


def _host_ref(op, a):
    with numpy.errstate(invalid="ignore", over="ignore"):
        return (numpy.sum, numpy.max, numpy.min)[op](a)


def _same(a, b, scale):
    if numpy.isnan(b):
        return numpy.isnan(a)
    if numpy.isinf(b):
        return a == b
    return abs(a - b) <= 1e-13 * max(scale, 1.0)


def test_noalloc_and_pg_reduce_follow_numpy_on_special_values():
    L, lib = _lib()
    from pyranda_gb300.grid import Grid
    g = Grid((64, 32, 16), (True, True, True), (0, 0, 0), (1, 1, 1))
    rng = numpy.random.default_rng(3)
    n = 64 * 32 * 16
    base = rng.standard_normal(n)
    cases = {
        "all -inf": numpy.full(n, -numpy.inf),
        "all +inf": numpy.full(n, numpy.inf),
        "one NaN": numpy.where(numpy.arange(n) == n // 3, numpy.nan, base),
        "one +inf": numpy.where(numpy.arange(n) == 77, numpy.inf, base),
        "+inf and -inf": numpy.where(numpy.arange(n) == 5, numpy.inf, numpy.where(numpy.arange(n) == 9, -numpy.inf,
                                                                                 base)),
        "random": base,
    }
    for name, a in cases.items():
        x = torch.from_numpy(a).cuda()
        for op in (0, 1, 2):
            for call in range(2):  # two calls in a row
                out = torch.empty((), dtype=torch.float64, device="cuda")
                rc = lib.pg_reduce_noalloc(op, ctypes.c_void_p(x.data_ptr()), x.numel(),
                                           ctypes.c_void_p(out.data_ptr()), _stream())
                L.check(rc, "pg_reduce_noalloc")
                ref = g.reduce(op, x)
                torch.cuda.synchronize()
                want = float(_host_ref(op, a))
                scale = float(numpy.nansum(numpy.abs(numpy.where(numpy.isfinite(a), a, 0.0))))
                assert _same(float(out), want, scale), (name, op, call, float(out), want)
                assert _same(float(ref), want, scale), (name, op, "pg_reduce", float(ref), want)
