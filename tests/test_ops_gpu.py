"""Parity of the CUDA compact operators with the oracle, through the C ABI.

Bar: relative L2 <= 1e-12 against the FP64 oracle for every operator, on
periodic and one-sided (NONE) directions, on tile-aligned and ragged sizes, on
null directions (n = 1 and n < 4) and on long lines (tile widths 32/16/8).
"""
import ctypes
import math

import numpy
import pytest

from tests.helpers import rel_l2, smooth_field, to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1.0e-12

CASES = [
    # (shape, periodic)
    ((32, 32, 32), (True, True, True)),
    ((40, 24, 16), (True, False, True)),
    ((24, 40, 12), (False, True, False)),
    ((9, 13, 11), (False, False, False)),
    ((8, 8, 8), (True, True, True)),
    ((100, 1, 1), (False, False, False)),
    ((64, 64, 1), (True, False, False)),
    ((48, 3, 10), (True, True, True)),
    ((300, 3, 2), (True, False, False)),
    ((600, 2, 9), (False, False, True)),
    ((1024, 2, 1), (True, False, False)),
]


def _ids(c):
    return "x".join(map(str, c[0])) + "-" + "".join("P" if p else "N" for p in c[1])


@pytest.fixture(scope="module")
def grids(oracle):
    from pyranda_gb300.grid import Grid
    out = {}
    for shape, per in CASES:
        x1 = (0.0, -0.5, 0.25)
        xn = (1.0, 2.0, 3.0)
        out[(shape, per)] = (Grid(shape, per, x1, xn), oracle.OracleGrid(shape, per, x1, xn))
    return out


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_d1_d8_filters(grids, case):
    g, o = grids[case]
    v = smooth_field(case[0], seed=1)
    dv = to_dev(v, torch)
    for d in range(3):
        assert rel_l2(to_host(g.d1(d, dv)), o.apply(0, d, v)) <= TOL, ("d1", d)
        assert rel_l2(to_host(g.d8(d, dv)), o.apply(1, d, v)) <= TOL, ("d8", d)
        assert rel_l2(to_host(g.filter("spectral", dv, d)), o.apply(2, d, v)) <= TOL, ("sf", d)
        assert rel_l2(to_host(g.filter("gaussian", dv, d)), o.apply(3, d, v)) <= TOL, ("gf", d)
        assert rel_l2(to_host(g.d2(d, dv)), o.apply(4, d, v)) <= TOL, ("d2", d)
        assert rel_l2(to_host(g.d4(d, dv)), o.apply(5, d, v)) <= TOL, ("d4", d)


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_composites(grids, case):
    g, o = grids[case]
    v = smooth_field(case[0], seed=2)
    w = smooth_field(case[0], seed=3)
    q = smooth_field(case[0], seed=4)
    dv, dw, dq = (to_dev(a, torch) for a in (v, w, q))
    assert rel_l2(to_host(g.filter("spectral", dv)), o.sfilter(v)) <= TOL
    assert rel_l2(to_host(g.filter("gaussian", dv)), o.gfilter(v)) <= TOL
    assert rel_l2(to_host(g.ring(dv)), o.ring(v, 2)) <= TOL
    assert rel_l2(to_host(g.ringv(dv, dw, dq)), o.ringv(v, w, q, 1)) <= TOL
    for a, b in zip(g.grad(dv), o.grad(v)):
        assert rel_l2(to_host(a), b) <= TOL
    assert rel_l2(to_host(g.div(dv, dw, dq)), o.div(v, w, q)) <= TOL
    assert rel_l2(to_host(g.laplacian(dv)), o.laplacian(v)) <= TOL
    t = [smooth_field(case[0], seed=10 + k) for k in range(9)]
    for a, b in zip(g.divT(*[to_dev(x, torch) for x in t]),
                    (o.div(t[0], t[3], t[6]), o.div(t[1], t[4], t[7]), o.div(t[2], t[5], t[8]))):
        assert rel_l2(to_host(a), b) <= TOL


@pytest.mark.parametrize("case", CASES[:4], ids=_ids)
def test_mesh(grids, case):
    g, o = grids[case]
    for which in range(8):
        assert numpy.array_equal(to_host(g.mesh(which)), o.mesh(which)), which


def test_in_place(grids):
    """out may alias in for single sweeps and the 3-sweep filters (tile-local)."""
    g, o = grids[CASES[1]]
    v = smooth_field(CASES[1][0], seed=5)
    for d in range(3):
        t = to_dev(v, torch)
        g.d1(d, t, out=t)
        assert rel_l2(to_host(t), o.apply(0, d, v)) <= TOL
    t = to_dev(v, torch)
    g.filter("spectral", t, out=t)
    assert rel_l2(to_host(t), o.sfilter(v)) <= TOL


def test_constants_preserved(grids):
    """Filters keep constants and d1/d8 of a constant vanish (difference form)."""
    for (shape, per), (g, _) in grids.items():
        c = g.field(torch.full(shape, 3.25, dtype=torch.float64, device="cuda"))
        assert torch.equal(g.filter("spectral", c), c)
        assert torch.equal(g.filter("gaussian", c), c)
        assert float(g.d1(0, c).abs().max()) == 0.0
        assert float(g.d8(0, c).abs().max()) == 0.0


def test_host_variants(grids):
    from pyranda_gb300 import _lib
    g, o = grids[CASES[1]]
    L = _lib.load()
    v = smooth_field(CASES[1][0], seed=6)
    out = numpy.zeros_like(v)
    P = ctypes.POINTER(ctypes.c_double)
    vin = v.ctypes.data_as(P)
    vout = out.ctypes.data_as(P)
    _lib.check(L.pg_d1_host(g.h, 1, vin, vout), "pg_d1_host")
    assert rel_l2(out, o.apply(0, 1, v)) <= TOL
    _lib.check(L.pg_d8_host(g.h, 2, vin, vout), "pg_d8_host")
    assert rel_l2(out, o.apply(1, 2, v)) <= TOL
    _lib.check(L.pg_filter_host(g.h, 0, 3, vin, vout), "pg_filter_host")
    assert rel_l2(out, o.sfilter(v)) <= TOL
    _lib.check(L.pg_ring_host(g.h, vin, vout), "pg_ring_host")
    assert rel_l2(out, o.ring(v, 2)) <= TOL


def test_errors_do_not_exit(grids):
    """Bad arguments come back as a status, never a process exit (compact_d1.f90:65-72 stopped)."""
    from pyranda_gb300 import _lib
    L = _lib.load()
    g, _ = grids[CASES[0]]
    assert L.pg_d1(g.h, 7, None, None, None) == _lib.PG_EINVAL
    assert L.pg_filter(g.h, 5, 0, None, None, None) == _lib.PG_EINVAL
    h = ctypes.c_void_p()
    grid = _lib.pg_grid()
    grid.n[0], grid.n[1], grid.n[2] = 6, 1, 1  # 4 <= n < 8 has no valid stencil
    assert L.pg_create(ctypes.byref(grid), ctypes.byref(h)) == _lib.PG_EBADSHAPE
    grid.n[0] = 0
    assert L.pg_create(ctypes.byref(grid), ctypes.byref(h)) == _lib.PG_EBADSHAPE


def test_reductions_and_timestep(grids):
    g, o = grids[CASES[0]]
    shape = CASES[0][0]
    u, v, w = (smooth_field(shape, s) for s in (7, 8, 9))
    c = 2.0 + numpy.abs(smooth_field(shape, 10))
    du, dvv, dw, dc = (to_dev(a, torch) for a in (u, v, w, c))
    d1, d2, d3 = o.spacing()[1]
    gl = min(d1, d2, d3)
    ref = 1.0 / numpy.max(numpy.abs(u) / d1 + numpy.abs(v) / d2 + numpy.abs(w) / d3 + numpy.abs(c) / gl)
    assert abs(float(g.courant(du, dvv, dw, dc)) - ref) <= 1e-15 * ref
    assert abs(float(g.courant(du, 0.0, 0.0, dc)) - 1.0 / numpy.max(numpy.abs(u) / d1 + numpy.abs(c) / gl)) <= 1e-16
    bulk = numpy.abs(w) * 1e-3
    ref = numpy.min(c * gl * gl / numpy.maximum(1e-12, bulk))
    assert abs(float(g.diff(to_dev(bulk, torch), dc)) - ref) <= 1e-14 * ref
    assert abs(float(g.reduce(0, du)) - u.sum()) <= 1e-12 * numpy.abs(u).sum()
    assert float(g.reduce(1, du)) == u.max()
    assert float(g.reduce(2, du)) == u.min()
    du[3, 4, 5] = float("nan")
    assert numpy.isnan(float(g.reduce(1, du)))


def test_rk_stage(grids):
    g, _ = grids[CASES[0]]
    shape = CASES[0][0]
    U = [smooth_field(shape, s) for s in (11, 12)]
    PHI = [smooth_field(shape, s) for s in (13, 14)]
    F = [smooth_field(shape, s) for s in (15, 16)]
    dt, A, B = 0.01, -0.48, 0.74
    dU = [to_dev(a, torch) for a in U]
    dP = [to_dev(a, torch) for a in PHI]
    dF = [to_dev(a, torch) for a in F]
    g.rk_stage(dU, dP, dF, torch.tensor(dt, dtype=torch.float64, device="cuda"), A, B)
    for k in range(2):
        phi = dt * F[k] + A * PHI[k]
        assert rel_l2(to_host(dP[k]), phi) <= 1e-15
        assert rel_l2(to_host(dU[k]), U[k] + B * phi) <= 1e-15


@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[3], CASES[9]], ids=_ids)
def test_fp32_sweeps_track_fp64(oracle, case):
    """The fast path (FP32 arithmetic, bit-level FP64<->FP32 conversion) stays
    within single-precision error of the oracle on every operator."""
    from pyranda_gb300.grid import Grid
    shape, per = case
    g = Grid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0), precision="fp32")
    o = oracle.OracleGrid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0))
    v = smooth_field(shape, seed=21)
    dv = to_dev(v, torch)
    for d in range(3):
        assert rel_l2(to_host(g.d1(d, dv)), o.apply(0, d, v)) <= 1e-5, ("d1", d)
        assert rel_l2(to_host(g.d8(d, dv)), o.apply(1, d, v)) <= 1e-5, ("d8", d)
        assert rel_l2(to_host(g.filter("spectral", dv, d)), o.apply(2, d, v)) <= 1e-6, ("sf", d)
        assert rel_l2(to_host(g.filter("gaussian", dv, d)), o.apply(3, d, v)) <= 1e-6, ("gf", d)
        # single-precision RHS of a second / fourth difference: cancellation of the field's smooth part
        assert rel_l2(to_host(g.d2(d, dv)), o.apply(4, d, v)) <= 1e-4, ("d2", d)
        assert rel_l2(to_host(g.d4(d, dv)), o.apply(5, d, v)) <= 1e-3, ("d4", d)
    c = g.field(torch.full(shape, 3.25, dtype=torch.float64, device="cuda"))
    assert torch.equal(g.filter("spectral", c), c)
    assert float(g.d1(0, c).abs().max()) == 0.0


def test_parcop_shim_numpy_roundtrip(oracle):
    """The f2py-named shim: setup/set_patch/ddx/sfilter/pring/... on numpy arrays."""
    from pyranda_gb300.parcop import parcop
    shape = (40, 24, 16)
    parcop.setup(0, 0, 0, 40, 24, 16, 1, 1, 1, 0, 0.0, 1.0, -0.5, 2.0, 0.25, 3.0,
                 "PERI", "PERI", "NONE", "NONE", "PERI", "PERI")
    parcop.setup(1, 0, 0, 16, 16, 16, 1, 1, 1, 0, 0.0, 1.0, 0.0, 1.0, 0.0, 1.0,
                 "NONE", "NONE", "NONE", "NONE", "NONE", "NONE")
    parcop.set_patch(0, 0)
    o = oracle.OracleGrid(shape, (True, False, True), (0.0, -0.5, 0.25), (1.0, 2.0, 3.0))
    v = smooth_field(shape, seed=31)
    assert rel_l2(parcop.ddx(v), o.ddx(v)) <= TOL
    assert rel_l2(parcop.ddy(v), o.ddy(v)) <= TOL
    assert rel_l2(parcop.dd8z(v), o.dd8(2, v)) <= TOL
    assert rel_l2(parcop.sfilter(v), o.sfilter(v)) <= TOL
    assert rel_l2(parcop.gfilter(v), o.gfilter(v)) <= TOL
    assert rel_l2(parcop.gfilterdir(v, 2), o.gfilterdir(v, 1)) <= TOL
    assert rel_l2(parcop.pring(v), o.ring(v, 2)) <= TOL
    assert rel_l2(parcop.dd4x(v), o.dd4(0, v)) <= TOL
    assert rel_l2(parcop.dd4y(v), o.dd4(1, v)) <= TOL
    assert rel_l2(parcop.plaplacian(v), o.laplacian(v)) <= TOL
    w = smooth_field(shape, seed=32)
    dx, dy, dz = parcop.divergencetensor(v, w, v, w, v, w, v, w, v)
    assert rel_l2(dy, o.div(w, v, w)) <= TOL
    gx, gy, gz = parcop.grads(v)
    assert rel_l2(gz, o.ddz(v)) <= TOL
    assert numpy.array_equal(parcop.xgrid(), o.mesh(0))
    assert numpy.array_equal(parcop.mesh_getgridlen(), o.mesh(6))
    with pytest.raises(ValueError):
        parcop.setup(2, 0, 0, 16, 16, 16, 1, 1, 1, 0, 0, 1, 0, 1, 0, 1, "SYMM", "NONE", "NONE", "NONE", "NONE", "NONE")


def test_diff_is_exact(grids):
    """The two-pass diffusion limit (FP32 candidates, FP64 quotients) equals the FP64 minimum bit for bit."""
    g, o = grids[CASES[0]]
    shape = CASES[0][0]
    r = numpy.random.default_rng(3)
    gl = min(o.spacing()[1])
    cases = [(1.0 + r.random(shape), r.random(shape) * 1e-3),
             (numpy.full(shape, 1.5), numpy.full(shape, 2e-3)),      # every point is a candidate
             (1.0 + r.random(shape), numpy.zeros(shape)),            # floored bulk
             (1.0 + r.random(shape), numpy.abs(r.standard_normal(shape)) * 1e5)]
    for rho, bulk in cases:
        ref = numpy.min(rho * gl * gl / numpy.maximum(1e-12, bulk))
        assert float(g.diff(to_dev(bulk, torch), to_dev(rho, torch))) == ref
    rho, bulk = cases[0]
    rho = rho.copy()
    rho[1, 2, 3] = float("nan")
    assert numpy.isnan(float(g.diff(to_dev(bulk, torch), to_dev(rho, torch))))


def test_bounded_wait_reports_timeout_and_context_survives(grids):
    """A device wait that never completes gives up, reports PG_ETIMEOUT, and the GPU keeps working."""
    from pyranda_gb300 import _lib
    g, o = grids[CASES[0]]
    st = ctypes.c_int(-1)
    assert g.lib.pg_device_status(g.h, ctypes.byref(st)) == 0 and st.value == 0
    assert g.lib.pg_wait_selftest(g.h, 50, None) == 0
    torch.cuda.synchronize()
    assert g.lib.pg_device_status(g.h, ctypes.byref(st)) == 0 and st.value == _lib.PG_ETIMEOUT
    assert g.lib.pg_device_status(g.h, ctypes.byref(st)) == 0 and st.value == 0   # read clears it
    shape = CASES[0][0]
    v = smooth_field(shape, 4)
    assert rel_l2(to_host(g.ddx(to_dev(v, torch))), o.ddx(v)) < 1e-12


@pytest.mark.parametrize("precision", ["fp32", "dense"])
@pytest.mark.parametrize("per", [(True, True, True), (False, True, False)], ids=["PPP", "NPN"])
def test_fp32_d8_rhs_is_exact(per, precision):
    """d8 and ring on the FP32 paths take their RHS in exact 64-bit fixed point.

    On a smooth field with a large mean the 8th difference cancels ~40 of the
    53 bits, so an FP32 RHS would be noise; with the exact RHS only the solve
    rounds -- the FP32 banded solve, or A^-1 in split TF32 on the tensor cores
    ('dense') -- and the result stays within 2e-6 relative L2 of the FP64 path.
    """
    from pyranda_gb300.grid import Grid
    shape = (64, 48, 40)
    x1, xn = (0.0, 0.0, 0.0), (1.0, 1.0, 1.0)
    g64 = Grid(shape, per, x1, xn, precision="fp64")
    g32 = Grid(shape, per, x1, xn, precision=precision)
    if precision == "dense":
        assert all(g32.dense_plan()[("d8", a)] for a in "xyz")
    x, y, z = (g64.mesh(d) for d in range(3))
    v = 5.0 + torch.sin(2 * math.pi * x) * torch.cos(2 * math.pi * y) + 0.5 * torch.sin(2 * math.pi * z + 0.3)
    for d in range(3):
        a, b = g64.d8(d, v), g32.d8(d, v)
        err = float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(a))
        assert err <= 2e-6, ("d8", d, err)
    a, b = g64.ring(v), g32.ring(v)
    assert float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(a)) <= 2e-6
    vs = [v, v * 0.5 - 1.0, torch.cos(2 * math.pi * y)]
    a, b = g64.ringv(*vs), g32.ringv(*vs)
    assert float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(a)) <= 2e-6


@pytest.mark.parametrize("precision", ["fp64", "fp32", "dense"])
@pytest.mark.parametrize("per", [(True, True, True), (False, True, False)], ids=["PPP", "NPN"])
def test_in_place_calls(per, precision):
    """in == out gives the out-of-place result bit for bit for every single-direction operator."""
    from pyranda_gb300.grid import Grid
    shape = (40, 24, 20)
    g = Grid(shape, per, (0.0, 0.0, 0.0), (1.0, 2.0, 3.0), precision=precision)
    v = to_dev(smooth_field(shape, seed=41), torch)
    ops = {"d1": lambda d, x, o: g.d1(d, x, out=o), "d2": lambda d, x, o: g.d2(d, x, out=o),
           "d4": lambda d, x, o: g.d4(d, x, out=o), "d8": lambda d, x, o: g.d8(d, x, out=o),
           "sf": lambda d, x, o: g.filter("spectral", x, d, out=o),
           "gf": lambda d, x, o: g.filter("gaussian", x, d, out=o)}
    for name, f in ops.items():
        for d in range(3):
            want = f(d, v, g.empty())
            w = g.field(v.clone())
            got = f(d, w, w)
            assert torch.equal(got, want), (name, d, float((got - want).abs().max()))
