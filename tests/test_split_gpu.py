"""Split-line sweeps (the reduced-system line solve) against the oracle.

With pg_set_line_split(h, 1) every banded sweep cuts its lines into segments
of 32 points, one thread per segment, joined by the reduced system of the
segments' end unknowns (the reference's parallel solver across ranks,
compact_basetype.f90:171-197, pentadiagonal.f90:160-626,
compact_d1.f90:242-337).  Bars:
  FP64: relative L2 <= 1e-12 against the oracle for every operator, on
        periodic and one-sided lines, ragged sizes, null directions and lines
        longer than the dense path's 1024 points;
  FP32: the FP32 arithmetic's level, <= 2e-6 against the oracle on smooth
        fields, the same order as the one-thread-per-line FP32 sweeps;
  in-place calls equal out-of-place calls bit for bit; an ensemble equals
  its members run alone bit for bit.
"""
import numpy
import pytest

from tests.helpers import rel_l2, smooth_field, to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1.0e-12

CASES = [
    ((32, 32, 32), (True, True, True)),
    ((40, 24, 16), (True, False, True)),
    ((24, 40, 12), (False, True, False)),
    ((9, 13, 11), (False, False, False)),
    ((8, 8, 8), (True, True, True)),
    ((65, 1, 3), (False, False, False)),
    ((64, 64, 1), (True, False, False)),
    ((48, 3, 10), (True, True, True)),
    ((300, 3, 2), (True, False, False)),
    ((100, 70, 1), (False, True, False)),
    ((2000, 2, 1), (True, False, False)),     # beyond the dense path's 1024 points
    ((8, 1, 4100), (False, False, False)),    # a long z line: 128 segments
]


def _ids(c):
    return "x".join(map(str, c[0])) + "-" + "".join("P" if p else "N" for p in c[1])


def _grid(shape, per, precision="fp64"):
    from pyranda_gb300.grid import Grid
    return Grid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0), precision=precision, line_split=True)


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_split_fp64_operators_match_oracle(oracle, case):
    shape, per = case
    g = _grid(shape, per)
    o = oracle.OracleGrid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0))
    v = smooth_field(shape, seed=11)
    dv = to_dev(v, torch)
    bad = []
    for d in range(3):
        for name, f, ref in (("d1", lambda: g.d1(d, dv), lambda: o.apply(0, d, v)),
                             ("d8", lambda: g.d8(d, dv), lambda: o.apply(1, d, v)),
                             ("sf", lambda: g.filter("spectral", dv, d), lambda: o.apply(2, d, v)),
                             ("gf", lambda: g.filter("gaussian", dv, d), lambda: o.apply(3, d, v)),
                             ("d2", lambda: g.d2(d, dv), lambda: o.apply(4, d, v)),
                             ("d4", lambda: g.d4(d, dv), lambda: o.apply(5, d, v))):
            e = rel_l2(to_host(f()), ref())
            if not e <= TOL:
                bad.append((name, d, e))
    w, q = smooth_field(shape, seed=12), smooth_field(shape, seed=13)
    dw, dq = to_dev(w, torch), to_dev(q, torch)
    comp = [("fbar", to_host(g.filter("spectral", dv)), o.sfilter(v)),
            ("gbar", to_host(g.filter("gaussian", dv)), o.gfilter(v)),
            ("ring", to_host(g.ring(dv)), o.ring(v, 2)),
            ("ringv", to_host(g.ringv(dv, dw, dq)), o.ringv(v, w, q, 1)),
            ("div", to_host(g.div(dv, dw, dq)), o.div(v, w, q)),
            ("lap", to_host(g.laplacian(dv)), o.laplacian(v))]
    for name, a, b in comp:
        e = rel_l2(a, b)
        if not e <= TOL:
            bad.append((name, e))
    gx, gy, gz = g.grad(dv)
    for a, b in zip((gx, gy, gz), o.grad(v)):
        e = rel_l2(to_host(a), b)
        if not e <= TOL:
            bad.append(("grad", e))
    assert not bad, bad


def _smooth(shape, seed):
    r = numpy.random.default_rng(seed)
    nx, ny, nz = shape
    x = numpy.arange(nx)[:, None, None] / nx
    y = numpy.arange(ny)[None, :, None] / ny
    z = numpy.arange(nz)[None, None, :] / nz
    f = numpy.zeros(shape)
    for _ in range(4):
        a, b, c = r.integers(0, 3, 3)
        f = f + r.standard_normal() * numpy.cos(2 * numpy.pi * (a * x + b * y + c * z) + r.uniform(0, 6))
    return numpy.asfortranarray(f + 2.0)


@pytest.mark.parametrize("case", [((64, 48, 40), (True, False, True)), ((256, 16, 24), (True, True, True)),
                                  ((40, 520, 3), (False, False, True)), ((64, 96, 32), (True, False, True)),
                                  ((32, 64, 128), (False, False, False)), ((96, 32, 64), (False, True, True))],
                         ids=_ids)
def test_split_fp32_matches_oracle(oracle, case):
    """FP32 arithmetic (exact fixed-point RHS for d8): the same error level as the FP32 one-thread-per-line sweeps.
    Lines whose length is a multiple of 32 take the register-resident form (y and z straight from global
    memory, x through a staged tile); the others the tile form."""
    from pyranda_gb300.grid import Grid
    shape, per = case
    g = _grid(shape, per, "fp32")
    g32 = Grid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0), precision="fp32")
    o = oracle.OracleGrid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0))
    v = _smooth(shape, 5)
    dv = to_dev(v, torch)
    bad = []
    for d in range(3):
        for op, name, f in ((0, "d1", lambda gg: gg.d1(d, dv)), (1, "d8", lambda gg: gg.d8(d, dv)),
                            (2, "sf", lambda gg: gg.filter("spectral", dv, d)),
                            (3, "gf", lambda gg: gg.filter("gaussian", dv, d))):
            ref = o.apply(op, d, v)
            es, e32 = rel_l2(to_host(f(g)), ref), rel_l2(to_host(f(g32)), ref)
            print("%s %d split %.2e  one-thread-per-line %.2e" % (name, d, es, e32))
            if not es <= max(2e-6, 4 * e32):
                bad.append((name, d, es, e32))
    assert not bad, bad


def test_split_in_place_equals_out_of_place():
    shape, per = (96, 40, 33), (True, False, True)
    for prec in ("fp64", "fp32"):
        g = _grid(shape, per, prec)
        v = to_dev(smooth_field(shape, seed=21), torch)
        for d in range(3):
            for f in (lambda x, out=None: g.d1(d, x, out=out), lambda x, out=None: g.filter("spectral", x, d, out=out),
                      lambda x, out=None: g.filter("gaussian", x, d, out=out), lambda x, out=None: g.d8(d, x, out=out)):
                ref = f(v)
                a = v.clone()
                f(a, out=a)
                assert torch.equal(a, ref), (prec, d)


def test_split_ensemble_equals_members():
    from pyranda_gb300.ensemble import EnsembleGrid
    from pyranda_gb300.grid import Grid
    spec = [((n, n, 1), (True, False, False), (0, 0, 0), ((n - 1) / n, 1.0, 1.0)) for n in (128, 192, 64, 128)]
    for prec in ("fp64", "fp32"):
        ens = EnsembleGrid(spec, precision=prec)
        ens.set_line_split(True)
        singles = [Grid(*s, precision=prec, line_split=True) for s in spec]
        host = [_smooth(s[0], 30 + i) for i, s in enumerate(spec)]
        v = ens.from_members(host)
        for d in (0, 1):
            for fe, fs in ((lambda x: ens.d1(d, x), lambda gg, x: gg.d1(d, x)),
                           (lambda x: ens.filter("spectral", x, d), lambda gg, x: gg.filter("spectral", x, d)),
                           (lambda x: ens.d8(d, x), lambda gg, x: gg.d8(d, x))):
                e = fe(v)
                for m, g in enumerate(singles):
                    assert torch.equal(ens.member_view(e, m), fs(g, to_dev(host[m], torch))), (prec, d, m)


def test_split_tgv_step_matches_oracle(oracle):
    """A Taylor-Green RK step through pyrandaSim with split-line sweeps (FP64) against the oracle."""
    from pyranda_gb300 import pyrandaSim, pyrandaTimestep, problems
    ss = problems.build_tgv(pyrandaSim, 48, lambda s: s.addPackage(pyrandaTimestep(s)), ns=True, silent=True)
    ss.grid.set_line_split(True)
    so = problems.build_tgv(oracle.OracleSim, 48, lambda s: s.addPackage("Timestep"), ns=True)
    for s in (ss, so):
        s.rk4(0.0, s.variables["dt"].data * 0.5)
    for name in ("rho", "rhou", "rhov", "Et", "p"):
        e = rel_l2(to_host(ss.variables[name].data), so.variables[name].data)
        assert e <= 1e-12, (name, e)


def test_split_fp32_differences_keep_a_large_mean(oracle):
    """A field with a large mean and a small variation (like the Taylor-Green
    pressure): the FP32 split sweeps take every RHS difference from FP32
    hi + lo pairs of the FP64 values, so d1 and the compact filter keep the
    FP32 accuracy of the result itself; rounding the values to FP32 first
    (the one-thread-per-line FP32 sweeps) loses log2(mean / variation) bits."""
    from pyranda_gb300.grid import Grid
    shape, per = (128, 64, 32), (True, True, False)
    g = _grid(shape, per, "fp32")
    g32 = Grid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0), precision="fp32")
    o = oracle.OracleGrid(shape, per, (0.0, -0.5, 0.25), (1.0, 2.0, 3.0))
    v = numpy.asfortranarray(71.4 + 0.1 * _smooth(shape, 9))
    dv = to_dev(v, torch)
    for d in range(3):
        ref = o.apply(0, d, v)
        es, e32 = rel_l2(to_host(g.d1(d, dv)), ref), rel_l2(to_host(g32.d1(d, dv)), ref)
        print("d1 %d: split %.2e  one-thread-per-line %.2e" % (d, es, e32))
        assert es <= 2e-6, (d, es)
        # the filtered field, measured against the size of the variation (not of the mean)
        ref = o.apply(2, d, v)
        es = numpy.linalg.norm((to_host(g.filter("spectral", dv, d)) - ref).ravel()) / numpy.linalg.norm(
            (v - v.mean()).ravel())
        assert es <= 1e-6, ("sf", d, es)


def test_autotuned_plan_is_cached_and_reapplied(tmp_path, monkeypatch):
    """The autotuner's plan is stored under the grid, GPU and library build;
    a second autotuned grid of the same shape applies it without timing
    (pg_set_sweep_plan) and computes the same bits."""
    from pyranda_gb300 import grid as G
    monkeypatch.setattr(G, "PLAN_CACHE", str(tmp_path / "plans.json"))
    shape, per = (64, 96, 32), (True, False, True)
    a = G.Grid(shape, per, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), precision="auto")
    b = G.Grid(shape, per, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), precision="auto")
    assert not a.plan_from_cache and b.plan_from_cache
    assert a.sweep_plan() == b.sweep_plan()
    v = to_dev(_smooth(shape, 3), torch)
    for d in range(3):
        assert torch.equal(a.d1(d, v), b.d1(d, v))
        assert torch.equal(a.filter("spectral", v, d), b.filter("spectral", v, d))
        assert torch.equal(a.d8(d, v), b.d8(d, v))
