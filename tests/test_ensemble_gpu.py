"""Ensembles of uneven grids against single grids and the oracle.

An ensemble runs the same per-line arithmetic as a single grid, only with
every member's lines in one launch, so each member's result must equal the
single-grid result bit for bit (operators, max/min reductions, time steps,
whole RK steps).  Sums are compared to a tolerance, since the per-member sum
adds in another order.  One Kelvin-Helmholtz member is also checked against
the oracle's numpy restatement of pyrandaSim.
"""
import numpy
import pytest

from tests.helpers import rel_l2, smooth_field, to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

# members share periodicity and null directions, not sizes
MEMBERS_3D = [((24, 16, 12), (True, False, True)), ((16, 20, 8), (True, False, True)),
              ((32, 8, 10), (True, False, True))]
MEMBERS_2D = [((40, 32, 1), (True, False, False)), ((64, 48, 1), (True, False, False)),
              ((32, 64, 1), (True, False, False)), ((48, 40, 1), (True, False, False))]


def _spec(members):
    out = []
    for i, (n, per) in enumerate(members):
        xn = [(1.0 + 0.25 * i) * (n[d] - 1) / n[d] if per[d] else 1.0 + 0.5 * d for d in range(3)]
        out.append((n, per, (0.0, 0.1 * i, 0.0), xn))
    return out


def _pair(members, precision="fp64"):
    from pyranda_gb300.ensemble import EnsembleGrid
    from pyranda_gb300.grid import Grid
    spec = _spec(members)
    ens = EnsembleGrid(spec, precision=precision)
    singles = [Grid(n, per, x1, xn, precision=precision) for (n, per, x1, xn) in spec]
    return ens, singles


def _fields(members, seed):
    return [smooth_field(n, seed + 7 * i) for i, (n, _) in enumerate(members)]


def _same(ens, singles, flat, outs, what):
    for m, g in enumerate(singles):
        a = ens.member_view(flat, m)
        b = outs[m]
        assert torch.equal(a, b), (what, m, float((a - b).abs().max()))


@pytest.mark.parametrize("members", [MEMBERS_3D, MEMBERS_2D], ids=["3d", "2d"])
@pytest.mark.parametrize("precision", ["fp64", "fp32", "dense"])
def test_operators_match_single_grids(members, precision):
    if precision == "dense" and members is MEMBERS_3D:
        pytest.skip("a member direction of 8 points has no dense form, so the ensemble sweeps that direction "
                    "banded while its other members alone would not")
    ens, singles = _pair(members, precision)
    host = _fields(members, 3)
    v = ens.from_members(host)
    vs = [to_dev(h, torch) for h in host]
    w = ens.from_members(_fields(members, 11))
    ws = [ens.member_view(w, m) for m in range(len(members))]
    for d in range(3):
        _same(ens, singles, ens.d1(d, v), [g.d1(d, vs[m]) for m, g in enumerate(singles)], "d1 %d" % d)
        _same(ens, singles, ens.d8(d, v), [g.d8(d, vs[m]) for m, g in enumerate(singles)], "d8 %d" % d)
        _same(ens, singles, ens.d2(d, v), [g.d2(d, vs[m]) for m, g in enumerate(singles)], "d2 %d" % d)
        _same(ens, singles, ens.d4(d, v), [g.d4(d, vs[m]) for m, g in enumerate(singles)], "d4 %d" % d)
    for kind in ("spectral", "gaussian"):
        for d in (0, 1, 2, 3):
            _same(ens, singles, ens.filter(kind, v, d),
                  [g.filter(kind, vs[m], d) for m, g in enumerate(singles)], "%s %d" % (kind, d))
    _same(ens, singles, ens.ring(v), [g.ring(vs[m]) for m, g in enumerate(singles)], "ring")
    _same(ens, singles, ens.laplacian(v), [g.laplacian(vs[m]) for m, g in enumerate(singles)], "laplacian")
    _same(ens, singles, ens.ringv(v, w, v), [g.ringv(vs[m], ws[m], vs[m]) for m, g in enumerate(singles)],
          "ringv")
    ge = ens.grad(v)
    gs = [g.grad(vs[m]) for m, g in enumerate(singles)]
    for c in range(3):
        _same(ens, singles, ge[c], [x[c] for x in gs], "grad %d" % c)
    _same(ens, singles, ens.div(v, w, v), [g.div(vs[m], ws[m], vs[m]) for m, g in enumerate(singles)], "div")
    for which in range(8):
        _same(ens, singles, ens.mesh(which), [g.mesh(which) for g in singles], "mesh %d" % which)


def test_operators_match_oracle(oracle):
    """Member by member against the CPU restatement (relative L2 <= 1e-12)."""
    ens, _ = _pair(MEMBERS_3D)
    spec = _spec(MEMBERS_3D)
    host = _fields(MEMBERS_3D, 5)
    v = ens.from_members(host)
    dx, fb = ens.ddx(v), ens.filter("spectral", v)
    rg = ens.ring(v)
    for m, (n, per, x1, xn) in enumerate(spec):
        og = oracle.OracleGrid(n, per, x1, xn)
        assert rel_l2(to_host(ens.member_view(dx, m)), og.ddx(host[m])) < 1e-12
        assert rel_l2(to_host(ens.member_view(fb, m)), og.sfilter(host[m])) < 1e-12
        assert rel_l2(to_host(ens.member_view(rg, m)), og.ring(host[m], 2)) < 1e-12


def test_reductions_and_time_steps():
    ens, singles = _pair(MEMBERS_2D)
    host = _fields(MEMBERS_2D, 21)
    v = ens.from_members(host)
    c = ens.from_members([numpy.abs(h) + 1.0 for h in host])
    w = ens.from_members(_fields(MEMBERS_2D, 4))
    vs = [to_dev(h, torch) for h in host]
    cs = [to_dev(numpy.abs(h) + 1.0, torch) for h in host]
    wsx = [to_dev(h, torch) for h in _fields(MEMBERS_2D, 4)]
    for op in (1, 2):   # max, min: exact in any order
        per = ens.reduce_members(op, v)
        ref = torch.stack([g.reduce(op, vs[m]) for m, g in enumerate(singles)])
        assert torch.equal(per, ref), op
        f = ens.reduce(op, v)
        assert torch.equal(ens.member_values(f), ref)
        assert torch.equal(f, ens.member_field(ref))
    s = ens.reduce_members(0, v)
    ref = torch.stack([t.sum() for t in vs])
    assert float(((s - ref).abs() / ref.abs().clamp(min=1e-30)).max()) < 1e-12
    dtc = ens.courant(v, w, 0.0, c)
    ref = torch.stack([g.courant(vs[m], wsx[m], 0.0, cs[m]) for m, g in enumerate(singles)])
    assert torch.equal(ens.member_values(dtc), ref)
    assert torch.equal(dtc, ens.member_field(ref))
    dtd = ens.diff(c, w.abs() + 0.5)
    ref = torch.stack([g.diff(cs[m], wsx[m].abs() + 0.5) for m, g in enumerate(singles)])
    assert torch.equal(dtd, ens.member_field(ref))


def test_rk_stage_with_dt_field():
    ens, _ = _pair(MEMBERS_2D)
    r = torch.Generator(device="cuda").manual_seed(1)
    U = [torch.rand(ens.npts, dtype=torch.float64, device="cuda", generator=r) for _ in range(3)]
    P = [torch.rand(ens.npts, dtype=torch.float64, device="cuda", generator=r) for _ in range(3)]
    F = [torch.rand(ens.npts, dtype=torch.float64, device="cuda", generator=r) for _ in range(3)]
    dt = ens.member_field(torch.linspace(1e-3, 4e-3, ens.m, dtype=torch.float64))
    A, B = -0.48, 0.74
    U0 = [u.clone() for u in U]
    P0 = [p.clone() for p in P]
    ens.rk_stage(U, P, F, dt, A, B)
    for i in range(3):
        p = A * P0[i] + dt * F[i]
        assert float((P[i] - p).abs().max()) <= 1e-15
        assert float((U[i] - (U0[i] + B * p)).abs().max()) <= 1e-15


def _packages(ss):
    from pyranda_gb300 import pyrandaBC, pyrandaTimestep
    ss.addPackage(pyrandaTimestep(ss))
    ss.addPackage(pyrandaBC(ss))


KH_VARS = ("rho", "rhou", "rhov", "Et", "p", "beta", "mu", "kappa")


def _kh_run_single(n, steps, precision, oracle_sim=None):
    from pyranda_gb300 import pyrandaSim
    from pyranda_gb300.problems import build_kh
    ss = build_kh(pyrandaSim, n, _packages, silent=True, precision=precision)
    t, dt = 0.0, ss.variables["dt"].data.clone()
    for _ in range(steps):
        t = ss.rk4(t, dt)
        dt = torch.minimum(ss.variables["dt"].data, 1.1 * dt)
    return ss


def _kh_run_ensemble(sizes, steps, precision, graphs=False):
    from pyranda_gb300.ensemble import pyrandaEnsemble
    from pyranda_gb300.problems import build_kh_ensemble
    ens = build_kh_ensemble(pyrandaEnsemble, sizes, _packages, silent=True, precision=precision)
    if graphs:
        ens.use_graphs(True)
    t, dt = 0.0, ens.variables["dt"].data.clone()
    for _ in range(steps):
        t = ens.rk4(t, dt)
        dt = torch.minimum(ens.variables["dt"].data, 1.1 * dt)
    return ens, t


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_kh_ensemble_equals_single_sims(precision):
    sizes = [32, 48, 40]
    ens, t = _kh_run_ensemble(sizes, 4, precision)
    for m, n in enumerate(sizes):
        ss = _kh_run_single(n, 4, precision)
        for name in KH_VARS:
            a = ens.grid.member_view(ens.variables[name].data, m)
            b = ss.variables[name].data
            assert torch.equal(a, b.expand_as(a)), (precision, n, name, float((a - b).abs().max()))
        assert float(t[m]) == pytest.approx(float(ss.time), rel=0, abs=0)


def test_kh_ensemble_graphs_equal_eager():
    sizes = [40, 32, 48, 32]
    e1, t1 = _kh_run_ensemble(sizes, 5, "fp32")
    e2, t2 = _kh_run_ensemble(sizes, 5, "fp32", graphs=True)
    for name in KH_VARS:
        assert torch.equal(e1.variables[name].data, e2.variables[name].data), name
    assert torch.equal(t1, t2)


def test_kh_ensemble_member_matches_oracle(oracle):
    """A 32^2 member after 3 steps against the numpy restatement of pyrandaSim."""
    from pyranda_gb300.problems import build_kh
    sizes = [32, 40]
    ens, _ = _kh_run_ensemble(sizes, 3, "fp64")

    def pk(ss):
        ss.addPackage("Timestep")
        ss.addPackage("BC")

    os_ = build_kh(oracle.OracleSim, 32, pk)
    t, dt = 0.0, float(numpy.asarray(os_.variables["dt"].data))
    for _ in range(3):
        t = os_.rk4(t, dt)
        dt = min(float(numpy.asarray(os_.variables["dt"].data)), 1.1 * dt)
    for name in ("rho", "rhou", "rhov", "Et"):
        a = to_host(ens.grid.member_view(ens.variables[name].data, 0))
        assert rel_l2(a, os_.variables[name].data) < 1e-11, name
