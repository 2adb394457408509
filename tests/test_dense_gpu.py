"""Dense split-TF32 tensor-core operators against the oracle and the FP64 banded path.

precision='dense' applies d1, d8 and the compact filter as dense n x n
matrices (D = A^-1 B built from the banded operator itself) with three TF32
MMAs per product and FP32 accumulation; the Gaussian filter and any
direction outside 16..1024 points use the FP32 banded sweeps.  Bounds, as
relative L2 against the oracle's result on the same input and against the
FP64 banded GPU result (FP32-level arithmetic; the FP32 banded path's error
on the same input is printed beside it):
  d1, d8, ring, div: <= 1e-5;   compact and Gaussian filters: <= 2e-6;
  the library status word stays PG_OK (no bounded wait gave up).
"""
import numpy
import pytest

from tests.helpers import rel_l2, smooth_field, to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

CASES = [
    ((64, 64, 64), (True, True, True)),
    ((48, 40, 32), (False, True, False)),
    ((300, 20, 1), (True, False, False)),     # x lines of two MMA column tiles, K padding
    ((24, 272, 2), (False, False, False)),    # y lines of three M tiles
    ((17, 9, 260), (True, True, False)),      # z lines of three M tiles; y has 9 < 16 points: FP32 banded
]


def _grids(n, per, fp32=False):
    from pyranda_gb300.grid import Grid
    xn = [1.0 + d for d in range(3)]
    gs = (Grid(n, per, (0, 0, 0), xn, precision="fp64"), Grid(n, per, (0, 0, 0), xn, precision="dense"))
    if fp32:
        gs = gs + (Grid(n, per, (0, 0, 0), xn, precision="fp32"),)
    return gs


D_TOL, F_TOL = 1e-5, 2e-6


def _status(g):
    import ctypes
    s = ctypes.c_int(-1)
    g.lib.pg_device_status(g.h, ctypes.byref(s))
    return s.value


def _smooth(n, seed):
    """A smooth seeded field (a few low modes) so the operators are well resolved."""
    r = numpy.random.default_rng(seed)
    nx, ny, nz = n
    x = numpy.arange(nx)[:, None, None] / nx
    y = numpy.arange(ny)[None, :, None] / ny
    z = numpy.arange(nz)[None, None, :] / nz
    f = numpy.zeros(n)
    for _ in range(4):
        a, b, c = r.integers(0, 3, 3)
        f = f + r.standard_normal() * numpy.cos(2 * numpy.pi * (a * x + b * y + c * z) + r.uniform(0, 6))
    return numpy.asfortranarray(f + 2.0)


@pytest.mark.parametrize("n,per", CASES)
def test_dense_operators_match_oracle(oracle, n, per):
    """Each dense operator against the oracle (the CPU restatement of parcop)
    on the same input, and, on a second line, against the FP64 banded GPU
    path; the FP32 banded path's error against the oracle is printed beside."""
    g64, gd, g32 = _grids(n, per, fp32=True)
    og = oracle.OracleGrid(n, per, (0, 0, 0), [1.0 + d for d in range(3)])
    hv, hrough, hw = _smooth(n, 1), smooth_field(n, 2), _smooth(n, 3)
    v, rough, w = to_dev(hv, torch), to_dev(hrough, torch), to_dev(hw, torch)
    cases = []
    for d in range(3):
        if n[d] == 1:
            continue
        cases += [("d1 %d" % d, lambda g, d=d: g.d1(d, v), lambda d=d: og.apply(0, d, hv), D_TOL),
                  ("d8 %d" % d, lambda g, d=d: g.d8(d, rough), lambda d=d: og.dd8(d, hrough), D_TOL),
                  ("sf %d" % d, lambda g, d=d: g.filter("spectral", v, d), lambda d=d: og.sfilterdir(hv, d), F_TOL),
                  ("gf %d" % d, lambda g, d=d: g.filter("gaussian", v, d), lambda d=d: og.gfilterdir(hv, d), F_TOL)]
    cases += [("fbar", lambda g: g.filter("spectral", v), lambda: og.sfilter(hv), F_TOL),
              ("ring", lambda g: g.ring(rough), lambda: og.ring(hrough, 2), D_TOL),
              ("div", lambda g: g.div(v, w, v), lambda: og.div(hv, hw, hv), D_TOL)]
    bad = []
    for name, f, fo, tol in cases:
        ref = fo()
        dense = to_host(f(gd))
        ed, e32 = rel_l2(dense, ref), rel_l2(to_host(f(g32)), ref)
        ed64 = rel_l2(dense, to_host(f(g64)))
        print("%-6s dense vs oracle %.2e (vs FP64 banded %.2e)  fp32-banded vs oracle %.2e  (tol %.0e)"
              % (name, ed, ed64, e32, tol))
        if not (ed < tol and ed64 < tol):
            bad.append((name, ed, ed64, tol))
    torch.cuda.synchronize()
    assert _status(gd) == 0
    assert not bad, bad


def test_dense_in_place():
    """out may alias in (the tiles of one line then read a private copy)."""
    n, per = (300, 20, 1), (True, False, False)
    g64, gd = _grids(n, per)
    v = to_dev(_smooth(n, 4), torch)
    ref = g64.filter("spectral", v, 0)
    a = v.clone()
    gd.filter("spectral", a, 0, out=a)
    assert rel_l2(to_host(a), to_host(ref)) < F_TOL
    b = v.clone()
    gd.d1(0, b, out=b)
    assert rel_l2(to_host(b), to_host(g64.d1(0, v))) < D_TOL


def test_dense_constant_is_exact():
    """Difference-form filters annihilate constants: with the FP64 add-back the result is v exactly."""
    n, per = (64, 48, 32), (True, False, True)
    _, gd = _grids(n, per)
    c = torch.full((32, 48, 64), 3.25, dtype=torch.float64, device="cuda").permute(2, 1, 0)
    out = gd.filter("spectral", c)
    assert float((out - 3.25).abs().max()) == 0.0


def test_dense_ensemble_matches_members():
    from pyranda_gb300.ensemble import EnsembleGrid
    from pyranda_gb300.grid import Grid
    spec = [((n, n, 1), (True, False, False), (0, 0, 0), ((n - 1) / n, 1.0, 1.0)) for n in (128, 192, 256, 128)]
    ens = EnsembleGrid(spec, precision="dense")
    singles = [Grid(*s, precision="dense") for s in spec]
    ref64 = [Grid(*s, precision="fp64") for s in spec]
    host = [_smooth(s[0], 10 + i) for i, s in enumerate(spec)]
    v = ens.from_members(host)
    for d in (0, 1):
        e = ens.d1(d, v)
        for m, g in enumerate(singles):
            vm = to_dev(host[m], torch)
            assert torch.equal(ens.member_view(e, m), g.d1(d, vm))
            assert rel_l2(to_host(ens.member_view(e, m)), to_host(ref64[m].d1(d, vm))) < D_TOL
    f = ens.filter("spectral", v)
    for m, g in enumerate(singles):
        assert torch.equal(ens.member_view(f, m), g.filter("spectral", to_dev(host[m], torch)))
