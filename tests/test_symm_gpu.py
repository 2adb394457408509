"""Symmetry planes (SYMM) and extended-data rows (XTND) against the oracle.

A non-periodic end may be a symmetry plane half a spacing outside its end
point (pyrandaMPI.py:101-131 maps a mesh's `symmetric` flags to SYMM).  Each
operator then has two variants (compact.f90:77-91): for fields symmetric about
the plane (the default of ddx / dd8x / filters) and for antisymmetric ones
(the bc = -1 argument, compact_operators.f90:30-35).  Their rows fold the
interior stencil about the plane (stencils.f90:2390-2453); antisymmetric rows
are evaluated as plain sums (compact_d1.f90:121-128, compact_r4.f90:108-117).
XTND takes the extended-data rows (stencils.f90:261-276 for d1, ...).  Bar:
relative L2 <= 1e-12 against the oracle in FP64, for every operator, both
variants, both line solves; the FP32 path within its own accuracy.
"""
import numpy
import pytest

from tests.helpers import rel_l2, smooth_field, to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1.0e-12
X1, XN = (0.0, -0.5, 0.25), (1.0, 2.0, 3.0)

CASES = [
    ((48, 20, 12), (False, True, False), (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "SYMM"))),
    ((40, 36, 10), (False, False, True), (("SYMM", "SYMM"), ("XTND", "SYMM"), ("NONE", "NONE"))),
    ((70, 9, 1), (False, False, False), (("XTND", "XTND"), ("SYMM", "XTND"), ("NONE", "NONE"))),
    ((8, 64, 3), (False, False, False), (("SYMM", "SYMM"), ("SYMM", "NONE"), ("NONE", "NONE"))),
    # equal line lengths with different ends: each direction keeps its own solve tables
    ((40, 12, 40), (False, False, False), (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "SYMM"))),
    ((64, 64, 64), (False, False, False), (("NONE", "NONE"), ("SYMM", "XTND"), ("SYMM", "SYMM"))),
]


def _ids(c):
    return "x".join(map(str, c[0])) + "-" + "-".join("".join(b[0] for b in e) for e in c[2])


@pytest.mark.parametrize("split", [False, True], ids=["line", "split"])
@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_symm_xtnd_operators_match_oracle(oracle, case, split):
    from pyranda_gb300.grid import Grid
    shape, per, bc = case
    g = Grid(shape, per, X1, XN, bc=bc, line_split=split)
    o = oracle.OracleGrid(shape, per, X1, XN, bc=bc)
    v = smooth_field(shape, seed=5)
    dv = to_dev(v, torch)
    bad = []
    for d in range(3):
        for sym in (1, -1):
            for op, f in ((0, lambda: g.d1(d, dv, sym=sym)), (1, lambda: g.d8(d, dv, sym=sym)),
                          (2, lambda: g.filter("spectral", dv, d, sym=(sym, sym, sym))),
                          (3, lambda: g.filter("gaussian", dv, d, sym=(sym, sym, sym)))):
                e = rel_l2(to_host(f()), o.apply_sym(op, d, sym, v))
                if not e <= TOL:
                    bad.append((op, d, sym, e))
        for op, f in ((4, lambda: g.d2(d, dv)), (5, lambda: g.d4(d, dv))):
            e = rel_l2(to_host(f()), o.apply(op, d, v))
            if not e <= TOL:
                bad.append((op, d, 1, e))
    w, q = smooth_field(shape, seed=6), smooth_field(shape, seed=7)
    e = rel_l2(to_host(g.div(dv, to_dev(w, torch), to_dev(q, torch))), o.div(v, w, q))
    if not e <= TOL:
        bad.append(("div", e))
    for sym in ((1, -1, 1), (-1, 1, -1)):
        e = rel_l2(to_host(g.filter("spectral", dv, sym=sym)), o.filter_sym(2, sym, v))
        if not e <= TOL:
            bad.append(("fbar", sym, e))
    e = rel_l2(to_host(g.ring(dv)), o.ring(v, 2))
    if not e <= TOL:
        bad.append(("ring", e))
    assert not bad, bad


def test_symm_fp32_and_dense_paths(oracle):
    """The fast paths on a grid with symmetry planes: FP32 banded and the autotuned path stay at
    FP32 accuracy for both variants (the antisymmetric one runs the FP32 banded sweep)."""
    from pyranda_gb300.grid import Grid
    shape, per = (64, 48, 40), (False, True, False)
    bc = (("SYMM", "NONE"), ("NONE", "NONE"), ("SYMM", "SYMM"))
    o = oracle.OracleGrid(shape, per, X1, XN, bc=bc)
    nx, ny, nz = shape
    x = numpy.arange(nx)[:, None, None] / nx
    y = numpy.arange(ny)[None, :, None] / ny
    z = numpy.arange(nz)[None, None, :] / nz
    v = numpy.asfortranarray(2.0 + numpy.cos(numpy.pi * x) * numpy.sin(2 * numpy.pi * y) * numpy.cos(numpy.pi * z)
                             + 0.0 * x)
    dv = to_dev(v, torch)
    for prec in ("fp32", "auto"):
        g = Grid(shape, per, X1, XN, bc=bc, precision=prec)
        for d in (0, 2):
            for sym in (1, -1):
                e = rel_l2(to_host(g.d1(d, dv, sym=sym)), o.apply_sym(0, d, sym, v))
                assert e <= 1e-5, (prec, d, sym, e)
                e = rel_l2(to_host(g.filter("spectral", dv, d, sym=(sym,) * 3)), o.apply_sym(2, d, sym, v))
                assert e <= 1e-6, (prec, "sf", d, sym, e)


def test_symm_fp32_split_paths(oracle):
    """SYMM / XTND ends on the FP32 split sweeps (lines of 64 and 96 points: the register-resident form,
    edge rows straight from global memory along y and z), both variants, at FP32 accuracy."""
    from pyranda_gb300.grid import Grid
    shape, per = (64, 96, 64), (False, False, False)
    bc = (("SYMM", "NONE"), ("XTND", "SYMM"), ("SYMM", "SYMM"))
    o = oracle.OracleGrid(shape, per, X1, XN, bc=bc)
    nx, ny, nz = shape
    x = numpy.arange(nx)[:, None, None] / nx
    y = numpy.arange(ny)[None, :, None] / ny
    z = numpy.arange(nz)[None, None, :] / nz
    v = numpy.asfortranarray(2.0 + numpy.cos(numpy.pi * x) * numpy.cos(numpy.pi * y) * numpy.cos(numpy.pi * z))
    dv = to_dev(v, torch)
    g = Grid(shape, per, X1, XN, bc=bc, precision="fp32", line_split=True)
    bad = []
    for d in range(3):
        for sym in (1, -1):
            e = rel_l2(to_host(g.d1(d, dv, sym=sym)), o.apply_sym(0, d, sym, v))
            bad += [("d1", d, sym, e)] if not e <= 1e-5 else []
            e = rel_l2(to_host(g.filter("spectral", dv, d, sym=(sym,) * 3)), o.apply_sym(2, d, sym, v))
            bad += [("sf", d, sym, e)] if not e <= 1e-6 else []
            e = rel_l2(to_host(g.d8(d, dv, sym=sym)), o.apply_sym(1, d, sym, v))
            bad += [("d8", d, sym, e)] if not e <= 1e-5 else []
    assert not bad, bad


@pytest.mark.parametrize("shape,bc", [((40, 1, 32), (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "NONE"))),
                                      ((36, 20, 24), (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")))])
def test_cylindrical_operators_match_oracle(oracle, shape, bc):
    """Cylindrical grids (x = radius, mesh.f90:213-225): div, divT, grad, the
    volume-weighted spectral filter and the mesh quantities against the oracle."""
    from pyranda_gb300.grid import Grid
    per = (False, True, True)
    x1, xn = (0.05, 0.0, 0.0), (1.0, 2.0 * numpy.pi * (shape[1] - 1) / shape[1], 1.5)
    g = Grid(shape, per, x1, xn, bc=bc, coordsys=1)
    o = oracle.OracleGrid(shape, per, x1, xn, bc=bc, coordsys=1)
    fs = [smooth_field(shape, seed=40 + i) for i in range(9)]
    ds = [to_dev(f, torch) for f in fs]
    bad = []
    e = rel_l2(to_host(g.div(ds[0], ds[1], ds[2])), o.div(fs[0], fs[1], fs[2]))
    bad += [("div", e)] if not e <= TOL else []
    for q, (a, b) in enumerate(zip(g.divT(*ds), o.divt(*fs))):
        e = rel_l2(to_host(a), b)
        bad += [("divT", q, e)] if not e <= TOL else []
    for q, (a, b) in enumerate(zip(g.grad(ds[0]), o.grad(fs[0]))):
        e = rel_l2(to_host(a), b)
        bad += [("grad", q, e)] if not e <= TOL else []
    e = rel_l2(to_host(g.filter("spectral", ds[3])), o.sfilter(fs[3]))
    bad += [("fbar", e)] if not e <= TOL else []
    for which in range(8):
        e = rel_l2(to_host(g.mesh(which)), o.mesh(which))
        bad += [("mesh", which, e)] if not e <= 1e-15 else []
    assert not bad, bad
