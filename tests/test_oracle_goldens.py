"""The oracle against the reference's own golden scalars (tests/cases/*.py).

The oracle is a CPU restatement of parcop and of pyranda's Python driver; these
tests pin it to the values the reference test-suite records, with the
reference's tolerance (1e-4 relative, tests/run_tests.py:84): its golden
scalars and its 2-D profile baselines (tests/baselines/*.dat, copied into
tests/golden/ by tests/golden/make_golden.py).
"""
import json
import os

import numpy
import pytest

from tests import scripts

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_scalars.json")))["values"]
TOL = 1.0e-4


def _close(v, name):
    g = GOLD[name]["value"]
    assert abs(v - g) / abs(g) < TOL, (name, v, g)
    return abs(v - g) / abs(g)


def test_unit_test_3d(oracle):
    err = scripts.unit_test(oracle.OracleSim)
    # the restatement reproduces the reference value far inside its tolerance
    assert _close(err, "unit-test-3D") < 1e-9


@pytest.mark.parametrize("n", [50, 100, 200, 300, 400])
def test_advection_1d(oracle, n):
    err = scripts.advection_1d(oracle.OracleSim, n)
    _close(err, "advec-1d-%d" % n)


def test_taylor_green_32(oracle):
    enst = scripts.taylor_green(oracle.OracleSim, 32, tstop=0.1, timestep=lambda s: s.addPackage("Timestep"))
    assert _close(enst, "taylorgreen") < 1e-9


def test_shu_osher(oracle):
    cr = scripts.shu_osher(oracle.OracleSim, packages=lambda s: (s.addPackage("BC"), s.addPackage("Timestep")))
    assert _close(cr, "shu-osher-CR") < 1e-8


@pytest.mark.parametrize("n", [16, 32, 64, 128, 256])
def test_heat_1d(oracle, n):
    """tests/cases/testHeat1D.py heat1D-analytic-N: lap on a one-sided line
    (c10d2 closures) with bc.const ends keeps the linear steady state; the
    golden 0.0 is absolute (tests/testObj.py:47-53), the restatement gives 0."""
    err = scripts.heat_1d(oracle.OracleSim, n, lambda s: s.addPackage("BC"))
    assert err < TOL and GOLD["heat1D-analytic-%d" % n]["value"] == 0.0
    assert err < 1e-12, err


@pytest.mark.parametrize("n", [25, 50, 100, 200, 400])
def test_integration(oracle, n):
    """tests/cases/testIntegration.py integration-N: the LSRK(5,4) scheme and
    its stage times (pyranda.py:758-810) on ddt(a) = a, ddt(b) = cos(6 t).
    Measured 3e-9 (N = 25) to 7e-5 (N = 400, where the summed error, 5e-11,
    is at the rounding level of the 400 steps)."""
    _close(scripts.integration(oracle.OracleSim, n), "integration-%d" % n)


def test_dense_operator_matches_banded(oracle):
    """A . (A^-1 B v) = B v: the dense D = A^-1 B of the line evaluator
    reproduces the banded solve applied to a field (compact_basetype.f90:199-205)."""
    g = oracle.OracleGrid((24, 1, 1), (True, False, False), (0, 0, 0), (1, 0, 0))
    r = numpy.random.default_rng(3)
    v = numpy.asfortranarray(r.standard_normal((24, 1, 1)))
    for op in (0, 1, 2, 3):
        D = g.dense(op, 0)
        ref = g.apply(op, 0, v)[:, 0, 0]
        assert numpy.allclose(D @ v[:, 0, 0], ref, rtol=0, atol=1e-12 * max(1.0, abs(ref).max()))


def test_oracle_polynomial_exactness(oracle):
    """One-sided d1 closures differentiate x, x^2, x^3 exactly (examples/unit_test.py:67-80)."""
    n = 32
    g = oracle.OracleGrid((n, 1, 1), (False, False, False), (0, 0, 0), (1, 0, 0))
    x = g.mesh(0)
    for p in (1, 2, 3):
        d = g.ddx(x ** p)
        assert numpy.abs(d - p * x ** (p - 1)).max() < 1e-12


def test_second_and_fourth_derivatives(oracle):
    """c10d2 / e4d4 / LapS restated (stencils.f90:358-513, compact_r3.f90,
    operators.f90:513-526).  The reference's tests hold no values for them, so
    the restatement is checked on known answers: d2 of sin is spectrally
    accurate on a periodic line and exact on quadratics with the one-sided
    closures; e4d4 converges at 4th order; the Laplacian of a quadratic is its
    constant."""
    import math
    errs = []
    for n in (32, 64):
        g = oracle.OracleGrid((n, 8, 8), (True, True, True), (0.0, 0.0, 0.0),
                              (2 * math.pi * (n - 1) / n, 1.0, 1.0))
        x = g.mesh(0)
        v = numpy.asfortranarray(numpy.sin(x))
        assert numpy.abs(g.d2(0, v) + numpy.sin(x)).max() < 1e-11
        errs.append(numpy.abs(g.dd4(0, v) / (2 * math.pi / n) ** 4 - numpy.sin(x)).max())
    assert 14.0 < errs[0] / errs[1] < 18.0          # 4th order: error / 16 per halving
    g = oracle.OracleGrid((24, 12, 10), (False, False, True), (0.0, 0.0, 0.0), (1.0, 2.0, 0.9))
    x, y = g.mesh(0), g.mesh(1)
    q = numpy.asfortranarray(3.0 * x * x - 0.5 * y * y + x * y)
    assert numpy.abs(g.d2(0, q) - 6.0).max() < 1e-10
    assert numpy.abs(g.d2(1, q) + 1.0).max() < 1e-10
    assert numpy.abs(g.laplacian(q) - 5.0).max() < 1e-10
    assert numpy.abs(g.dd4(2, q)).max() == 0.0      # constant along the periodic z lines


def _bc_ts(s):
    s.addPackage("BC")
    s.addPackage("Timestep")


GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


@pytest.mark.parametrize("n", [64, 128])
def test_euler_2d_profile(oracle, n):
    """tests/cases/test2deuler.py euler-2d-N: the density profile of the 2-D
    Sod problem (examples/euler.py) against the reference's baseline file,
    by tests/testObj.py:checkProfile at the reference tolerance 1e-4.  The
    restatement reproduces the baseline to rounding."""
    x, rho = scripts.euler_2d(oracle.OracleSim, n, _bc_ts)
    base = numpy.loadtxt(os.path.join(GOLDEN_DIR, "euler-2d-%d.dat" % n))
    assert numpy.abs(x - base[0]).max() < 1e-12
    assert scripts.profile_error(os.path.join(GOLDEN_DIR, "euler-2d-%d.dat" % n), x, rho) < 1e-10


def test_kelvin_helmholtz_2d_profile(oracle):
    """tests/cases/test2deuler.py KH-2d-64: the density profile of
    examples/KH.py (AFLES terms, courant and diffusion time-step limits,
    grad) at t = 1.5 against the reference's baseline file."""
    x, rho = scripts.kelvin_helmholtz_2d(oracle.OracleSim, 64, _bc_ts)
    path = os.path.join(GOLDEN_DIR, "KelvinHelmholtzKH-2d-64.dat")
    assert numpy.abs(x - numpy.loadtxt(path)[0]).max() < 1e-12
    assert scripts.profile_error(path, x, rho) < 1e-10


def test_euler_rz_profile(oracle):
    """tests/cases/test2deuler.py euler-RZ-128 (examples/eulerRZ.py): cylindrical
    coordinates with a symmetry plane at the axis -- the cylindrical div / divT
    (operators.f90:55-64, :123-146), the volume-weighted filter (:876-883) and
    the symmetric / antisymmetric operator variants (stencils.f90:2390-2453)."""
    x, p = scripts.euler_rz(oracle.OracleSim, 128, lambda s: s.addPackage("BC"))
    path = os.path.join(GOLDEN_DIR, "euler-RZ-128.dat")
    assert numpy.abs(x - numpy.loadtxt(path)[0]).max() < 1e-12
    assert scripts.profile_error(path, x, p) < 1e-10


@pytest.mark.parametrize("name,run", [
    ("euler-SPH-1D", lambda o: scripts.euler_sph_1d(o.OracleSim, 128, _bc_ts)),
    ("euler-SPH-2D", lambda o: scripts.euler_sph_2d(o.OracleSim, 32, _bc_ts)),
    ("cylinder_omesh-2d-64", lambda o: scripts.cylinder_omesh(o.OracleSim, 64, _bc_ts)),
])
def test_spherical_and_curvilinear_profiles(oracle, name, run):
    """tests/cases/test2deuler.py euler-SPH-1D / euler-SPH-2D (spherical
    coordinates: mesh.f90:169-244, the spherical div / divT of
    operators.f90:64-76, :147-173, the filter of CellVol-weighted fields over
    the filtered cell volume :884-889, ring and the time-step limits on the
    d1 d2 d3 and GridLen fields) and tests/cases/testCylinder.py
    cylinder_omesh-2d-64 (a curvilinear O-mesh: the Jacobian of the supplied
    coordinates, mesh.f90:245-358, the metric div, the slip wall with the
    metric normal, pyrandaBC.py:198-264, and the curvilinear courant limit,
    pyrandaTimestep.py:45-56) against the reference's baseline files."""
    x, v = run(oracle)
    path = os.path.join(GOLDEN_DIR, name + ".dat")
    assert numpy.abs(x - numpy.loadtxt(path)[0]).max() < 1e-12
    assert scripts.profile_error(path, x, v) < 1e-10


def test_symmetry_plane_closures_known_answers(oracle):
    """SYMM ends (stencils.f90:2390-2453): with a symmetry plane half a
    spacing below the first point, the folded closures of a symmetric field
    cos(k (x - xs)) (xs the plane) give its derivative -k sin(k (x - xs)) to
    the interior scheme's accuracy at the end rows too, and the antisymmetric
    variant does the same for sin(k (x - xs)); the one-sided closures of the
    same grid are far less accurate at the ends."""
    n = 64
    dx = 1.0 / n
    x1, xn = 0.5 * dx, 1.0 - 0.5 * dx   # nodes at (i + 1/2) dx: the plane at x = 0
    k = 2.0 * numpy.pi * 1.5
    for sym, f, fp in ((1, numpy.cos, lambda t: -k * numpy.sin(k * t)), (-1, numpy.sin, lambda t: k * numpy.cos(k * t))):
        g = oracle.OracleGrid((n, 1, 1), (False, False, False), (x1, 0, 0), (xn, 0, 0),
                              bc=(("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")))
        x = g.mesh(0)
        v = f(k * x)
        d = g.apply_sym(0, 0, sym, v)
        err_end = numpy.abs(d[:6, 0, 0] - fp(x[:6, 0, 0])).max() / k
        assert err_end < 1e-7, (sym, err_end)
    # the one-sided rows at the same end, for comparison
    g1 = oracle.OracleGrid((n, 1, 1), (False, False, False), (x1, 0, 0), (xn, 0, 0))
    x = g1.mesh(0)
    e1 = numpy.abs(g1.apply(0, 0, numpy.cos(k * x))[:6, 0, 0] + k * numpy.sin(k * x[:6, 0, 0])).max() / k
    assert e1 > 1e-6


def test_cylindrical_divergence_known_answers(oracle):
    """Cylindrical div (operators.f90:55-64): div(r e_r) = 2 and
    div(r^2 e_r) = 3 r exactly up to the compact derivative's error on a
    polynomial, and the angular and axial terms of a field that does not vary
    in angle or along the axis vanish."""
    n = (48, 1, 16)
    g = oracle.OracleGrid(n, (False, True, True), (0.5, 0.0, 0.0), (1.5, 0.0, 1.0), coordsys=1,
                          bc=(("NONE", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")))
    r = g.mesh(0)
    zero = numpy.zeros(n)
    assert numpy.abs(g.div(r, zero, zero) - 2.0).max() < 1e-10
    assert numpy.abs(g.div(r * r, zero, zero) - 3.0 * r).max() < 1e-9


def test_curvilinear_affine_map_known_answers(oracle):
    """On an affine map x = M (A, B, C) + x0 the first-derivative operator is
    exact (one-sided closures included), so the metrics of mesh.f90:245-358
    are the inverse of M and det J is det M at every point; grad of a linear
    field c . x is c, and the divergence of x e_x + 2 y e_y is 3."""
    n = (20, 16, 12)
    M = numpy.array([[1.0, 0.3, 0.1], [-0.2, 0.9, 0.05], [0.1, -0.15, 1.2]])
    g = oracle.OracleGrid(n, (False, False, False), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), coordsys=3)
    A, B, C = numpy.meshgrid(*[numpy.linspace(0.0, 1.0, m) for m in n], indexing="ij")
    x = M[0, 0] * A + M[0, 1] * B + M[0, 2] * C + 0.5
    y = M[1, 0] * A + M[1, 1] * B + M[1, 2] * C - 0.25
    z = M[2, 0] * A + M[2, 1] * B + M[2, 2] * C
    g.set_mesh_x3(x, y, z, mesh_periodic=True)
    Minv = numpy.linalg.inv(M)
    for r in range(3):          # dA/dx dA/dy dA/dz, dB/.., dC/..
        for c in range(3):
            assert numpy.abs(g.mesh(11 + 3 * r + c) - Minv[r, c]).max() < 1e-12, (r, c)
    assert numpy.abs(g.mesh(10) - numpy.linalg.det(M)).max() < 1e-12
    cvec = (0.7, -1.3, 2.1)
    grads = g.grad(cvec[0] * x + cvec[1] * y + cvec[2] * z)
    for q in range(3):
        assert numpy.abs(grads[q] - cvec[q]).max() < 1e-10, q
    assert numpy.abs(g.div(x, 2.0 * y, numpy.zeros(n)) - 3.0).max() < 1e-10


def test_spherical_known_answers(oracle):
    """Spherical grids (mesh.f90:169-244, operators.f90:64-76, :197-201): the
    divergence of r e_r is 3, the gradient of r^2 is 2 r e_r (the one-sided
    closures are exact on polynomials of these degrees), and the mesh
    d3 = r sin(theta) dz."""
    n = (24, 10, 12)
    g = oracle.OracleGrid(n, (False, False, True), (0.5, 0.6, 0.0), (2.0, 2.4, 1.0), coordsys=2)
    r, th = g.mesh(0), g.mesh(1)
    z = numpy.zeros(n)
    assert numpy.abs(g.div(r, z, z) - 3.0).max() < 1e-10
    gr = g.grad(r * r)
    assert numpy.abs(gr[0] - 2.0 * r).max() < 1e-10
    assert numpy.abs(gr[1]).max() < 1e-12 and numpy.abs(gr[2]).max() < 1e-12
    dz = (1.0 - 0.0) / (n[2] - 1)
    assert numpy.abs(g.mesh(5) - r * numpy.sin(th) * dz).max() < 1e-14
