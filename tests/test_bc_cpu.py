"""The oracle's boundary conditions on hand-made planes (pyranda/pyrandaBC.py):
BENO (:510-521), symm (:748-788), slip (:267-465) and farfield (:566-745),
restated in oracle/oracle.py.  No GPU."""
import numpy
import pytest

from oracle import oracle


def _sim(per=(False, False, False), n=(16, 12, 10)):
    mesh = {"x1": [0.0, 0.0, 0.0], "xn": [1.0, 1.0, 1.0], "nn": list(n), "periodic": list(per)}
    s = oracle.OracleSim("bc", mesh)
    s.addPackage("BC")
    s.EOM("ddt(:rho:) = -ddx(:rho:*:u:)\n:v: = :u:\n:w: = :u:\n:p: = :rho:\n")
    r = numpy.random.default_rng(3)
    for k in ("rho", "u", "v", "w", "p"):
        s.variables[k].data[...] = r.uniform(0.5, 2.0, n)
    return s


def test_beno_known_answers():
    B = oracle._BC.BENO
    u1, u2, u3 = numpy.array([0.0, 1.0, 0.0, 0.0]), numpy.array([1.0, 2.0, 1.0, -1.0]), numpy.array([1.5, 3.0, 3.0, 0.5])
    # row 0: d1 = 1, d2 = 0.5 -> the smaller step; row 1: d2 = 0 -> no step;
    # row 2: d1 = 1, d2 = -1 (signs disagree) -> u1; row 3: d1 = -1, d2 = -2.5 -> u1 + d1
    numpy.testing.assert_array_equal(B(u1, u2, u3, False), [0.5, 1.0, 0.0, -1.0])
    # norm: limited to [min(0, u2), max(0, u2)]
    numpy.testing.assert_array_equal(B(numpy.array([3.0]), numpy.array([4.0]), numpy.array([4.5]), True), [3.5])
    # u1 = 3 kept (d1 d2 = 0), then limited to [min(0, u2), max(0, u2)] = [-1, 0]
    numpy.testing.assert_array_equal(B(numpy.array([3.0]), numpy.array([-1.0]), numpy.array([-5.0]), True), [0.0])


@pytest.mark.parametrize("anti", [False, True])
def test_symm_mirrors_the_next_planes(anti):
    s = _sim()
    a0 = s.variables["rho"].data.copy()
    s.packages["BC"].symm("rho", ["x1", "yn"], anti=anti, npts=4)
    a = s.variables["rho"].data
    m = -1.0 if anti else 1.0
    numpy.testing.assert_array_equal(a[0:4, :-4, :], m * a0[7:3:-1, :-4, :])
    numpy.testing.assert_array_equal(a[:, -4:, :], m * a[:, -5:-9:-1, :])
    numpy.testing.assert_array_equal(a[4:, :-4, :], a0[4:, :-4, :])


def test_slip_removes_the_normal_velocity():
    s = _sim()
    u0 = {k: s.variables[k].data.copy() for k in ("u", "v", "w")}
    s.packages["BC"].slipbc([["u", "v", "w"]], ["y1", "xn"])   # one velocity of three components
    d = s.variables
    assert numpy.all(d["v"].data[:, 0, :] == 0.0)          # y1: the normal is -y
    assert numpy.all(d["u"].data[-1, :, :] == 0.0)         # xn: the normal is +x
    # tangential components: second-order extrapolation (the speed cannot grow when the normal part is removed)
    numpy.testing.assert_allclose(d["w"].data[3:-1, 0, :], (2 * u0["w"][3:-1, 1, :] - u0["w"][3:-1, 2, :]))
    numpy.testing.assert_array_equal(d["u"].data[:, 3:-3, :][1:-1], u0["u"][:, 3:-3, :][1:-1])


def test_farfield_keeps_a_free_stream():
    s = _sim()
    g = 1.4
    ref = {"rho0": 1.2, "u0": 0.3, "v0": -0.1, "w0": 0.05, "p0": 1.0, "gamma": g,
           "rho": "rho", "u": "u", "v": "v", "w": "w", "p": "p"}
    bc = s.packages["BC"]
    for d in ("x1", "xn", "y1", "yn", "z1", "zn"):
        bc.BCdata["farfield-properties-%s" % d] = ref
    for k, v in (("rho", 1.2), ("u", 0.3), ("v", -0.1), ("w", 0.05), ("p", 1.0)):
        s.variables[k].data[...] = v
    bc.farfieldbc(["x1", "xn", "y1", "yn", "z1", "zn"])
    for k, v in (("rho", 1.2), ("u", 0.3), ("v", -0.1), ("w", 0.05), ("p", 1.0)):
        numpy.testing.assert_allclose(s.variables[k].data, v, rtol=1e-14, atol=1e-15)


def test_periodic_directions_are_not_touched():
    s = _sim(per=(True, False, False))
    a0 = s.variables["rho"].data.copy()
    s.packages["BC"].symm("rho", ["x1", "xn"])
    s.packages["BC"].exitbc("rho", ["x1"])
    numpy.testing.assert_array_equal(s.variables["rho"].data, a0)
