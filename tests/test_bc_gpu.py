"""pyrandaBC on device fields against the oracle's restatement
(pyranda/pyrandaBC.py): extrap, const, field, exit (BENO), symm, slip and
farfield, each applied to the same fields on both sides; the conditions
that only move and combine values agree bit for bit, farfield (sqrt, pow)
to 1e-13 relative."""
import numpy
import pytest

from tests.helpers import to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N = (16, 12, 10)
NAMES = ("rho", "u", "v", "w", "p")
EOM = "ddt(:rho:) = -ddx(:rho:*:u:)\n:v: = :u:\n:w: = :u:\n:p: = :rho:\n"


def _pair(oracle, seed):
    from pyranda_gb300 import pyrandaBC, pyrandaSim
    mesh = {"x1": [0.0, 0.0, 0.0], "xn": [1.0, 1.0, 1.0], "nn": list(N), "periodic": [False, False, False]}
    ss = pyrandaSim("bc", dict(mesh), silent=True)
    ss.addPackage(pyrandaBC(ss))
    ss.EOM(EOM)
    so = oracle.OracleSim("bc", dict(mesh))
    so.addPackage("BC")
    so.EOM(EOM)
    r = numpy.random.default_rng(seed)
    for k in NAMES:
        a = r.uniform(0.5, 2.0, N) * (1.0 if k in ("rho", "p") else r.choice([-1.0, 1.0], N))
        ss.variables[k].data.copy_(to_dev(a, torch))
        so.variables[k].data[...] = a
    return ss, so


def _compare(ss, so, tol=0.0):
    for k in NAMES:
        a, b = to_host(ss.variables[k].data), so.variables[k].data
        if tol == 0.0:
            assert numpy.array_equal(a, b), (k, numpy.abs(a - b).max())
        else:
            assert numpy.abs(a - b).max() <= tol * numpy.abs(b).max(), (k, numpy.abs(a - b).max())


def test_bc_conditions_match_oracle(oracle):
    ss, so = _pair(oracle, 1)
    bs, bo = ss.packages["BC"], so.packages["BC"]
    ends = ["x1", "xn", "y1", "yn", "z1", "zn"]
    steps = [
        lambda b: b.extrap(["rho", "p"], ends),
        lambda b: b.extrap(["u"], ["x1", "yn"], 1),
        lambda b: b.const(["w"], ["z1", "xn"], 0.25),
        lambda b: b.exitbc(["u", "v"], ends),
        lambda b: b.exitbc(["w"], ["x1", "yn"], True),
        lambda b: b.symm(["rho"], ["x1", "zn"]),
        lambda b: b.symm(["u"], ["y1"], True, 2),
        lambda b: b.slipbc([["u", "v", "w"]], ["x1", "xn", "y1", "yn"]),
    ]
    for k, f in enumerate(steps):
        f(bs)
        f(bo)
        _compare(ss, so)
    # field: the boundary plane of a given field
    r = numpy.random.default_rng(9).uniform(-1.0, 1.0, N)
    bs.applyBC("field", ["p"], ["x1", "yn"], to_dev(r, torch))
    bo.applyBC("field", ["p"], ["x1", "yn"], numpy.asfortranarray(r))
    _compare(ss, so)


@pytest.mark.parametrize("mach", [0.5, 1.6])
def test_farfield_matches_oracle(oracle, mach):
    ss, so = _pair(oracle, 2)
    g = 1.4
    # interior velocity of the given Mach number against the local sound speed, either sign
    for sim, put in ((ss, lambda k, a: ss.variables[k].data.copy_(to_dev(a, torch))),
                     (so, lambda k, a: so.variables[k].data.__setitem__(Ellipsis, a))):
        rho = to_host(ss.variables["rho"].data) if sim is ss else so.variables["rho"].data
        p = to_host(ss.variables["p"].data) if sim is ss else so.variables["p"].data
        c = numpy.sqrt(g * p / rho)
        r = numpy.random.default_rng(5)
        for k, f in (("u", 0.8), ("v", 0.5), ("w", 0.3)):
            put(k, mach * f * c * r.choice([-1.0, 1.0], N))
    ref = {"rho0": 1.1, "u0": 0.4, "v0": -0.2, "w0": 0.1, "p0": 0.9, "gamma": g,
           "rho": "rho", "u": "u", "v": "v", "w": "w", "p": "p"}
    ends = ["x1", "xn", "y1", "yn", "z1", "zn"]
    for b in (ss.packages["BC"], so.packages["BC"]):
        for d in ends:
            b.BCdata["farfield-properties-%s" % d] = ref
        b.farfieldbc(ends)
    _compare(ss, so, 1e-13)
