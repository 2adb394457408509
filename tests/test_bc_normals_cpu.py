"""The boundary normals of the slip and far-field conditions on curvilinear
grids (pyrandaBC.py:198-264): the product's torch form against the oracle's
numpy form, on the metrics of an O-mesh and of a sheared wavy grid computed
by the oracle.  Host tensors stand in for the device fields (the formulas are
torch operations on whole fields); no GPU."""
import numpy
import pytest

from oracle import oracle

torch = pytest.importorskip("torch")


class _FakeGrid:
    """The plane helpers of pyranda_gb300.grid.Grid on host tensors."""

    @staticmethod
    def get_plane(a, axis, k):
        idx = [slice(None)] * 3
        idx["xyz".index(axis)] = k
        return a[tuple(idx)]


class _FakeSim:
    def __init__(self, og):
        self.og = og
        self.grid = _FakeGrid()

        class _M:
            coordsys = 3
        self.mesh = _M()
        self.variables = {}

    def getVar(self, name):
        table = {"dtJ": 10, "dAx": 11, "dAy": 12, "dAz": 13, "dBx": 14, "dBy": 15, "dBz": 16, "dCx": 17,
                 "dCy": 18, "dCz": 19}
        return torch.from_numpy(numpy.ascontiguousarray(self.og.mesh(table[name])))


def _grid(kind):
    if kind == "omesh":
        n = (32, 24, 1)
        og = oracle.OracleGrid(n, (True, False, False), (0, 0, 0), (1, 2, 1), coordsys=3)
        i = numpy.arange(n[0])[:, None, None] * numpy.ones(n)
        r = 1.0 + numpy.arange(n[1])[None, :, None] / (n[1] - 1) * 9.0 * numpy.ones(n)
        th = i / n[0] * 2.0 * numpy.pi
        og.set_mesh_x3(r * numpy.cos(th), r * numpy.sin(th), numpy.zeros(n), mesh_periodic=False)
    else:
        n = (20, 16, 12)
        og = oracle.OracleGrid(n, (False, False, False), (0, 0, 0), (1, 1, 1), coordsys=3)
        A, B, C = numpy.meshgrid(*[numpy.linspace(0, 1, m) for m in n], indexing="ij")
        og.set_mesh_x3(A + 0.08 * numpy.sin(2 * numpy.pi * B) + 0.1 * B, B + 0.06 * numpy.sin(2 * numpy.pi * A),
                       C + 0.04 * numpy.sin(2 * numpy.pi * A) * numpy.cos(B), mesh_periodic=True)
    return og


@pytest.mark.parametrize("kind", ["omesh", "wavy"])
def test_curvilinear_boundary_normals_match_oracle(kind):
    from pyranda_gb300.pyrandaBC import pyrandaBC
    og = _grid(kind)
    sim = _FakeSim(og)
    bc = pyrandaBC.__new__(pyrandaBC)   # the package without a simulation's registration
    bc.pyranda = sim
    bc.BCdata = {}
    osim = type("S", (), {"coordsys": 3, "getVar": lambda self, nm: sim.getVar(nm).numpy()})()
    obc = oracle._BC.__new__(oracle._BC)
    obc.sim = osim
    obc.BCdata = {}
    ends = ["y1", "yn"] if kind == "omesh" else ["x1", "xn", "y1", "yn", "z1", "zn"]
    for d in ends:
        k = 0 if d[1] == "1" else -1
        got = bc.getNorms(d, k)
        want = obc.normal(d, k)
        for q in range(3):
            numpy.testing.assert_allclose(got[q].numpy(), want[q], rtol=0, atol=1e-14)
        mag = sum(g.numpy() ** 2 for g in got)
        numpy.testing.assert_allclose(mag, 1.0, rtol=1e-13)
    if kind == "omesh":
        # the wall of the O-mesh (y1, r = 1): the normal is radial, pointing into the cylinder
        n1, n2, _ = [t.numpy()[:, 0] for t in bc.getNorms("y1", 0)]
        th = numpy.arange(32) / 32 * 2.0 * numpy.pi
        numpy.testing.assert_allclose(numpy.abs(n1 * numpy.cos(th) + n2 * numpy.sin(th)), 1.0, atol=1e-6)
