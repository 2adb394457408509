"""The f2py-named shim (pyranda_gb300/parcop.py) maps parcop's arguments onto
the grid handle: boundary codes per end (parcop.f90:23-61), the coordinate
system, setup_mesh_x3 (:73-81), getVar's names (:84-128) and the
communicator hand-over (:385-403).  A recording stand-in replaces the CUDA
grid, so no GPU is needed."""
import numpy
import pytest

torch = pytest.importorskip("torch")


class _RecGrid:
    made = []

    def __init__(self, n, periodic, x1, xn, bc=None, coordsys=0):
        self.args = dict(n=n, periodic=periodic, x1=x1, xn=xn, bc=bc, coordsys=coordsys)
        self.calls = []
        _RecGrid.made.append(self)

    def field(self, v):
        return numpy.asarray(v, dtype=numpy.float64)

    def set_mesh_coords(self, x, y, z, mesh_periodic=True):
        self.calls.append(("set_mesh_coords", x.shape, mesh_periodic))

    def mesh(self, which):
        self.calls.append(("mesh", which))
        return torch.full((2, 2, 1), float(which), dtype=torch.float64)


@pytest.fixture
def shim(monkeypatch):
    from pyranda_gb300 import parcop as mod
    monkeypatch.setattr(mod, "Grid", _RecGrid)
    _RecGrid.made = []
    return mod._Parcop()


def test_setup_maps_ends_and_coordinate_system(shim):
    shim.setup(0, 0, None, 16, 12, 1, 1, 1, 1, 3, 0.0, 1.0, -1.0, 1.0, 0.0, 0.0,
               "PERI", "PERI", "symm", "NONE", "XTND", "NONE")
    g = _RecGrid.made[-1]
    assert g.args["n"] == (16, 12, 1)
    assert g.args["periodic"] == [True, False, False]
    assert g.args["bc"] == [("NONE", "NONE"), ("SYMM", "NONE"), ("XTND", "NONE")]
    assert g.args["coordsys"] == 3
    assert g.args["x1"] == (0.0, -1.0, 0.0) and g.args["xn"] == (1.0, 1.0, 0.0)


def test_bad_codes_and_decompositions_raise(shim):
    with pytest.raises(ValueError):
        shim.setup(0, 0, None, 8, 8, 8, 1, 1, 1, 0, 0, 1, 0, 1, 0, 1, "PERI", "PERI", "WALL", "NONE", "NONE", "NONE")
    with pytest.raises(ValueError):
        shim.setup(0, 0, None, 8, 8, 8, 2, 1, 1, 0, 0, 1, 0, 1, 0, 1, "PERI", "PERI", "NONE", "NONE", "NONE", "NONE")


def test_setup_mesh_x3_getvar_and_comm(shim):
    shim.setup(1, 0, None, 2, 2, 1, 1, 1, 1, 3, 0, 1, 0, 1, 0, 0, "NONE", "NONE", "NONE", "NONE", "NONE", "NONE")
    g = _RecGrid.made[-1]
    x = numpy.zeros((2, 2, 1))
    shim.setup_mesh_x3(1, 0, x, x, x, False)
    assert g.calls[-1] == ("set_mesh_coords", (2, 2, 1), False)
    table = {"x": 0, "y": 1, "z": 2, "d1": 3, "d2": 4, "d3": 5, "dtJ": 10, "dAx": 11, "dAy": 12, "dAz": 13,
             "dBx": 14, "dBy": 15, "dBz": 16, "dCx": 17, "dCy": 18, "dCz": 19}
    for name, which in table.items():
        out = shim.getvar(name.ljust(3), 2, 2, 1)   # f2py passes CHARACTER(LEN=3), blank padded
        assert numpy.all(out == which) and g.calls[-1] == ("mesh", which)
    with pytest.raises(ValueError):
        shim.getvar("dXx", 2, 2, 1)
    assert shim.commfrompy(1, 0, [0] * 7) is None
    with pytest.raises(KeyError):
        shim.commfrompy(5, 0, [0] * 7)
