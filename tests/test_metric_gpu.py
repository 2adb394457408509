"""Spherical, ratio-zoned spherical and curvilinear grids, and the field-scaled
forms of cylindrical ones, against the oracle.

Spherical grids (mesh.f90:169-244) keep the radius, the polar angle and the
azimuth with d1 = dx, d2 = r dy, d3 = r sin(theta) dz; curvilinear grids
(mesh.f90:245-358) take their coordinates from the caller and their metrics
from the first-derivative operator.  The operators apply the metric forms of
operators.f90:54-209 (grad, div, divT), :527-559 (Laplacian), :884-889 (the
filter of CellVol-weighted fields over the filtered cell volume) and ring
with the mesh fields d1 d2 d3 (:615-699); the time-step limits use the same
fields (pyrandaTimestep.py:42-77).  Bar: relative L2 <= 1e-12 against the
oracle, the mesh fields and the time steps included.
"""
import numpy
import pytest

from tests.helpers import rel_l2, smooth_field, to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

TOL = 1.0e-12

SPHERICAL = [
    # (shape, periodic, x1, xn, bc, coordsys)
    ((24, 16, 20), (False, False, True), (0.5, 0.3, 0.0), (2.0, 2.8, 1.5),
     (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")), 2),
    ((40, 1, 16), (False, False, True), (0.6, 1.56, -0.2), (6.2, 1.58, 0.2),
     (("NONE", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")), 2),
    ((32, 12, 10), (False, False, False), (0.5, 0.4, 0.0), (3.0, 2.6, 1.0),
     (("NONE", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")), 4),
]


def _coords_curv(shape, x1, xn, periodic_map):
    """Node coordinates numpy.linspace(x1, xn, n) per direction, mapped smoothly
    (a sheared, wavy grid), or an O-mesh when periodic_map is set."""
    lin = [numpy.linspace(x1[d], xn[d], num=shape[d]) for d in range(3)]
    A, B, C = numpy.meshgrid(*lin, indexing="ij")
    if periodic_map:  # x = r cos(theta), y = r sin(theta) with theta = 2 pi i / n (periodic in i)
        i = numpy.arange(shape[0])[:, None, None] * numpy.ones(shape)
        theta = i / shape[0] * 2.0 * numpy.pi
        r = 1.0 + B
        return r * numpy.cos(theta), r * numpy.sin(theta), C
    x = A + 0.08 * numpy.sin(2.0 * numpy.pi * B / (xn[1] - x1[1])) + 0.1 * B
    y = B + 0.06 * numpy.sin(2.0 * numpy.pi * A / (xn[0] - x1[0]))
    z = C + 0.04 * numpy.sin(2.0 * numpy.pi * A / (xn[0] - x1[0])) * numpy.cos(B)
    return x, y, z


CURVILINEAR = [
    # (shape, periodic, x1, xn, periodic_map, mesh_periodic)
    ((24, 20, 16), (False, False, False), (0.0, 0.0, 0.0), (2.0, 1.5, 1.0), False, True),
    ((32, 24, 1), (True, False, False), (0.0, 0.0, 0.0), (1.0, 2.0, 1.0), True, False),
    ((20, 16, 12), (False, True, False), (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), False, True),
]


def _fields(shape, k=9, seed=60):
    fs = [smooth_field(shape, seed=seed + i) for i in range(k)]
    return fs, [to_dev(f, torch) for f in fs]


def _courant_np(o, coordsys, u, v, w, c):
    """pyrandaTimestep.py:42-63 on the oracle's mesh fields."""
    d1, d2, d3, gl = o.mesh(3), o.mesh(4), o.mesh(5), o.mesh(6)
    if coordsys == 3:
        dAdx, dAdy, dBdx, dBdy = o.mesh(11), o.mesh(12), o.mesh(14), o.mesh(15)
        magA = numpy.sqrt(dAdx * dAdx + dAdy * dAdy)
        magB = numpy.sqrt(dBdx * dBdx + dBdy * dBdy)
        uA = (u * dAdx + v * dAdy) / magA
        uB = (u * dBdx + v * dBdy) / magB
        vrate = numpy.abs(uA) / d1 + numpy.abs(uB) / d2
    else:
        vrate = numpy.abs(u) / d1 + numpy.abs(v) / d2 + numpy.abs(w) / d3
    return 1.0 / numpy.max(vrate + numpy.abs(c) / gl)


def _diff_np(o, bulk, rho):
    gl = o.mesh(6)
    return numpy.min(rho * gl * gl / numpy.maximum(1.0e-12, bulk))


def _check_ops(g, o, shape, coordsys, nmesh):
    fs, ds = _fields(shape)
    bad = []

    def cmp(name, a, b, tol=TOL):
        e = rel_l2(to_host(a), b)
        if not e <= tol:
            bad.append((name, e))

    for which in range(nmesh):
        cmp(("mesh", which), g.mesh(which), o.mesh(which))
    cmp("div", g.div(ds[0], ds[1], ds[2]), o.div(fs[0], fs[1], fs[2]))
    for q, (a, b) in enumerate(zip(g.divT(*ds), o.divt(*fs))):
        cmp(("divT", q), a, b)
    for q, (a, b) in enumerate(zip(g.grad(ds[3]), o.grad(fs[3]))):
        cmp(("grad", q), a, b)
    cmp("fbar", g.filter("spectral", ds[4]), o.sfilter(fs[4]))
    cmp("gbar", g.filter("gaussian", ds[5]), o.gfilter(fs[5]))
    cmp("ring", g.ring(ds[6]), o.ring(fs[6], 2))
    cmp("ringV", g.ringv(ds[6], ds[7], ds[8]), o.ringv(fs[6], fs[7], fs[8], 1))
    # time-step limits: positive speeds, bulk viscosities and densities
    u, v, w, c = (numpy.abs(f) + 0.1 for f in fs[:4])
    dt = float(g.courant(to_dev(u, torch), to_dev(v, torch), to_dev(w, torch), to_dev(c, torch)))
    dto = _courant_np(o, coordsys, u, v, w, c)
    if not abs(dt - dto) <= 1e-12 * dto:
        bad.append(("courant", dt, dto))
    bulk, rho = numpy.abs(fs[4]) * 1e-3, numpy.abs(fs[5]) + 0.5
    dd = float(g.diff(to_dev(bulk, torch), to_dev(rho, torch)))
    ddo = _diff_np(o, bulk, rho)
    if not abs(dd - ddo) <= 1e-12 * ddo:
        bad.append(("diff", dd, ddo))
    return bad


@pytest.mark.parametrize("shape,per,x1,xn,bc,coordsys", SPHERICAL)
def test_spherical_operators_match_oracle(oracle, shape, per, x1, xn, bc, coordsys):
    """Spherical grids (coordsys 2) and ratio-zoned ones (coordsys 4): mesh
    fields, div, divT, grad, both filters, ring, ringV and the time-step limits;
    the Laplacian of coordsys 2 (coordsys 4 has none in the reference)."""
    from pyranda_gb300.grid import Grid
    from pyranda_gb300._lib import PgError
    g = Grid(shape, per, x1, xn, bc=bc, coordsys=coordsys)
    o = oracle.OracleGrid(shape, per, x1, xn, bc=bc, coordsys=coordsys)
    bad = _check_ops(g, o, shape, coordsys, 10)
    f = smooth_field(shape, seed=90)
    if coordsys == 2:
        e = rel_l2(to_host(g.laplacian(to_dev(f, torch))), o.laplacian(f))
        bad += [("lap", e)] if not e <= TOL else []
    else:
        with pytest.raises(PgError):
            g.laplacian(to_dev(f, torch))
    assert not bad, bad


@pytest.mark.parametrize("shape,per,x1,xn,periodic_map,mesh_periodic", CURVILINEAR)
def test_curvilinear_operators_match_oracle(oracle, shape, per, x1, xn, periodic_map, mesh_periodic):
    """Curvilinear grids (coordsys 3): the metrics of supplied coordinates --
    by the non-periodic first derivative ('periodicGrid', mesh.f90:246-307) or
    the grid's own -- then every mesh field, div, divT, grad, both filters,
    ring, ringV and the time-step limits; no Laplacian in the reference."""
    from pyranda_gb300.grid import Grid
    from pyranda_gb300._lib import PgError
    g = Grid(shape, per, x1, xn, coordsys=3)
    o = oracle.OracleGrid(shape, per, x1, xn, coordsys=3)
    x, y, z = _coords_curv(shape, x1, xn, periodic_map)
    g.set_mesh_coords(to_dev(x, torch), to_dev(y, torch), to_dev(z, torch), mesh_periodic)
    o.set_mesh_x3(x, y, z, mesh_periodic)
    bad = _check_ops(g, o, shape, 3, 20)
    with pytest.raises(PgError):
        g.laplacian(to_dev(smooth_field(shape, seed=91), torch))
    assert not bad, bad


def test_curvilinear_default_coordinates_are_the_nodes(oracle):
    """Before coordinates are supplied, a curvilinear grid takes the nodes
    linspace(x1, xn, n) of each direction (pyrandaMesh.py:96-108): its metrics
    are those of the Cartesian grid of the same nodes."""
    from pyranda_gb300.grid import Grid
    shape, per, x1, xn = (20, 16, 12), (False, False, False), (0.0, -1.0, 0.5), (2.0, 1.0, 1.5)
    g = Grid(shape, per, x1, xn, coordsys=3)
    o = oracle.OracleGrid(shape, per, x1, xn, coordsys=3)
    for which in range(20):
        e = rel_l2(to_host(g.mesh(which)), o.mesh(which))
        assert e <= TOL, (which, e)
    # the inverse Jacobian of an axis-aligned uniform grid is diagonal: dA/dx = 1
    numpy.testing.assert_allclose(to_host(g.mesh(11)), 1.0, rtol=1e-10)
    assert numpy.abs(to_host(g.mesh(12))).max() < 1e-10


@pytest.mark.parametrize("shape,bc", [((36, 20, 24), (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "NONE"))),
                                      ((40, 1, 32), (("SYMM", "NONE"), ("NONE", "NONE"), ("NONE", "NONE")))])
def test_cylindrical_laplacian_and_ring_match_oracle(oracle, shape, bc):
    """Cylindrical grids: the Laplacian d(r df/dr)/dr / r + d2y / r^2 + d2z
    (operators.f90:527-543) and ring / ringV scaled by the mesh d2 = r dy
    (operators.f90:636-639, mesh.f90:213-216)."""
    from pyranda_gb300.grid import Grid
    per = (False, True, True)
    x1, xn = (0.05, 0.0, 0.0), (1.0, 2.0 * numpy.pi * (shape[1] - 1) / shape[1], 1.5)
    g = Grid(shape, per, x1, xn, bc=bc, coordsys=1)
    o = oracle.OracleGrid(shape, per, x1, xn, bc=bc, coordsys=1)
    fs, ds = _fields(shape, 3, seed=70)
    bad = []
    for name, a, b in (("lap", g.laplacian(ds[0]), o.laplacian(fs[0])),
                       ("ring", g.ring(ds[1]), o.ring(fs[1], 2)),
                       ("ringV", g.ringv(ds[0], ds[1], ds[2]), o.ringv(fs[0], fs[1], fs[2], 1))):
        e = rel_l2(to_host(a), b)
        bad += [(name, e)] if not e <= TOL else []
    assert not bad, bad
