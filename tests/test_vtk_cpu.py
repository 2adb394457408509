"""pyranda's VTK dumps (pyrandaIO.py:53-230) from host arrays: layout and bytes."""
import os
import struct

import numpy

from pyranda_gb300 import vtk


def _grid(shape):
    i, j, k = numpy.meshgrid(*[numpy.arange(n, dtype=numpy.float64) for n in shape], indexing="ij")
    return [numpy.asfortranarray(0.5 + i), numpy.asfortranarray(-1.0 + 0.25 * j), numpy.asfortranarray(2.0 + k)]


def test_binary_layout(tmp_path):
    shape = (4, 3, 2)
    xyz = _grid(shape)
    rho = numpy.asfortranarray(numpy.random.default_rng(0).random(shape))
    path = str(tmp_path / "d")
    vtk.write_binary(path, xyz, {"rho": rho}, ["rho"], 7, 0.125)
    raw = open(path + ".vtk", "rb").read()
    head = (b"# vtk DataFile Version 3.0 \nvtk output \nBINARY \nDATASET STRUCTURED_GRID \n"
            b"DIMENSIONS  4 3 2  \nFIELD FieldData 2 \nTIME 1 1 float \n")
    assert raw.startswith(head)
    p = len(head)
    assert struct.unpack(">f", raw[p:p + 4])[0] == 0.125
    p += 4
    assert raw[p:p + 15] == b"CYCLE 1 1 int \n"
    p += 15
    assert struct.unpack(">i", raw[p:p + 4])[0] == 7
    p += 4
    line = b"POINTS 24 float  \n"
    assert raw[p:p + len(line)] == line
    p += len(line)
    # points: (x, y, z) per point, i fastest, big-endian float32 -- written here value by value
    want = b"".join(struct.pack(">f", a[i, j, k]) for k in range(2) for j in range(3) for i in range(4)
                    for a in xyz)
    assert raw[p:p + len(want)] == want
    p += len(want)
    line = b"\nPOINT_DATA 24  \nSCALARS rho float \nLOOKUP_TABLE default \n"
    assert raw[p:p + len(line)] == line
    p += len(line)
    want = b"".join(struct.pack(">f", rho[i, j, k]) for k in range(2) for j in range(3) for i in range(4))
    assert raw[p:] == want


def test_binary_2d_remap_and_flat_z(tmp_path):
    # one point in y, several in z: written as a (nx, nz, 1) grid with z -> y and z = 0
    shape = (3, 1, 4)
    xyz = _grid(shape)
    f = numpy.asfortranarray(numpy.arange(12, dtype=numpy.float64).reshape(shape, order="F"))
    path = str(tmp_path / "r")
    vtk.write_binary(path, xyz, {"f": f}, ["f"], 0, 0.0)
    raw = open(path + ".vtk", "rb").read()
    assert b"DIMENSIONS  3 4 1  \n" in raw
    p = raw.index(b"POINTS 12 float  \n") + len(b"POINTS 12 float  \n")
    pts = numpy.frombuffer(raw[p:p + 12 * 12], dtype=">f4").reshape(12, 3)
    assert numpy.array_equal(pts[:, 1], xyz[2].ravel(order="F").astype(numpy.float32))
    assert not pts[:, 2].any()
    vals = numpy.frombuffer(raw[-48:], dtype=">f4")
    assert numpy.array_equal(vals, f.ravel(order="F").astype(numpy.float32))


def test_ascii_and_visit(tmp_path):
    shape = (2, 2, 1)
    xyz = _grid(shape)
    path = vtk.dump_path(str(tmp_path), 12)
    os.makedirs(os.path.dirname(path))
    vtk.write_ascii(path, xyz, {"u": xyz[0]}, ["u"], 12, 0.5)
    text = open(path + ".vtk").read()
    assert text.startswith("# vtk DataFile Version 3.0 \nvtk output \nASCII \nDATASET STRUCTURED_GRID \n"
                           "FIELD FieldData 2 \nCYCLE 1 1 int \n12 \nTIME 1 1 double \n0.5 \n"
                           "DIMENSIONS  2 2 1  \nPOINTS 4 float  \n0.5 -1.0 2.0 1.5 -1.0 2.0 ")
    assert text.endswith("\nSCALARS u float \nLOOKUP_TABLE default \n0.5 1.5 0.5 1.5 ")
    assert path.endswith(os.path.join("vis0000012", "proc-000000.0000012"))
    vtk.write_visit(str(tmp_path), [[0, 0.0], [12, 0.5]])
    assert open(os.path.join(str(tmp_path), "pyranda.visit")).read() == (
        "!NBLOCKS 1 \n!TIME 0.0 \nvis0000000/proc-000000.0000000.vtk\n"
        "!TIME 0.5 \nvis0000012/proc-000000.0000012.vtk\n")
