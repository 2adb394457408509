"""Visualisation dumps in pyranda's VTK format, from device fields.

``pyrandaSim.write(wVars)`` (pyranda/pyranda.py:431-470) writes, per call,
``<rootname>/vis<cycle, 7 digits>/proc-<rank, 6 digits>.<cycle, 7 digits>.vtk``
and rewrites ``<rootname>/pyranda.visit`` (the list of dumps).  The file is a
legacy VTK STRUCTURED_GRID (pyranda/pyrandaIO.py:53-230):

* BINARY (pyranda's default): header lines, a FieldData block with TIME
  (one big-endian float32) and CYCLE (one big-endian int32), POINTS as
  big-endian float32 (x, y, z) per point with i fastest, then POINT_DATA with
  one big-endian float32 SCALARS block per variable.  With ``make2d`` a grid
  of one point in x or y and more than one in z is written as an (a, b, 1)
  grid, and a z coordinate that is constant on a one-plane grid becomes 0.
* ASCII: the same fields as text, each value followed by a space.

One GPU owns the whole grid, so there is one block (rank 0); the reference's
ghost exchange (pyrandaMPI.py:514-560) leaves a single block unchanged.
"""
import os

import numpy

PROC_DIGITS = 6
VIS_DIGITS = 7


def _f32be(a):
    return numpy.ascontiguousarray(a, dtype=">f4").tobytes()


def _layout(fx, fy, fz, make2d):
    """Coordinates after the 2-D remapping; returns (fx, fy, fz, shape, reshape)."""
    fx, fy, fz = (numpy.array(a, dtype=numpy.float64, order="F") for a in (fx, fy, fz))
    ax, ay, az = fx.shape
    reshape = None
    if make2d and az > 1 and (ax == 1 or ay == 1):
        if ax == 1:
            ax, ay, az = ay, az, 1
            fx[:, :, :] = fy
            fy[:, :, :] = fz
            fz[:, :, :] = 0.0
        else:
            ay, az = az, 1
            fy[:, :, :] = fz
            fz[:, :, :] = 0.0
        reshape = (ax, ay, 1)
        fx, fy, fz = (a.reshape(reshape, order="F") for a in (fx, fy, fz))
    if az == 1 and fz.max() == fz.min():
        fz[:, :, :] = 0.0
    return fx, fy, fz, (ax, ay, az), reshape


def write_binary(path, coords, fields, names, cycle, time, make2d=True):
    """path + '.vtk'; coords (x, y, z) and fields[name] are F-ordered (nx, ny, nz) host arrays."""
    fx, fy, fz, (ax, ay, az), reshape = _layout(*coords, make2d)
    npts = ax * ay * az
    pts = numpy.stack([fx.ravel(order="F"), fy.ravel(order="F"), fz.ravel(order="F")], axis=1)
    with open(path + ".vtk", "wb") as f:
        f.write(b"# vtk DataFile Version 3.0 \nvtk output \nBINARY \nDATASET STRUCTURED_GRID \n")
        f.write(("DIMENSIONS  %s %s %s  \n" % (ax, ay, az)).encode())
        f.write(b"FIELD FieldData 2 \nTIME 1 1 float \n")
        f.write(numpy.array([time], dtype=">f4").tobytes())
        f.write(b"CYCLE 1 1 int \n")
        f.write(numpy.array([cycle], dtype=">i4").tobytes())
        f.write(("POINTS %s float  \n" % npts).encode())
        f.write(_f32be(pts))
        f.write(("\nPOINT_DATA %s  " % npts).encode())
        for name in names:
            f.write(("\nSCALARS %s float \nLOOKUP_TABLE default \n" % name).encode())
            d = numpy.asarray(fields[name], dtype=numpy.float64)
            if reshape:
                d = d.reshape(reshape, order="F")
            f.write(_f32be(d.ravel(order="F")))


def write_ascii(path, coords, fields, names, cycle, time):
    """path + '.vtk' in the ASCII form (no 2-D remapping, as the reference's ASCII writer)."""
    fx, fy, fz = (numpy.asarray(a, dtype=numpy.float64) for a in coords)
    ax, ay, az = fx.shape
    with open(path + ".vtk", "w") as f:
        f.write("# vtk DataFile Version 3.0 \nvtk output \nASCII \nDATASET STRUCTURED_GRID \n")
        f.write("FIELD FieldData 2 \nCYCLE 1 1 int \n%d \nTIME 1 1 double \n%s \n" % (cycle, time))
        f.write("DIMENSIONS  %s %s %s  \n" % (ax, ay, az))
        f.write("POINTS %s float  \n" % (ax * ay * az))
        for x, y, z in zip(fx.ravel(order="F"), fy.ravel(order="F"), fz.ravel(order="F")):
            f.write("%s %s %s " % (x, y, z))
        f.write("\nPOINT_DATA %s  " % (ax * ay * az))
        for name in names:
            f.write("\nSCALARS %s float \nLOOKUP_TABLE default \n" % name)
            for v in numpy.asarray(fields[name], dtype=numpy.float64).ravel(order="F"):
                f.write("%s " % v)


def dump_path(rootname, cycle, rank=0):
    """<rootname>/vis<cycle>/proc-<rank>.<cycle> (without '.vtk')."""
    vis = "vis" + str(cycle).zfill(VIS_DIGITS)
    return os.path.join(rootname, vis, "proc-%s.%s" % (str(rank).zfill(PROC_DIGITS), str(cycle).zfill(VIS_DIGITS)))


def write_visit(rootname, history, nblocks=1):
    """<rootname>/pyranda.visit listing every dump of `history` ([cycle, time] pairs)."""
    with open(os.path.join(rootname, "pyranda.visit"), "w") as f:
        f.write("!NBLOCKS %s \n" % nblocks)
        for cycle, time in history:
            f.write("!TIME %s \n" % time)
            for p in range(nblocks):
                f.write("%s\n" % os.path.join("vis" + str(cycle).zfill(VIS_DIGITS),
                                              "proc-%s.%s.vtk" % (str(p).zfill(PROC_DIGITS),
                                                                  str(cycle).zfill(VIS_DIGITS))))
