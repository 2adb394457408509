"""Restart files in pyranda's format, from and to device fields.

A restart is the directory ``<rootname>/restart<suffix>`` (suffix
``_<cycle, 7 digits>`` by default) holding (pyranda/pyranda.py:475-589,
979-1130):

* ``serial.dat`` -- one line, the ``repr`` of a dict with the mesh options,
  EOM and IC strings, the decomposition ``[px, py, pz]`` and ``procMap``
  (first and last global index of every rank's block), the package modules,
  ``time``, ``deltat``, ``cycle``, ``vizDumpHistory``, the string map
  ``sMap`` and ``vars`` (variable name -> slot, names sorted), plus
  ``local_vars`` when the caller passed any;
* ``proc-<rank, 5 digits>.bin`` -- the rank's block of every variable as
  one FP64 array of shape (ax, ay, az, nvars) written in C order
  (``ndarray.tofile``), read back with a C-order reshape; a variable that is
  a single number is stored broadcast over the block.

One GPU owns the whole grid, so this writer produces one block
(decomposition [1, 1, 1]); the reader also accepts restarts of several
blocks, placing each block by ``procMap``.  Package modules are recorded
under the reference's names (``pyranda.pyrandaTimestep``, ...) so that either
code can read the other's restarts.
"""
import glob
import os
import sys

import numpy

RESTART_DIGITS = 7


def restart_dir(rootname, cycle, suffix=None):
    if not suffix:
        suffix = "_" + str(cycle).zfill(RESTART_DIGITS)
    return os.path.join(rootname, "restart" + suffix)


def write_files(dump, serial_data, arrays, shape):
    """serial.dat and proc-00000.bin; arrays: name -> host array of `shape` or a number."""
    os.makedirs(dump, exist_ok=True)
    names = sorted(arrays)
    serial_data = dict(serial_data)
    serial_data["vars"] = {n: i for i, n in enumerate(names)}
    po = numpy.get_printoptions()
    numpy.set_printoptions(threshold=sys.maxsize, linewidth=sys.maxsize)
    try:
        text = str(serial_data)
    finally:
        numpy.set_printoptions(**po)
    with open(os.path.join(dump, "serial.dat"), "w") as f:
        f.write(text)
    data = numpy.zeros(tuple(shape) + (len(names),), dtype=numpy.float64, order="F")
    for i, n in enumerate(names):
        data[:, :, :, i] = arrays[n]
    with open(os.path.join(dump, "proc-%s.bin" % "0".zfill(5)), "wb") as f:
        data.tofile(f)


def find_dump(rootname, suffix=None):
    if not suffix:
        dumps = sorted(glob.glob(os.path.join(rootname, "restart*")))
        if not dumps:
            raise FileNotFoundError("no restart under %s" % rootname)
        return dumps[-1]
    return os.path.join(rootname, "restart_%s" % suffix)


def read_serial(dump):
    from numpy import array, int32, int64, float64  # noqa: F401  (names the repr may contain)
    with open(os.path.join(dump, "serial.dat")) as f:
        return eval(f.readline())


def read_blocks(dump, serial_data, shape):
    """Assemble every variable of the whole grid (name -> F-ordered host array) from the rank blocks."""
    px, py, pz = [int(v) for v in serial_data["decomp"]]
    nx, ny, nz = shape
    ax, ay, az = nx // px, ny // py, nz // pz
    nv = len(serial_data["vars"])
    out = {n: numpy.zeros(shape, dtype=numpy.float64, order="F") for n in serial_data["vars"]}
    for rank in range(px * py * pz):
        g1 = [int(v) for v in serial_data["procMap"]["%s-g1" % rank]]
        gn = [int(v) + 1 for v in serial_data["procMap"]["%s-gn" % rank]]
        blk = numpy.fromfile(os.path.join(dump, "proc-%s.bin" % str(rank).zfill(5)), dtype=numpy.float64)
        blk = blk.reshape((ax, ay, az, nv), order="C")
        for n, i in serial_data["vars"].items():
            out[n][g1[0]:gn[0], g1[1]:gn[1], g1[2]:gn[2]] = blk[:gn[0] - g1[0], :gn[1] - g1[1], :gn[2] - g1[2], i]
    return out
