"""``parcop.parcop`` drop-in: the f2py module's names over libpyranda_gpu.so.

pyranda's Python layer talks to the Fortran library through the f2py module
``pyranda.parcop.parcop`` (built from pyranda/parcop/parcop.f90), e.g.
``parcop.parcop.ddx(val)`` (pyrandaMPI.py:669-740).  This module offers the
same entry points, argument order and return values:

    from pyranda_gb300.parcop import parcop
    parcop.setup(patch, level, comm, nx, ny, nz, px, py, pz, coordsys,
                 x1, xn, y1, yn, z1, zn, bx1, bxn, by1, byn, bz1, bzn)
    parcop.set_patch(patch, level)
    dval = parcop.ddx(val)

Arrays may be numpy arrays (copied to the GPU and back, returning a new
F-ordered numpy array as f2py does) or torch CUDA tensors in the (nx,ny,nz)
Fortran layout (kept on the device).  As in parcop, the (patch, level) pair
selected by ``set_patch`` is the active grid; ``setup`` makes the new grid
active (objects.f90:35-49, :77-89).

Scope: one GPU (px = py = pz = 1); every coordinate system (0 Cartesian,
1 cylindrical, 2 spherical, 3 curvilinear with ``setup_mesh_x3``, 4
ratio-zoned spherical); boundary codes PERI, NONE, SYMM and XTND.  A
decomposition over several processes raises instead of silently misbehaving.
"""
import numpy
import torch

from .grid import Grid


class _Parcop:
    def __init__(self):
        self._grids = {}
        self._active = None

    # parcop.f90:23-61
    def setup(self, patch, level, comm, nx, ny, nz, px, py, pz, coordsys, x1, xn, y1, yn, z1, zn,
              bx1, bxn, by1, byn, bz1, bzn):
        if px * py * pz != 1:
            raise ValueError("one GPU holds the whole grid: px*py*pz must be 1")
        per, bc = [], []
        for lo, hi in ((bx1, bxn), (by1, byn), (bz1, bzn)):
            lo, hi = str(lo).strip().upper(), str(hi).strip().upper()
            for b in (lo, hi):
                if b not in ("PERI", "NONE", "SYMM", "XTND"):
                    raise ValueError("boundary code %r is not PERI, NONE, SYMM or XTND" % b)
            per.append(lo == "PERI")
            bc.append(tuple("NONE" if b == "PERI" else b for b in (lo, hi)))
        g = Grid((nx, ny, nz), per, (x1, y1, z1), (xn, yn, zn), bc=bc, coordsys=int(coordsys))
        self._grids[(patch, level)] = g
        self._active = g

    def setup_mesh(self, patch, level):
        """parcop.f90:64-70: the mesh of every coordinate system but the curvilinear one
        is generated by setup."""
        if (patch, level) not in self._grids:
            raise KeyError("patch %s level %s was not set up" % (patch, level))

    def setup_mesh_x3(self, patch, level, x1, x2, x3, meshPer):
        """parcop.f90:73-81: the coordinates of a curvilinear patch and its metrics."""
        g = self._grids[(patch, level)]
        g.set_mesh_coords(*[self._in_for(g, v) for v in (x1, x2, x3)], mesh_periodic=bool(meshPer))

    def set_patch(self, patch, level):
        self._active = self._grids[(patch, level)]

    def remove(self, patch, level):
        self._grids.pop((patch, level), None)

    # ---------------------------------------------------------------- helpers
    def _g(self):
        if self._active is None:
            raise RuntimeError("parcop.setup has not been called")
        return self._active

    @staticmethod
    def _in_for(g, v):
        if isinstance(v, torch.Tensor):
            return g.field(v)
        return g.field(numpy.asfortranarray(numpy.asarray(v, dtype=numpy.float64)))

    def _in(self, v):
        g = self._g()
        if isinstance(v, torch.Tensor):
            return g.field(v), True
        return g.field(numpy.asfortranarray(numpy.asarray(v, dtype=numpy.float64))), False

    @staticmethod
    def _out(t, device):
        if device:
            return t
        return numpy.asfortranarray(t.permute(2, 1, 0).cpu().numpy().transpose(2, 1, 0))

    def _unary(self, fn, val):
        v, dev = self._in(val)
        return self._out(fn(v), dev)

    # ------------------------------------------------------------- operators
    def ddx(self, val, nx=None, ny=None, nz=None):  # parcop.f90:225-233
        return self._unary(self._g().ddx, val)

    def ddy(self, val, nx=None, ny=None, nz=None):  # parcop.f90:235-243
        return self._unary(self._g().ddy, val)

    def ddz(self, val, nx=None, ny=None, nz=None):  # parcop.f90:245-253
        return self._unary(self._g().ddz, val)

    def dd4x(self, val, nx=None, ny=None, nz=None):  # parcop.f90:255-261
        return self._unary(lambda v: self._g().d4(0, v), val)

    def dd4y(self, val, nx=None, ny=None, nz=None):  # parcop.f90:263-269
        return self._unary(lambda v: self._g().d4(1, v), val)

    def dd4z(self, val, nx=None, ny=None, nz=None):  # parcop.f90:271-277
        return self._unary(lambda v: self._g().d4(2, v), val)

    def plaplacian(self, val, nx=None, ny=None, nz=None):  # parcop.f90:303-311
        return self._unary(self._g().laplacian, val)

    def dd8x(self, val, nx=None, ny=None, nz=None):  # parcop.f90:279-285
        return self._unary(lambda v: self._g().d8(0, v), val)

    def dd8y(self, val, nx=None, ny=None, nz=None):
        return self._unary(lambda v: self._g().d8(1, v), val)

    def dd8z(self, val, nx=None, ny=None, nz=None):
        return self._unary(lambda v: self._g().d8(2, v), val)

    def pring(self, val, nx=None, ny=None, nz=None):  # parcop.f90:313-322
        return self._unary(self._g().ring, val)

    def pringv(self, vx, vy, vz, nx=None, ny=None, nz=None):  # parcop.f90:324-333
        a, dev = self._in(vx)
        b, _ = self._in(vy)
        c, _ = self._in(vz)
        return self._out(self._g().ringv(a, b, c), dev)

    def sfilter(self, val, nx=None, ny=None, nz=None):  # parcop.f90:337-346
        return self._unary(lambda v: self._g().filter("spectral", v), val)

    def gfilter(self, val, nx=None, ny=None, nz=None):  # parcop.f90:348-357
        return self._unary(lambda v: self._g().filter("gaussian", v), val)

    def gfilterdir(self, val, direction, nx=None, ny=None, nz=None):  # parcop.f90:359-368
        return self._unary(lambda v: self._g().filter("gaussian", v, int(direction) - 1), val)

    def grads(self, val, nx=None, ny=None, nz=None):  # parcop.f90:371-379
        v, dev = self._in(val)
        return tuple(self._out(t, dev) for t in self._g().grad(v))

    def divergence(self, fx, fy, fz, nx=None, ny=None, nz=None):  # parcop.f90:202-211
        a, dev = self._in(fx)
        b, _ = self._in(fy)
        c, _ = self._in(fz)
        return self._out(self._g().div(a, b, c), dev)

    def divergencetensor(self, fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz, nx=None, ny=None,
                         nz=None):  # parcop.f90:213-223
        args = [self._in(f) for f in (fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz)]
        dev = args[0][1]
        return tuple(self._out(t, dev) for t in self._g().divT(*[a for a, _ in args]))

    # ------------------------------------------------------------------ mesh
    def _mesh(self, which):
        return self._out(self._g().mesh(which), False)

    def xgrid(self, nx=None, ny=None, nz=None):  # parcop.f90:130-135
        return self._mesh(0)

    def ygrid(self, nx=None, ny=None, nz=None):
        return self._mesh(1)

    def zgrid(self, nx=None, ny=None, nz=None):
        return self._mesh(2)

    def dxgrid(self, nx=None, ny=None, nz=None):  # parcop.f90:154-159
        return self._mesh(3)

    def dygrid(self, nx=None, ny=None, nz=None):
        return self._mesh(4)

    def dzgrid(self, nx=None, ny=None, nz=None):
        return self._mesh(5)

    def mesh_getgridlen(self, nx=None, ny=None, nz=None):  # parcop.f90:186-191
        return self._mesh(6)

    def mesh_getcellvol(self, nx=None, ny=None, nz=None):  # parcop.f90:179-184
        return self._mesh(7)

    _VARS = {"x": 0, "y": 1, "z": 2, "d1": 3, "d2": 4, "d3": 5, "dAx": 11, "dAy": 12, "dAz": 13, "dBx": 14,
             "dBy": 15, "dBz": 16, "dCx": 17, "dCy": 18, "dCz": 19, "dtJ": 10}

    def getvar(self, vname, nx=None, ny=None, nz=None):  # parcop.f90:84-128
        key = str(vname).strip()
        if key not in self._VARS:
            raise ValueError("mesh variable %r is not one of parcop's getVar names" % key)
        return self._mesh(self._VARS[key])

    # single-process communicators (comm.f90): every rank id is 0
    def commfrompy(self, patch, level, comm_list):
        """parcop.f90:385-403 commFromPy: the seven communicators of a patch handed
        over from Python; one process owns the GPU, so there is nothing to store."""
        if (patch, level) not in self._grids:
            raise KeyError("patch %s level %s was not set up" % (patch, level))

    def commx(self):
        return 0

    commy = commz = commxy = commyz = commxz = commx


parcop = _Parcop()
