"""Boundary conditions on device fields (pyranda/pyrandaBC.py:58-160).

``extrap`` (second-order or constant extrapolation) and ``const`` overwrite a
boundary plane of a non-periodic direction.  One GPU owns every boundary, so
the processor-boundary tests of the reference are the non-periodic tests.
"""
from .pyrandaPackage import pyrandaPackage


class pyrandaBC(pyrandaPackage):

    def __init__(self, pysim):
        pyrandaPackage.__init__(self, "BC", pysim)
        self.bcList = {}
        self.BCdata = {}

    def get_sMap(self):
        self.sMap = {"bc.extrap(": "self.packages['BC'].extrap(",
                     "bc.const(": "self.packages['BC'].const("}

    def _owns(self, direction):
        p = self.pyranda.PyMPI
        return getattr(p, direction[0] + ("1proc" if direction[1] == "1" else "nproc"))


    def extrap(self, var, direction, order=2):
        var = var if isinstance(var, list) else [var]
        direction = direction if isinstance(direction, list) else [direction]
        for d in direction:
            for v in var:
                self.extrapolate(v, d, order)

    def extrapolate(self, var, direction, order):
        if not self._owns(direction):
            return
        g = self.pyranda.grid
        a = self.pyranda.variables[var].data
        ax = direction[0]
        t, s1, s2 = (0, 1, 2) if direction[1] == "1" else (-1, -2, -3)
        if order == 2:
            g.set_plane(a, ax, t, 2 * g.get_plane(a, ax, s1) - g.get_plane(a, ax, s2))
        else:
            g.set_plane(a, ax, t, g.get_plane(a, ax, s1))

    def const(self, var, direction, val):
        var = var if isinstance(var, list) else [var]
        direction = direction if isinstance(direction, list) else [direction]
        for d in direction:
            for v in var:
                self.constant(v, d, val)

    def constant(self, var, direction, val):
        if not self._owns(direction):
            return
        a = self.pyranda.variables[var].data
        self.pyranda.grid.set_plane(a, direction[0], 0 if direction[1] == "1" else -1, val)
