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

    def _plane(self, direction, k):
        return self.pyranda.grid.plane(direction[0], k)

    def extrap(self, var, direction, order=2):
        var = var if isinstance(var, list) else [var]
        direction = direction if isinstance(direction, list) else [direction]
        for d in direction:
            for v in var:
                self.extrapolate(v, d, order)

    def extrapolate(self, var, direction, order):
        if not self._owns(direction):
            return
        a = self.pyranda.variables[var].data
        t, s1, s2 = (0, 1, 2) if direction[1] == "1" else (-1, -2, -3)
        if order == 2:
            a[self._plane(direction, t)] = 2 * a[self._plane(direction, s1)] - a[self._plane(direction, s2)]
        else:
            a[self._plane(direction, t)] = a[self._plane(direction, s1)]

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
        a[self._plane(direction, 0 if direction[1] == "1" else -1)] = val
