"""Time-step limits (pyranda/pyrandaTimestep.py:42-87) as device reductions.

``courant`` and ``diff`` run one fused reduction kernel each and return a
device scalar, so the time step never leaves the GPU inside an RK step.
"""
import torch

from .pyrandaPackage import pyrandaPackage


class pyrandaTimestep(pyrandaPackage):

    def __init__(self, pysim):
        pyrandaPackage.__init__(self, "Timestep", pysim)
        self.dx = pysim.mesh.d1
        self.dy = pysim.mesh.d2
        self.dz = pysim.mesh.d3
        self.pysim = pysim
        self.GridLen = pysim.mesh.GridLen

    def get_sMap(self):
        self.sMap = {"dt.courant(": "self.packages['Timestep'].courant(",
                     "dt.diff(": "self.packages['Timestep'].diff(",
                     "dt.diffDir(": "self.packages['Timestep'].diffDir("}

    def courant(self, u, v, w, c):
        """1 / max(|u|/d1 + |v|/d2 + |w|/d3 + |c|/GridLen)  (pyrandaTimestep.py:42-67)."""
        return self.pysim.grid.courant(u, v, w, c)

    def diff(self, bulk, density):
        """min(rho * GridLen^2 / max(1e-12, bulk))  (pyrandaTimestep.py:71-77)."""
        return self.pysim.grid.diff(bulk, density)

    def diffDir(self, bulk, density, delta):
        drate = density * delta * delta / torch.clamp(bulk, min=1.0e-12)
        return self.pysim.PyMPI.min3D(drate)
