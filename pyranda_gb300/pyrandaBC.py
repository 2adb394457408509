"""Boundary conditions on device fields (pyranda/pyrandaBC.py).

Each condition overwrites boundary planes of a non-periodic direction with
torch operations on the device fields (no host copies, so they record in a
CUDA graph).  One GPU owns every boundary, so the processor-boundary tests of
the reference are the non-periodic tests.

  extrap / const           pyrandaBC.py:58-160
  field                    pyrandaBC.py:162-187 (x and y ends, as the reference)
  exit (BENO extrapolation) pyrandaBC.py:468-521 (x and y ends, as the reference)
  symm                     pyrandaBC.py:748-788
  slip                     pyrandaBC.py:190-465 (x and y ends, as the reference)
  farfield (Riemann)       pyrandaBC.py:524-745

slip and farfield take the boundary normal from the mesh metrics
(pyrandaBC.py:198-264), which parcop allocates for curvilinear meshes only
(mesh.f90:113-115).  On curvilinear meshes it is the cross product of the
metric rows rebuilt from the inverse Jacobian; on the other meshes the same
cross product is a unit axis vector: +x on the x ends, -y on the y ends, +z
on the z ends (d(x,y,z)/d(A,B,C) = diag(dx, dy, dz)).
"""
import math

import torch

from .pyrandaPackage import pyrandaPackage

# the normal of each boundary of a Cartesian mesh (see the module docstring)
_CART_NORMAL = {"x": (1.0, 0.0, 0.0), "y": (0.0, -1.0, 0.0), "z": (0.0, 0.0, 1.0)}


class pyrandaBC(pyrandaPackage):

    def __init__(self, pysim):
        pyrandaPackage.__init__(self, "BC", pysim)
        self.bcList = {}
        self.BCdata = {}

    def get_sMap(self):
        self.sMap = {"bc.extrap(": "self.packages['BC'].extrap(",
                     "bc.const(": "self.packages['BC'].const(",
                     "bc.exit(": "self.packages['BC'].exitbc(",
                     "bc.slip(": "self.packages['BC'].slipbc(",
                     "bc.field(": "self.packages['BC'].applyBC('field',",
                     "bc.farfield(": "self.packages['BC'].farfieldbc(",
                     "bc.symm(": "self.packages['BC'].symm("}

    def _owns(self, direction):
        p = self.pyranda.PyMPI
        return getattr(p, direction[0] + ("1proc" if direction[1] == "1" else "nproc"))

    # ------------------------------------------------------------ plane helpers
    def _get(self, var, direction, k):
        return self.pyranda.grid.get_plane(self.pyranda.variables[var].data, direction[0], k)

    def _set(self, var, direction, k, value):
        self.pyranda.grid.set_plane(self.pyranda.variables[var].data, direction[0], k, value)

    @staticmethod
    def _listed(x):
        return x if isinstance(x, list) else [x]

    def applyBC(self, func, var, direction, val=None):
        f = getattr(self, func)
        for d in self._listed(direction):
            for v in self._listed(var):
                if val is not None:
                    f(v, d, val)
                else:
                    f(v, d)

    # ------------------------------------------------------------ extrap / const / field
    def extrap(self, var, direction, order=2):
        for d in self._listed(direction):
            for v in self._listed(var):
                self.extrapolate(v, d, order)

    def extrapolate(self, var, direction, order):
        if not self._owns(direction):
            return
        t, s1, s2 = (0, 1, 2) if direction[1] == "1" else (-1, -2, -3)
        if order == 2:
            self._set(var, direction, t, 2 * self._get(var, direction, s1) - self._get(var, direction, s2))
        else:
            self._set(var, direction, t, self._get(var, direction, s1))

    def const(self, var, direction, val):
        for d in self._listed(direction):
            for v in self._listed(var):
                self.constant(v, d, val)

    def constant(self, var, direction, val):
        if not self._owns(direction):
            return
        self._set(var, direction, 0 if direction[1] == "1" else -1, val)

    def field(self, var, direction, field):
        """The boundary plane of var takes the same plane of `field` (a device field)."""
        if direction[0] == "z" or not self._owns(direction):
            return
        k = 0 if direction[1] == "1" else -1
        self._set(var, direction, k, self.pyranda.grid.get_plane(field, direction[0], k))

    # ------------------------------------------------------------ exit (BENO)
    def exitbc(self, var, direction, norm=False):
        for d in self._listed(direction):
            for v in self._listed(var):
                self.exit_boundary(v, d, norm)

    def exit_boundary(self, var, direction, norm):
        if direction[0] == "z" or not self._owns(direction):
            return
        k = (0, 1, 2) if direction[1] == "1" else (-1, -2, -3)
        u1, u2, u3 = (self._get(var, direction, q) for q in k)
        self._set(var, direction, k[0], self.BENO(u1, u2, u3, norm))

    @staticmethod
    def BENO(u1, u2, u3, norm):
        """Limited extrapolation (pyrandaBC.py:510-521): the smaller of the
        first- and second-order steps, none where they disagree in sign."""
        d1 = u2 - u1
        d2 = (2.0 * u2 - u3) - u1
        beno = torch.where(torch.abs(d1) <= torch.abs(d2), u1 + d1, u1 + d2)
        beno = torch.where(d1 * d2 <= 0.0, u1, beno)
        if norm:
            beno = torch.maximum(torch.minimum(beno, torch.clamp(u2, min=0.0)), torch.clamp(u2, max=0.0))
        return beno

    # ------------------------------------------------------------ symm
    def symm(self, var, direction, anti=False, npts=4):
        anti_mult = -1.0 if anti else 1.0
        for d in self._listed(direction):
            for v in self._listed(var):
                self.symmetric(v, d, anti_mult, npts)

    def symmetric(self, var, direction, antiMult, npts):
        """The npts boundary planes take the mirror image of the next npts (times antiMult)."""
        if not self._owns(direction):
            return
        a = self.pyranda.variables[var].data
        ax = "xyz".index(direction[0])
        n = a.shape[ax]
        dst, src = (0, npts) if direction[1] == "1" else (n - npts, n - 2 * npts)
        a.narrow(ax, dst, npts).copy_(a.narrow(ax, src, npts).flip(ax) * antiMult)

    # ------------------------------------------------------------ slip
    def slipbc(self, var, direction):
        """pyrandaBC.py:190-196: each entry of var is one velocity, the list of
        its component names (a single name is a one-component velocity)."""
        for d in self._listed(direction):
            for v in self._listed(var):
                self.slipvelbc(self._listed(v), d)

    def getNorms(self, direction, k):
        """The unit boundary normal on plane k of a boundary (pyrandaBC.py:198-264),
        cached per boundary like the reference's BCdata entries."""
        if getattr(self.pyranda.mesh, "coordsys", 0) != 3:
            return _CART_NORMAL[direction[0]]
        key = "normal-%s" % direction
        if key not in self.BCdata:
            g = self.pyranda.getVar
            dAdx, dAdy, dAdz = g("dAx"), g("dAy"), g("dAz")
            dBdx, dBdy, dBdz = g("dBx"), g("dBy"), g("dBz")
            dCdx, dCdy, dCdz = g("dCx"), g("dCy"), g("dCz")
            detJ = g("dtJ")
            m = {"xA": (-dBdz * dCdy + dBdy * dCdz) * detJ, "xB": (dAdz * dCdy - dAdy * dCdz) * detJ,
                 "xC": (-dAdz * dBdy + dAdy * dBdz) * detJ, "yA": (dBdz * dCdx - dBdx * dCdz) * detJ,
                 "yB": (-dAdz * dCdx + dAdx * dCdz) * detJ, "yC": (dAdz * dBdx - dAdx * dBdz) * detJ,
                 "zA": (-dBdy * dCdx + dBdx * dCdy) * detJ, "zB": (dAdy * dCdx - dAdx * dCdy) * detJ,
                 "zC": (-dAdy * dBdx + dAdx * dBdy) * detJ}
            t1, t2 = {"x": ("B", "C"), "y": ("A", "C"), "z": ("A", "B")}[direction[0]]
            a1, a2, a3 = m["x" + t1], m["y" + t1], m["z" + t1]
            b1, b2, b3 = m["x" + t2], m["y" + t2], m["z" + t2]
            n1 = a2 * b3 - a3 * b2
            n2 = -(a1 * b3 - a3 * b1)
            n3 = a1 * b2 - a2 * b1
            mag = torch.sqrt(n1 * n1 + n2 * n2 + n3 * n3)
            grid = self.pyranda.grid
            self.BCdata[key] = [grid.get_plane(n / mag, direction[0], k).clone() for n in (n1, n2, n3)]
        return self.BCdata[key]

    def slipvelbc(self, velocity, direction):
        """Free slip: extrapolate the velocity components, remove the normal
        component, and never let the speed grow (pyrandaBC.py:267-465)."""
        if direction[0] == "z":  # the reference has x and y ends only
            return
        for uu in velocity:
            self.extrapolate(uu, direction, order=2)
        if not self._owns(direction):
            return
        k = 0 if direction[1] == "1" else -1
        nrm = self.getNorms(direction, k)
        planes = [self._get(v, direction, k) for v in velocity]
        udotn = 0.0
        for q, u in enumerate(planes):
            udotn = udotn + u * nrm[q]
        mag0 = torch.sqrt(sum(u * u for u in planes))
        new = [u - udotn * nrm[q] for q, u in enumerate(planes)]
        magf = torch.sqrt(sum(u * u for u in new))
        for v, u in zip(velocity, new):
            self._set(v, direction, k, torch.where(magf > mag0, u * mag0 / magf, u))

    # ------------------------------------------------------------ farfield
    def getnormal(self, direction):
        return self.getNorms(direction, 0 if direction[1] == "1" else -1)

    def Reimann(self, direction, Rhoref, Uref, Vref, Wref, Pref, gamma, rhoi, Ui, Vi, Wi, Pi):
        """Boundary state from the Riemann invariants of the interior and the
        free stream (pyrandaBC.py:566-609)."""
        nx, ny, nz = self.getnormal(direction)
        Vni = Ui * nx + Vi * ny + Wi * nz
        Vno = Uref * nx + Vref * ny + Wref * nz
        SSo = math.sqrt(gamma * Pref / Rhoref)
        SSi = torch.sqrt(gamma * Pi / rhoi)
        tmp = torch.sqrt(Ui ** 2 + Vi ** 2 + Wi ** 2) / SSi
        sup = tmp >= 1.0
        Rplus = torch.where(sup, Vno + 2.0 * SSo / (gamma - 1.0), Vni + 2.0 * SSi / (gamma - 1.0))
        Rminus = torch.where(sup, Vni - 2.0 * SSi / (gamma - 1.0), Vno - 2.0 * SSo / (gamma - 1.0))
        Vnormal = (Rminus + Rplus) * 0.5
        SSb = (Rplus - Rminus) * (gamma - 1.0) * 0.25
        out = Vnormal >= 0.0
        Ub = torch.where(out, Ui + (Vnormal - Vni) * nx, Uref + (Vnormal - Vno) * nx)
        Vb = torch.where(out, Vi + (Vnormal - Vni) * ny, Vref + (Vnormal - Vno) * ny)
        Wb = torch.where(out, Wi + (Vnormal - Vni) * nz, Wref + (Vnormal - Vno) * nz)
        aux = 1.0 / (gamma - 1.0)
        rhob = torch.where(out, ((rhoi ** gamma * SSb ** 2) / (gamma * Pi)) ** aux,
                           ((Rhoref ** gamma * SSb ** 2) / (gamma * Pref)) ** aux)
        Pb = rhob * SSb ** 2 / gamma
        Etb = Pb / (gamma - 1.0) + 0.5 * rhob * (Ub * Ub + Vb * Vb + Wb * Wb)
        return rhob, Ub, Vb, Wb, Etb, Pb

    def farfieldbc(self, direction):
        for d in self._listed(direction):
            self.farfield(d)

    def farfield(self, direction):
        """Needs BCdata['farfield-properties-<direction>'] = {rho0, u0, v0, w0,
        p0, gamma, and the variable names rho, u, v, w, p}, as the reference."""
        ref = self.BCdata["farfield-properties-%s" % direction]
        if not self._owns(direction):
            return
        names = [ref[k] for k in ("rho", "u", "v", "w", "p")]
        b, i = (0, 1) if direction[1] == "1" else (-1, -2)
        rhoi, Ui, Vi, Wi, Pi = (self._get(v, direction, i) for v in names)
        rhob, Ub, Vb, Wb, Etb, Pb = self.Reimann(direction, ref["rho0"], ref["u0"], ref["v0"], ref["w0"], ref["p0"],
                                                 ref["gamma"], rhoi, Ui, Vi, Wi, Pi)
        for v, val in zip(names, (rhob, Ub, Vb, Wb, Pb)):
            self._set(v, direction, b, val)
