"""ORACLE — test infrastructure only.

ctypes binding of the FP64 CPU restatement in ``parcop_oracle.cpp`` plus a
numpy restatement of pyranda's Python driver layer (``pyrandaSim`` with its
EOM/IC string translator, LSRK(5,4) ``rk4``, the ``Timestep`` and ``BC``
packages).  It exists so the test-suite can check the CUDA library and the
product's ``pyrandaSim`` against an independent CPU computation, and so that
``bench.py`` can time a CPU baseline.  The product never imports this module.

Reference files restated here (paths within the pyranda project):
  pyranda/pyranda.py:34-131 (init), :231-370 (EOM/setIC), :376-428
  (updateFlux/updateVars), :607-736 (operators), :758-810 (rk4), :812-869 (sMap)
  pyranda/pyrandaUtils.py:22-141 (fortran3d, findVar)
  pyranda/pyrandaEq.py:16-48, pyranda/pyrandaMesh.py:33-56,214-233
  pyranda/pyrandaTimestep.py:42-77, pyranda/pyrandaBC.py:58-160
  pyranda/pyrandaMPI.py:307-326 (sum3D/max3D/min3D on one rank)
"""
import ctypes
import os
import re
import subprocess

import numpy

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libparcop_oracle.so")
_lib = None


def build():
    """Compile the oracle library (make in this directory)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        D = ctypes.POINTER(ctypes.c_double)
        I = ctypes.POINTER(ctypes.c_int)
        L.og_create.argtypes = [I, I, D, D, ctypes.POINTER(P)]
        L.og_create2.argtypes = [I, I, I, ctypes.c_int, D, D, ctypes.POINTER(P)]
        L.og_apply_sym.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, D, D]
        L.og_filter3_sym.argtypes = [P, ctypes.c_int, I, D, D]
        L.og_destroy.argtypes = [P]
        L.og_apply.argtypes = [P, ctypes.c_int, ctypes.c_int, D, D]
        L.og_laplacian.argtypes = [P, D, D]
        L.og_filter3.argtypes = [P, ctypes.c_int, D, D]
        L.og_ring.argtypes = [P, D, D, ctypes.c_int]
        L.og_ringv.argtypes = [P, D, D, D, D, ctypes.c_int]
        L.og_grad.argtypes = [P, D, D, D, D]
        L.og_div.argtypes = [P, D, D, D, D]
        L.og_divt.argtypes = [P, ctypes.POINTER(D), ctypes.POINTER(D)]
        L.og_mesh.argtypes = [P, ctypes.c_int, D]
        L.og_set_mesh_x3.argtypes = [P, D, D, D, ctypes.c_int]
        L.og_spacing.argtypes = [P, D, D]
        L.og_dense.argtypes = [P, ctypes.c_int, ctypes.c_int, D]
        L.og_threads.restype = ctypes.c_int
        L.og_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _f64(a):
    """F-ordered float64 copy/view of a (nx,ny,nz) array (the parcop layout)."""
    return numpy.asfortranarray(numpy.asarray(a, dtype=numpy.float64))


OP_D1, OP_D8, OP_SF, OP_GF, OP_D2, OP_D4 = 0, 1, 2, 3, 4, 5


class OracleGrid:
    """One parcop patch: parcop.f90:23-61 ``setup`` on a Cartesian mesh."""

    def __init__(self, n, periodic, x1, xn, bc=None, coordsys=0):
        """bc: per direction (lower, upper) end codes 'NONE' / 'SYMM' / 'XTND' (non-periodic
        directions); coordsys 0 Cartesian, 1 cylindrical, 2 spherical, 3 curvilinear
        (coordinates by ``set_mesh_x3``), 4 spherical with ratio-zoned radii."""
        L = lib()
        n = (ctypes.c_int * 3)(*[int(v) for v in n])
        per = (ctypes.c_int * 3)(*[1 if p else 0 for p in periodic])
        a = (ctypes.c_double * 3)(*[float(v) for v in x1])
        b = (ctypes.c_double * 3)(*[float(v) for v in xn])
        codes = {"NONE": 0, "SYMM": 1, "XTND": 2}
        bc = bc or (("NONE", "NONE"),) * 3
        bcs = (ctypes.c_int * 6)(*[codes[bc[d][e]] for d in range(3) for e in range(2)])
        self.coordsys = int(coordsys)
        h = ctypes.c_void_p()
        rc = L.og_create2(n, per, bcs, self.coordsys, a, b, ctypes.byref(h))
        if rc != 0:
            raise ValueError("oracle: bad grid")
        self.h = h
        self.shape = (n[0], n[1], n[2])

    def __del__(self):
        try:
            if self.h:
                lib().og_destroy(self.h)
        except Exception:
            pass

    def _out(self):
        return numpy.zeros(self.shape, dtype=numpy.float64, order="F")

    def apply(self, op, direction, v):
        v = _f64(v)
        out = self._out()
        lib().og_apply(self.h, op, direction, _dp(v), _dp(out))
        return out

    def apply_sym(self, op, direction, sym, v):
        """The operator variant for symmetric (+1) or antisymmetric (-1) fields at a SYMM end."""
        v = _f64(v)
        out = self._out()
        lib().og_apply_sym(self.h, op, direction, int(sym), _dp(v), _dp(out))
        return out

    def filter_sym(self, op, sym, v):
        """x -> y -> z filter (op 2 compact, 3 Gaussian) with one variant sign per direction."""
        v = _f64(v)
        out = self._out()
        s3 = (ctypes.c_int * 3)(*[int(x) for x in sym])
        lib().og_filter3_sym(self.h, op, s3, _dp(v), _dp(out))
        return out

    def ddx(self, v):
        return self.apply(OP_D1, 0, v)

    def ddy(self, v):
        return self.apply(OP_D1, 1, v)

    def ddz(self, v):
        return self.apply(OP_D1, 2, v)

    def dd8(self, direction, v):
        return self.apply(OP_D8, direction, v)

    def d2(self, direction, v):
        return self.apply(OP_D2, direction, v)

    def dd4(self, direction, v):
        return self.apply(OP_D4, direction, v)

    def laplacian(self, v):
        v = _f64(v)
        out = self._out()
        if lib().og_laplacian(self.h, _dp(v), _dp(out)) != 0:
            raise ValueError("oracle: the reference's Laplacian has no branch for coordsys %d" % self.coordsys)
        return out

    def sfilter(self, v):
        v = _f64(v)
        out = self._out()
        lib().og_filter3(self.h, OP_SF, _dp(v), _dp(out))
        return out

    def gfilter(self, v):
        v = _f64(v)
        out = self._out()
        lib().og_filter3(self.h, OP_GF, _dp(v), _dp(out))
        return out

    def gfilterdir(self, v, direction):
        return self.apply(OP_GF, direction, v)

    def sfilterdir(self, v, direction):
        return self.apply(OP_SF, direction, v)

    def ring(self, v, L=2):
        v = _f64(v)
        out = self._out()
        lib().og_ring(self.h, _dp(v), _dp(out), L)
        return out

    def ringv(self, f, g, h, L=1):
        f, g, h = _f64(f), _f64(g), _f64(h)
        out = self._out()
        lib().og_ringv(self.h, _dp(f), _dp(g), _dp(h), _dp(out), L)
        return out

    def grad(self, v):
        v = _f64(v)
        gx, gy, gz = self._out(), self._out(), self._out()
        lib().og_grad(self.h, _dp(v), _dp(gx), _dp(gy), _dp(gz))
        return gx, gy, gz

    def div(self, fx, fy, fz):
        fx, fy, fz = _f64(fx), _f64(fy), _f64(fz)
        out = self._out()
        lib().og_div(self.h, _dp(fx), _dp(fy), _dp(fz), _dp(out))
        return out

    def divt(self, *f):
        """divT of the nine components fxx fxy fxz fyx fyy fyz fzx fzy fzz -> [dfx, dfy, dfz]."""
        fs = [_f64(x) for x in f]
        outs = [self._out() for _ in range(3)]
        fa = (ctypes.POINTER(ctypes.c_double) * 9)(*[_dp(x) for x in fs])
        oa = (ctypes.POINTER(ctypes.c_double) * 3)(*[_dp(x) for x in outs])
        lib().og_divt(self.h, fa, oa)
        return outs

    def mesh(self, which):
        """0-2 coordinates, 3-5 d1 d2 d3, 6 GridLen, 7 CellVol, 8-9 CellVolS/G,
        10 det J, 11-19 the inverse Jacobian dA/dx .. dC/dz (curvilinear)."""
        out = self._out()
        if lib().og_mesh(self.h, which, _dp(out)) != 0:
            raise ValueError("oracle: mesh quantity %d is not defined on this grid" % which)
        return out

    def set_mesh_x3(self, x, y, z, mesh_periodic=True):
        """setup_mesh_x3 (parcop.f90:73-81): the coordinates of a curvilinear grid."""
        x, y, z = _f64(x), _f64(y), _f64(z)
        if lib().og_set_mesh_x3(self.h, _dp(x), _dp(y), _dp(z), 1 if mesh_periodic else 0) != 0:
            raise ValueError("oracle: set_mesh_x3 needs a curvilinear grid")

    def spacing(self):
        pd = (ctypes.c_double * 3)()
        md = (ctypes.c_double * 3)()
        lib().og_spacing(self.h, pd, md)
        return list(pd), list(md)

    def dense(self, op, direction):
        n = self.shape[direction]
        D = numpy.zeros((n, n), dtype=numpy.float64)
        rc = lib().og_dense(self.h, op, direction, _dp(D))
        if rc != 0:
            raise ValueError("oracle: null operator")
        return D


def set_threads(t):
    lib().og_set_threads(int(t))


def threads():
    return int(lib().og_threads())


# ---------------------------------------------------------------------------
# String translator: pyrandaUtils.py:22-141
# ---------------------------------------------------------------------------
def find_var_scalar(string):
    out = []
    for nv in re.findall(":.*?:", string):
        if not any(ch in nv for ch in "[]{}#%*@"):
            out.append(nv.replace(":", ""))
    return out


def find_var_vector(string):
    return [s.replace(":[", "").replace("]:", "") for s in re.findall(r":\[.*?\]:", string)]


def find_var(string, kind, unique=True):
    v = find_var_scalar(string) if kind == "scalar" else find_var_vector(string)
    return list(set(v)) if unique else v


def fortran3d(form, smap):
    form = form.replace(" ", "").strip()
    var_data = 'self.variables["%s"].data'
    for ivar in find_var(form, "scalar"):
        k = ":%s:" % ivar
        if k not in smap:
            smap[k] = var_data % ivar
    for ivar in find_var(form, "vector"):
        k = ":[%s]:" % ivar
        if k not in smap:
            smap[k] = var_data % ivar
    for m in smap:
        form = form.replace(m, smap[m])
    return form


def split_lines(s):
    lines = [el.replace(" ", "") for el in s.split("\n") if el]
    lines = [el for el in lines if el]
    return [el for el in lines if el.strip()[0] != "#"]


class _Var:
    def __init__(self, name):
        self.name = name
        self.data = None

    def sum(self):
        return float(numpy.sum(self.data))


class _Eq:
    """pyrandaEq.py:16-48"""

    def __init__(self, eqstr, smap):
        self.eqstr = eqstr
        self.kind = "ALG"
        self.rank = 1
        if "=" in eqstr:
            self.LHS = find_var(eqstr.split("=")[0], "scalar", unique=False)
            self.rank = len(self.LHS)
        else:
            self.LHS = None
        srhs = fortran3d(eqstr.split("=")[1] if self.LHS else eqstr, smap)
        self.RHS = eval("lambda self: " + srhs, _EVAL_GLOBALS)
        if "ddt(" in eqstr:
            self.kind = "PDE"


class _Timestep:
    """pyrandaTimestep.py:42-77"""

    name = "Timestep"

    def __init__(self, sim):
        self.sim = sim
        self.sMap = {"dt.courant(": "self.packages['Timestep'].courant(",
                     "dt.diff(": "self.packages['Timestep'].diff(",
                     "dt.diffDir(": "self.packages['Timestep'].diffDir("}

    def courant(self, u, v, w, c):
        s = self.sim
        if s.coordsys == 3:  # pyrandaTimestep.py:45-56: speeds along the A and B grid lines
            dAdx, dAdy, dBdx, dBdy = s.getVar("dAx"), s.getVar("dAy"), s.getVar("dBx"), s.getVar("dBy")
            magA = numpy.sqrt(dAdx * dAdx + dAdy * dAdy)
            magB = numpy.sqrt(dBdx * dBdx + dBdy * dBdy)
            uA = (u * dAdx + v * dAdy) / magA
            uB = (u * dBdx + v * dBdy) / magB
            vrate = numpy.abs(uA) / s.d1 + numpy.abs(uB) / s.d2
        else:
            vrate = numpy.abs(u) / s.d1 + numpy.abs(v) / s.d2 + numpy.abs(w) / s.d3
        crate = numpy.abs(c) / s.GridLen
        return 1.0 / numpy.max(vrate + crate)

    def diff(self, bulk, density):
        delta = self.sim.GridLen
        drate = density * delta * delta / numpy.maximum(1.0e-12, bulk)
        return numpy.min(drate)

    def diffDir(self, bulk, density, delta):
        drate = density * delta * delta / numpy.maximum(1.0e-12, bulk)
        return numpy.min(drate)


class _BC:
    """pyrandaBC.py on one rank: extrap / const (:58-160), field (:162-187),
    slip (:190-465), exit (:468-521), farfield (:524-745), symm (:748-788).
    A boundary is owned when its direction is non-periodic and has more than
    one point.  slip and farfield take the boundary normal from the cross
    product of the metric rows (:198-264): on curvilinear grids from the
    inverse Jacobian; on the others d(x,y,z)/d(A,B,C) = diag(dx, dy, dz)
    gives +x on the x ends, -y on the y ends, +z on the z ends."""

    name = "BC"
    NORMAL = {"x": (1.0, 0.0, 0.0), "y": (0.0, -1.0, 0.0), "z": (0.0, 0.0, 1.0)}

    def __init__(self, sim):
        self.sim = sim
        self.BCdata = {}
        self.sMap = {"bc.extrap(": "self.packages['BC'].extrap(",
                     "bc.const(": "self.packages['BC'].const(",
                     "bc.exit(": "self.packages['BC'].exitbc(",
                     "bc.slip(": "self.packages['BC'].slipbc(",
                     "bc.field(": "self.packages['BC'].applyBC('field',",
                     "bc.farfield(": "self.packages['BC'].farfieldbc(",
                     "bc.symm(": "self.packages['BC'].symm("}

    def _owns(self, d):
        ax = "xyz".index(d[0])
        return self.sim.shape[ax] > 1 and not self.sim.options["periodic"][ax]

    def applyBC(self, func, var, direction, val=None):
        f = getattr(self, func)
        for d in (direction if isinstance(direction, list) else [direction]):
            for v in (var if isinstance(var, list) else [var]):
                if val is not None:
                    f(v, d, val)
                else:
                    f(v, d)

    def field(self, var, d, field):
        if d[0] == "z" or not self._owns(d):
            return
        k = 0 if d[1] == "1" else -1
        self.sim.variables[var].data[self._slice(d, k)] = field[self._slice(d, k)]

    @staticmethod
    def BENO(u1, u2, u3, norm):
        d1 = u2 - u1
        d2 = (2.0 * u2 - u3) - u1
        beno = numpy.where(numpy.abs(d1) <= numpy.abs(d2), u1 + d1, u1 + d2)
        beno = numpy.where(d1 * d2 <= 0.0, u1, beno)
        if norm:
            beno = numpy.maximum(numpy.minimum(beno, numpy.maximum(0.0, u2)), numpy.minimum(0.0, u2))
        return beno

    def exitbc(self, var, direction, norm=False):
        for d in (direction if isinstance(direction, list) else [direction]):
            for v in (var if isinstance(var, list) else [var]):
                if d[0] == "z" or not self._owns(d):
                    continue
                a = self.sim.variables[v].data
                k = (0, 1, 2) if d[1] == "1" else (-1, -2, -3)
                a[self._slice(d, k[0])] = self.BENO(a[self._slice(d, k[0])], a[self._slice(d, k[1])],
                                                    a[self._slice(d, k[2])], norm)

    def symm(self, var, direction, anti=False, npts=4):
        m = -1.0 if anti else 1.0
        for d in (direction if isinstance(direction, list) else [direction]):
            for v in (var if isinstance(var, list) else [var]):
                if not self._owns(d):
                    continue
                a = self.sim.variables[v].data
                ax = "xyz".index(d[0])
                n = a.shape[ax]
                dst, src = (0, npts) if d[1] == "1" else (n - npts, n - 2 * npts)
                a[self._slice(d, slice(dst, dst + npts))] = numpy.flip(
                    a[self._slice(d, slice(src, src + npts))], axis=ax) * m

    def slipbc(self, var, direction):
        """pyrandaBC.py:190-196: each entry of var is one velocity (a list of its
        component names; a single name is a one-component velocity)."""
        for d in (direction if isinstance(direction, list) else [direction]):
            for v in (var if isinstance(var, list) else [var]):
                self._slip(v if isinstance(v, list) else [v], d)

    def _slip(self, velocity, d):
        if d[0] == "z":
            return
        self.extrap(velocity, d, 2)
        if not self._owns(d):
            return
        k = 0 if d[1] == "1" else -1
        nrm = self.normal(d, k)
        planes = [self.sim.variables[v].data[self._slice(d, k)].copy() for v in velocity]
        udotn = 0.0
        for q, u in enumerate(planes):
            udotn = udotn + u * nrm[q]
        mag0 = 0.0
        for u in planes:
            mag0 += u ** 2
        mag0 = numpy.sqrt(mag0)
        new = [u - udotn * nrm[q] for q, u in enumerate(planes)]
        magf = 0.0
        for u in new:
            magf += u ** 2
        magf = numpy.sqrt(magf)
        for v, u in zip(velocity, new):
            self.sim.variables[v].data[self._slice(d, k)] = numpy.where(magf > mag0, u * mag0 / magf, u)

    def normal(self, d, k):
        """The unit normal (n1, n2, n3) on plane k of boundary d (pyrandaBC.py:233-264):
        the cross product of the metric rows d(x,y,z)/d(.) of the two tangential grid
        directions, the metric rows rebuilt from the inverse Jacobian and det J (:198-231)."""
        if self.sim.coordsys != 3:
            return self.NORMAL[d[0]]
        key = "normal-%s" % d
        if key not in self.BCdata:
            g = self.sim.getVar
            dAdx, dAdy, dAdz = g("dAx"), g("dAy"), g("dAz")
            dBdx, dBdy, dBdz = g("dBx"), g("dBy"), g("dBz")
            dCdx, dCdy, dCdz = g("dCx"), g("dCy"), g("dCz")
            detJ = g("dtJ")
            m = {"xA": (-dBdz * dCdy + dBdy * dCdz) * detJ, "xB": (dAdz * dCdy - dAdy * dCdz) * detJ,
                 "xC": (-dAdz * dBdy + dAdy * dBdz) * detJ, "yA": (dBdz * dCdx - dBdx * dCdz) * detJ,
                 "yB": (-dAdz * dCdx + dAdx * dCdz) * detJ, "yC": (dAdz * dBdx - dAdx * dBdz) * detJ,
                 "zA": (-dBdy * dCdx + dBdx * dCdy) * detJ, "zB": (dAdy * dCdx - dAdx * dCdy) * detJ,
                 "zC": (-dAdy * dBdx + dAdx * dBdy) * detJ}
            t1, t2 = {"x": ("B", "C"), "y": ("A", "C"), "z": ("A", "B")}[d[0]]
            a1, a2, a3 = m["x" + t1], m["y" + t1], m["z" + t1]
            b1, b2, b3 = m["x" + t2], m["y" + t2], m["z" + t2]
            n1 = (a2 * b3 - a3 * b2)
            n2 = -(a1 * b3 - a3 * b1)
            n3 = (a1 * b2 - a2 * b1)
            mag = numpy.sqrt(n1 * n1 + n2 * n2 + n3 * n3)
            n1 /= mag
            n2 /= mag
            n3 /= mag
            self.BCdata[key] = [a[self._slice(d, k)] for a in (n1, n2, n3)]
        return self.BCdata[key]

    def Reimann(self, d, Rhoref, Uref, Vref, Wref, Pref, gamma, rhoi, Ui, Vi, Wi, Pi):
        nx, ny, nz = self.normal(d, 0 if d[1] == "1" else -1)
        Vni = Ui * nx + Vi * ny + Wi * nz
        Vno = Uref * nx + Vref * ny + Wref * nz
        SSo = numpy.sqrt(gamma * Pref / Rhoref)
        SSi = numpy.sqrt(gamma * Pi / rhoi)
        tmp = numpy.sqrt(Ui ** 2 + Vi ** 2 + Wi ** 2) / SSi
        Rplus = numpy.where(tmp >= 1.0, Vno + 2.0 * SSo / (gamma - 1.0), Vni + 2.0 * SSi / (gamma - 1.0))
        Rminus = numpy.where(tmp >= 1.0, Vni - 2.0 * SSi / (gamma - 1.0), Vno - 2.0 * SSo / (gamma - 1.0))
        Vnormal = (Rminus + Rplus) * 0.5
        SSb = (Rplus - Rminus) * (gamma - 1.0) * 0.25
        Ub = numpy.where(Vnormal >= 0.0, Ui + (Vnormal - Vni) * nx, Uref + (Vnormal - Vno) * nx)
        Vb = numpy.where(Vnormal >= 0.0, Vi + (Vnormal - Vni) * ny, Vref + (Vnormal - Vno) * ny)
        Wb = numpy.where(Vnormal >= 0.0, Wi + (Vnormal - Vni) * nz, Wref + (Vnormal - Vno) * nz)
        aux = 1.0 / (gamma - 1.0)
        rhob = numpy.where(Vnormal >= 0.0, ((rhoi ** gamma * SSb ** 2) / (gamma * Pi)) ** aux,
                           ((Rhoref ** gamma * SSb ** 2) / (gamma * Pref)) ** aux)
        Pb = rhob * SSb ** 2 / gamma
        Etb = Pb / (gamma - 1.0) + 0.5 * rhob * (Ub * Ub + Vb * Vb + Wb * Wb)
        return rhob, Ub, Vb, Wb, Etb, Pb

    def farfieldbc(self, direction):
        for d in (direction if isinstance(direction, list) else [direction]):
            ref = self.BCdata["farfield-properties-%s" % d]
            if not self._owns(d):
                continue
            names = [ref[k] for k in ("rho", "u", "v", "w", "p")]
            b, i = (0, 1) if d[1] == "1" else (-1, -2)
            inner = [self.sim.variables[v].data[self._slice(d, i)].copy() for v in names]
            out = self.Reimann(d, ref["rho0"], ref["u0"], ref["v0"], ref["w0"], ref["p0"], ref["gamma"], *inner)
            for v, val in zip(names, (out[0], out[1], out[2], out[3], out[5])):
                self.sim.variables[v].data[self._slice(d, b)] = val

    @staticmethod
    def _slice(direction, k):
        ax = "xyz".index(direction[0])
        idx = [slice(None)] * 3
        idx[ax] = k
        return tuple(idx)

    def extrap(self, var, direction, order=2):
        var = var if isinstance(var, list) else [var]
        direction = direction if isinstance(direction, list) else [direction]
        for d in direction:
            for v in var:
                a = self.sim.variables[v].data
                if self.sim.shape["xyz".index(d[0])] <= 1:
                    continue
                if d[1] == "1":
                    t, s1, s2 = 0, 1, 2
                else:
                    t, s1, s2 = -1, -2, -3
                if order == 2:
                    a[self._slice(d, t)] = 2 * a[self._slice(d, s1)] - a[self._slice(d, s2)]
                else:
                    a[self._slice(d, t)] = a[self._slice(d, s1)]

    def const(self, var, direction, val):
        var = var if isinstance(var, list) else [var]
        direction = direction if isinstance(direction, list) else [direction]
        for d in direction:
            for v in var:
                if self.sim.shape["xyz".index(d[0])] <= 1:
                    continue
                a = self.sim.variables[v].data
                a[self._slice(d, 0 if d[1] == "1" else -1)] = val


_EVAL_GLOBALS = {"numpy": numpy}
try:
    import scipy.special  # noqa: F401  (erf in the sMap)
    import scipy
    _EVAL_GLOBALS["scipy"] = scipy
except Exception:  # pragma: no cover
    pass


def default_mesh_options():
    """pyrandaMesh.py:214-233"""
    return {"x1": [0.0, 0.0, 0.0], "xn": [1, 1, 1], "nn": [1, 1, 1],
            "periodic": [False, False, False], "symmetric": [[False, False], [False, False], [False, False]],
            "coordsys": 0}


class OracleSim:
    """numpy restatement of pyrandaSim (pyranda.py) on the oracle operators."""

    def __init__(self, name, mesh_str):
        self.name = name
        opts = default_mesh_options()

        def set_options(ind, x1, xn, nn, periodic=False):
            opts["x1"][ind] = x1
            opts["xn"][ind] = xn
            opts["nn"][ind] = nn
            opts["periodic"][ind] = periodic

        if isinstance(mesh_str, dict):  # a mesh_options dictionary (pyrandaMesh.py:214-233)
            for k, v in mesh_str.items():
                opts[k] = v
        else:
            msmap = {"xdom=(": "set_options(0,", "ydom=(": "set_options(1,", "zdom=(": "set_options(2,"}
            for line in split_lines(mesh_str):
                exec(fortran3d(line, dict(msmap)), {"set_options": set_options, "numpy": numpy})
        self.options = opts
        self.nx, self.ny, self.nz = opts["nn"]
        self.npts = self.nx * self.ny * self.nz
        self.dx = (opts["xn"][0] - opts["x1"][0]) / max(self.nx - 1, 1)
        self.dy = (opts["xn"][1] - opts["x1"][1]) / max(self.ny - 1, 1)
        self.dz = (opts["xn"][2] - opts["x1"][2]) / max(self.nz - 1, 1)
        self.shape = (self.nx, self.ny, self.nz)
        # pyrandaMPI.py:101-131: symmetric ends of non-periodic directions are SYMM
        sym = opts.get("symmetric", [[False, False]] * 3)
        bc = [["SYMM" if (sym[d][e] and not opts["periodic"][d]) else "NONE" for e in range(2)] for d in range(3)]
        self.coordsys = int(opts.get("coordsys", 0))
        self.grid = OracleGrid(self.shape, opts["periodic"], opts["x1"], opts["xn"], bc=bc,
                               coordsys=self.coordsys)
        if self.coordsys == 3:
            self.grid.set_mesh_x3(*self._curvilinear_coords(opts), mesh_periodic=opts.get("periodicGrid", True))
        # pyrandaMesh.py:143-191: the mesh coordinates in x-y-z space; the native
        # (r, theta, z) or (r, theta, phi) ones are kept beside them
        x, y, z = self.grid.mesh(0), self.grid.mesh(1), self.grid.mesh(2)
        self.coordsNative = None
        if self.coordsys in (1, 2, 4):
            self.coordsNative = [x, y, z]
            if self.coordsys == 1:
                x, y = x * numpy.cos(y), x * numpy.sin(y)
            else:
                r, th, phi = x, y, z
                x = r * numpy.sin(th) * numpy.cos(phi)
                y = r * numpy.sin(th) * numpy.sin(phi)
                z = r * numpy.cos(th)
        self.meshx, self.meshy, self.meshz = x, y, z
        self.d1 = self.grid.mesh(3)
        self.d2 = self.grid.mesh(4)
        self.d3 = self.grid.mesh(5)
        self.GridLen = self.grid.mesh(6)
        self.zero = numpy.zeros(self.shape, order="F")
        self.equations = []
        self.conserved = []
        self.variables = {}
        self.packages = {}
        self.nPDE = 0
        self.time = 0.0
        self.deltat = 0.0
        self.cycle = 0
        self._smap()

    def _curvilinear_coords(self, opts):
        """pyrandaMesh.py:92-131: node coordinates numpy.linspace(x1, xn, nn) per
        direction, replaced point by point by opts['function'](i, j, k) when given."""
        lin = [numpy.linspace(opts["x1"][d], opts["xn"][d], num=self.shape[d]) for d in range(3)]
        x, y, z = [numpy.asfortranarray(a) for a in numpy.meshgrid(*lin, indexing="ij")]
        fn = opts.get("function")
        if fn:
            for i in range(self.nx):
                for j in range(self.ny):
                    for k in range(self.nz):
                        x[i, j, k], y[i, j, k], z[i, j, k] = fn(i, j, k)
        return x, y, z

    # pyrandaMPI.py:657-661 / parcop.f90:84-128
    _VARS = {"x": 0, "y": 1, "z": 2, "d1": 3, "d2": 4, "d3": 5, "dtJ": 10, "dAx": 11, "dAy": 12, "dAz": 13,
             "dBx": 14, "dBy": 15, "dBz": 16, "dCx": 17, "dCy": 18, "dCz": 19}

    def getVar(self, name):
        return self.grid.mesh(self._VARS[name])

    # pyranda.py:812-869
    def _smap(self):
        s = {}
        s["div("] = "self.div("
        s["ddx("] = "self.ddx("
        s["ddy("] = "self.ddy("
        s["ddz("] = "self.ddz("
        s["fbar("] = "self.filter("
        s["gbar("] = "self.gfilter("
        s["gbarx("] = "self.gfilterx("
        s["gbary("] = "self.gfiltery("
        s["gbarz("] = "self.gfilterz("
        s["grad("] = "self.grad("
        s["simtime"] = "self.time"
        s["deltat"] = "self.deltat"
        s["divT("] = "self.divT("
        s["lap("] = "self.laplacian("
        s["ring("] = "self.ring("
        s["ringV("] = "self.ringV("
        s["dd4x("] = "self.dd4x("
        s["dd4y("] = "self.dd4y("
        s["dd4z("] = "self.dd4z("
        s["dd8x("] = "self.dd8x("
        s["dd8y("] = "self.dd8y("
        s["dd8z("] = "self.dd8z("
        s["sum("] = "self.sum3D("
        s["mean("] = "1.0/float(self.npts) * self.sum3D("
        s["sign("] = "numpy.sign("
        s["dot("] = "numpy.dot("
        s["abs("] = "numpy.abs("
        s["sqrt("] = "numpy.sqrt("
        s["sin("] = "numpy.sin("
        s["cos("] = "numpy.cos("
        s["tanh("] = "numpy.tanh("
        s["exp("] = "numpy.exp("
        s["where("] = "numpy.where("
        s["max("] = "self.max3D("
        s["min("] = "self.min3D("
        s["3d("] = "self.emptyScalar("
        s["pi"] = "numpy.pi"
        s["gridLen"] = "self.GridLen"
        s["erf("] = "scipy.special.erf("
        s["meshx"] = "self.meshx"
        s["meshy"] = "self.meshy"
        s["meshz"] = "self.meshz"
        s["meshVar("] = "self.getVar("
        self.sMap = s

    def addPackage(self, kind):
        pkg = _Timestep(self) if kind == "Timestep" else _BC(self)
        self.packages[pkg.name] = pkg
        self.sMap.update(pkg.sMap)

    def emptyScalar(self, val=0.0):
        return numpy.zeros(self.shape, order="F") + val

    def sum3D(self, a):
        return numpy.sum(a)

    def max3D(self, a):
        return numpy.max(a)

    def min3D(self, a):
        return numpy.min(a)

    def var(self, name):
        return self.variables[name]

    def eval(self, expr):
        return eval(fortran3d(expr, self.sMap), _EVAL_GLOBALS, {"self": self})

    # pyranda.py:607-736
    def apply_sym(self, op, direction, sym, v):
        """The operator variant for symmetric (+1) or antisymmetric (-1) fields at a SYMM end."""
        v = _f64(v)
        out = self._out()
        lib().og_apply_sym(self.h, op, direction, int(sym), _dp(v), _dp(out))
        return out

    def filter_sym(self, op, sym, v):
        """x -> y -> z filter (op 2 compact, 3 Gaussian) with one variant sign per direction."""
        v = _f64(v)
        out = self._out()
        s3 = (ctypes.c_int * 3)(*[int(x) for x in sym])
        lib().og_filter3_sym(self.h, op, s3, _dp(v), _dp(out))
        return out

    def ddx(self, v):
        return 0.0 if self.nx <= 1 else self.grid.ddx(v)

    def ddy(self, v):
        return 0.0 if self.ny <= 1 else self.grid.ddy(v)

    def ddz(self, v):
        return 0.0 if self.nz <= 1 else self.grid.ddz(v)

    def dd4x(self, v):
        return self.grid.dd4(0, v)

    def dd4y(self, v):
        return self.grid.dd4(1, v)

    def dd4z(self, v):
        return self.grid.dd4(2, v)

    def laplacian(self, v):
        return self.grid.laplacian(v)

    def divT(self, fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz):
        z = self.zero
        f = [x if isinstance(x, numpy.ndarray) else z + x for x in (fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz)]
        return self.grid.divt(*f)

    def dd8x(self, v):
        return self.grid.dd8(0, v)

    def dd8y(self, v):
        return self.grid.dd8(1, v)

    def dd8z(self, v):
        return self.grid.dd8(2, v)

    def div(self, f1, f2=None, f3=None):
        z = self.zero
        if f2 is None and f3 is None:
            if self.nx > 1:
                return self.grid.div(f1, z, z)
            if self.ny > 1:
                return self.grid.div(z, f1, z)
            if self.nz > 1:
                return self.grid.div(z, z, f1)
            return 0.0
        if f3 is None:
            if self.nx > 1 and self.ny > 1:
                return self.grid.div(f1, f2, z)
            if self.nz > 1 and self.ny > 1:
                return self.grid.div(z, f1, f2)
            if self.nz > 1 and self.nx > 1:
                return self.grid.div(f1, z, f2)
            if self.nx > 1:
                return self.grid.div(f1, z, z)
            if self.ny > 1:
                return self.grid.div(z, f1, z)
            if self.nz > 1:
                return self.grid.div(z, z, f1)
            return 0.0
        return self.grid.div(f1, f2, f3)

    def grad(self, v):
        return list(self.grid.grad(v))

    def ring(self, v):
        return self.grid.ring(v, 2)

    def ringV(self, vx, vy, vz):
        return self.grid.ringv(vx, vy, vz, 1)

    def filter(self, v):
        return self.grid.sfilter(v)

    def gfilter(self, v):
        return self.grid.gfilter(v)

    def gfilterx(self, v):
        return self.grid.gfilterdir(v, 0)

    def gfiltery(self, v):
        return self.grid.gfilterdir(v, 1)

    def gfilterz(self, v):
        return self.grid.gfilterdir(v, 2)

    def _addvar(self, name):
        if name not in self.variables:
            v = _Var(name)
            v.data = self.emptyScalar()
            self.variables[name] = v

    # pyranda.py:231-285
    def EOM(self, eom, eomDict=None):
        if eomDict:
            for item in eomDict:
                eom = eom.replace(item, str(eomDict[item]))
        lines = [el for el in eom.split("\n") if el]
        lines = [el for el in lines if el.strip()[0] != "#"]
        names = []
        for eq in lines:
            names += find_var(eq, "scalar")
        for n in sorted(set(names)):
            self._addvar(n)
        for eq in lines:
            peq = _Eq(eq, self.sMap)
            self.equations.append(peq)
            if peq.kind == "PDE":
                self.nPDE += 1
                self.conserved.append(peq.LHS[0])

    # pyranda.py:305-370
    def setIC(self, ics, icDict=None):
        if icDict:
            for item in icDict:
                ics = ics.replace(item, str(icDict[item]))
        lines = split_lines(ics)
        names = []
        for eq in lines:
            names += find_var(eq, "scalar")
        for n in sorted(set(names)):
            self._addvar(n)
        ns = {"self": self}
        for ic in lines:
            exec(fortran3d(ic, self.sMap), _EVAL_GLOBALS, ns)
        self.updateVars()

    def updateFlux(self):
        flux = {}
        for eq in self.equations:
            if eq.kind == "PDE":
                flux[eq.LHS[0]] = eq.RHS(self)
        return flux

    def updateVars(self):
        for eq in self.equations:
            if eq.kind != "ALG":
                continue
            rhs = eq.RHS(self)
            if not eq.LHS:
                continue
            if eq.rank == 1:
                self.variables[eq.LHS[0]].data = rhs
            else:
                for ii in range(len(rhs)):
                    self.variables[eq.LHS[ii]].data = rhs[ii]

    # pyranda.py:758-810: Carpenter-Kennedy LSRK(5,4), ALG update after every stage
    ARK = [0.0, -6234157559845. / 12983515589748., -6194124222391. / 4410992767914.,
           -31623096876824. / 15682348800105., -12251185447671. / 11596622555746.]
    BRK = [494393426753. / 4806282396855., 4047970641027. / 5463924506627.,
           9795748752853. / 13190207949281., 4009051133189. / 8539092990294.,
           1348533437543. / 7166442652324.]
    ETA = [494393426753. / 4806282396855., 4702696611523. / 9636871101405.,
           3614488396635. / 5249666457482., 9766892798963. / 10823461281321., 1.0]

    def rk4(self, time, dt):
        phi = {U: numpy.zeros(self.shape, order="F") for U in self.conserved}
        time_i = time
        self.deltat = dt
        for ii in range(5):
            flux = self.updateFlux()
            for U in self.conserved:
                tmp1 = self.ARK[ii] * phi[U]
                phi[U] = dt * flux[U] + tmp1
                tmp2 = self.BRK[ii] * phi[U]
                self.variables[U].data = self.variables[U].data + tmp2
            time = time_i + self.ETA[ii] * dt
            self.time = time
            self.updateVars()
        self.cycle += 1
        return time
