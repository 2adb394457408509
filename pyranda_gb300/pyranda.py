"""pyrandaSim on one GB300: the EOM/setIC/rk4/ddx/filter API of pyranda.

Mirrors pyranda/pyranda.py (class pyrandaSim) with device-resident fields:
every variable's ``data`` is a torch float64 tensor of shape (nx, ny, nz) in
Fortran order on the GPU, the compact operators run in ``libpyranda_gpu.so``,
the LSRK(5,4) update is one fused kernel per stage, and global reductions
(``sum``/``max``/``min`` and the time-step limits) return device scalars so a
whole RK step can be recorded in a CUDA graph (``pyrandaSim.use_graphs``).
"""
import gc
import math
import os

import numpy
import torch

from . import pgmath
from ._lib import PG_DIR_ALL
from .fuse import RK_DONE
from .grid import Grid, flush_pending
from .pyrandaUtils import findVar, fortran3d, splitLines

# LSRK(5,4) of Carpenter & Kennedy (pyranda.py:760-779)
ARK = [0.0, -6234157559845. / 12983515589748., -6194124222391. / 4410992767914.,
       -31623096876824. / 15682348800105., -12251185447671. / 11596622555746.]
BRK = [494393426753. / 4806282396855., 4047970641027. / 5463924506627.,
       9795748752853. / 13190207949281., 4009051133189. / 8539092990294.,
       1348533437543. / 7166442652324.]
ETA = [494393426753. / 4806282396855., 4702696611523. / 9636871101405.,
       3614488396635. / 5249666457482., 9766892798963. / 10823461281321., 1.0]

EVAL_GLOBALS = {"numpy": pgmath, "scipy": pgmath.scipy, "torch": torch, "math": math}


def _num(x):
    """A Python number from a number or a 0-d tensor."""
    if isinstance(x, torch.Tensor):
        return float(x.reshape(-1)[0].item())
    return float(x) if x is not None else 0.0


def pyrandaRestart(rootname, suffix=None, precision="fp64", device=None):
    """pyranda.py:979-1072: a pyrandaSim from a restart (this library's or the reference's).

    Returns [pysim, local_vars] as the reference does.  Packages are mapped
    by module name onto this library's (pyrandaTimestep, pyrandaBC).
    """
    from . import restart
    from .pyrandaBC import pyrandaBC
    from .pyrandaTimestep import pyrandaTimestep
    dump = restart.find_dump(rootname, suffix)
    serial = restart.read_serial(dump)
    local = {}
    if "local_vars" in serial:
        lv = serial.pop("local_vars")
        for name, fn in lv.pop("numpyArrays", {}).items():
            local[name] = numpy.load(fn + ".npy")
        local.update(lv)
    sim = pyrandaSim(rootname, serial["mesh"], precision=precision, device=device)
    known = {"pyrandaTimestep": pyrandaTimestep, "pyrandaBC": pyrandaBC}
    for pack in serial["packages"]:
        base = pack.split(".")[-1]
        if base not in known:
            raise ValueError("restart needs package %s, which this library does not provide" % pack)
        sim.addPackage(known[base](sim))
    sim.sMap = serial["sMap"]
    sim.EOM(serial["EOM"])
    sim.setIC(serial["ICs"], addOnly=True)
    sim.time = serial["time"]
    sim.deltat = serial["deltat"]
    sim.cycle = serial["cycle"]
    sim.vizDumpHistory = serial.get("vizDumpHistory", [])
    data = restart.read_blocks(dump, serial, (sim.nx, sim.ny, sim.nz))
    scalars = set(serial.get("scalars", []))
    pyscalars = set(serial.get("pyscalars", []))
    for name in serial["vars"]:
        if name in sim.variables:
            if name in pyscalars:
                sim.variables[name].data = float(data[name].flat[0])
            elif name in scalars:
                sim.variables[name].data = torch.full((), float(data[name].flat[0]), dtype=torch.float64,
                                                      device=sim.grid.device)
            else:
                sim.variables[name].data = sim.grid.field(numpy.ascontiguousarray(data[name]))
    if sim.mesh.coordsys == 3 and all(k in serial["vars"] for k in ("meshx", "meshy", "meshz")):
        # pyranda.py:1064-1069: a curvilinear mesh is rebuilt from the coordinates the
        # restart holds, and the packages start again on it
        sim._set_curvilinear(*[sim.variables[k].data for k in ("meshx", "meshy", "meshz")])
        for pk in sim.packages.values():
            pk.__init__(sim)
            pk.get_sMap()
    return [sim, local]


def defaultMeshOptions():
    """pyranda/pyrandaMesh.py:214-233"""
    return {"x1": [0.0, 0.0, 0.0], "xn": [1, 1, 1], "nn": [1, 1, 1],
            "periodic": [False, False, False], "periodicGrid": True,
            "symmetric": [[False, False], [False, False], [False, False]],
            "dim": 1, "coordsys": 0, "function": None, "id": 0, "pn": [0, 0, 0]}


class pyrandaVar:
    """pyranda/pyrandaVar.py: a named field with global reductions."""

    def __init__(self, name, kind=None, rank="scalar"):
        self.name = name
        self.kind = kind
        self.rank = rank
        self.data = None
        self.allocated = False
        self.sim = None

    def __allocate__(self, sim):
        if self.allocated:
            return
        self.sim = sim
        self.data = sim.emptyScalar()
        self.allocated = True

    def _reduce(self, op, data=None):
        d = self.data if data is None else data
        return self.sim.grid.reduce_value(op, d)

    def sum(self, axis=None, idata=None):
        d = self.data if idata is None else idata
        if axis is None:
            return self._reduce(0, d)
        return self.sim.PyMPI._axis_sum(d, axis)

    def mean(self, axis=None, idata=None):
        s = self.sum(axis=axis, idata=idata)
        if axis is None:
            return s / self.sim.grid.member_points
        s = numpy.asarray(s)
        return s * s.size / float(self.sim.npts)

    def var(self, axis=None):
        bar = self.mean(axis=axis)
        bar2 = self.mean(axis=axis, idata=self.data ** 2)
        return bar2 - bar * bar

    def numpy(self):
        """Host copy (numpy, F-ordered) of the device field."""
        d = self.data
        if isinstance(d, torch.Tensor):
            return numpy.asfortranarray(d.detach().cpu().numpy())
        return d

    def __getitem__(self, given):
        return numpy.squeeze(self.numpy()[given])


class pyrandaEq:
    """pyranda/pyrandaEq.py:16-48: one EOM line compiled to a lambda."""

    def __init__(self, eqstr, sMap):
        self.eqstr = eqstr
        self.kind = "ALG"
        self.active = True
        self.rank = 1
        if "=" in eqstr:
            self.LHS = findVar(eqstr.split("=")[0], "scalar", unique=False)
            self.rank = len(self.LHS)
        else:
            self.LHS = None
        srhs = fortran3d(eqstr.split("=")[1] if self.LHS else eqstr, sMap)
        self.sRHS = srhs
        self.RHS = eval("lambda self: " + srhs, EVAL_GLOBALS)
        if "ddt(" in eqstr:
            self.kind = "PDE"


class _Mesh:
    """Mesh data of pyrandaMesh (pyranda/pyrandaMesh.py:58-208), Cartesian."""

    def __init__(self):
        self.options = {}
        self.coords = None
        self.shape = None
        self.coordsys = 0


class pyrandaGPU:
    """The single-GPU counterpart of pyrandaMPI: reductions and layout helpers.

    One rank owns the whole grid, so every processor-boundary flag is true and
    the reductions of pyrandaMPI.py:307-326 are device reductions.
    """

    def __init__(self, sim):
        self.sim = sim
        self.grid = sim.grid
        self.nx, self.ny, self.nz = sim.nx, sim.ny, sim.nz
        self.ax, self.ay, self.az = sim.nx, sim.ny, sim.nz
        self.px = self.py = self.pz = 1
        self.master = True
        self.periodic = sim.meshOptions["periodic"]
        per = self.periodic
        self.x1proc = self.xnproc = (not per[0]) and self.nx > 1
        self.y1proc = self.ynproc = (not per[1]) and self.ny > 1
        self.z1proc = self.znproc = (not per[2]) and self.nz > 1
        self.chunk_3d_lo = numpy.zeros(3, dtype=numpy.int32)
        self.chunk_3d_hi = numpy.array([self.nx - 1, self.ny - 1, self.nz - 1], dtype=numpy.int32)
        self.chunk_3d_size = numpy.array([self.nx, self.ny, self.nz], dtype=numpy.int32)

    def setPatch(self):
        """parcop kept one active patch; every call here names its grid, so this is a no-op."""

    def emptyScalar(self):
        return self.grid.zeros()

    def sum3D(self, data):
        return self.grid.reduce(0, data) if isinstance(data, torch.Tensor) else data * self.sim.npts

    def max3D(self, data):
        return self.grid.reduce(1, data) if isinstance(data, torch.Tensor) else data

    def min3D(self, data):
        return self.grid.reduce(2, data) if isinstance(data, torch.Tensor) else data

    def mean3D(self, data):
        return self.sum3D(data) / float(self.sim.npts)

    def _axis_sum(self, data, axis):
        d = data if isinstance(data, torch.Tensor) else torch.as_tensor(data)
        if isinstance(axis, (tuple, list)):
            axis = tuple(axis)
        return d.sum(dim=axis).cpu().numpy()

    # pyrandaMPI.py:353-470 line/plane sums, returned on the host
    def xsum(self, data):
        return self._axis_sum(data, 0)

    def ysum(self, data):
        return self._axis_sum(data, 1)

    def zsum(self, data):
        return self._axis_sum(data, 2)

    def xysum(self, data):
        return self._axis_sum(data, (0, 1))

    def xzsum(self, data):
        return self._axis_sum(data, (0, 2))

    def yzsum(self, data):
        return self._axis_sum(data, (1, 2))

    xbar, ybar, zbar = xsum, ysum, zsum

    def subsum3xz(self, data):
        return self.xzsum(data)


class pyrandaSim:
    """pyranda/pyranda.py:34-131 on one GPU.

    Extra keyword arguments (not in the reference):
      precision: 'fp64' (reference arithmetic) or 'fp32' (single-precision
                 compact sweeps on FP64 fields; FP64 RK state and reductions)
      device:    torch device of the fields (default: current CUDA device)
    """

    def __init__(self, name, meshOptions, silent=False, precision="fp64", device=None):
        self.name = name
        self.silent = silent
        self.ioformat = "BINARY"   # viz dumps: "BINARY" or "ASCII" (pyrandaIO.py:25)
        self.vizDumpHistory = []
        self.mesh = _Mesh()
        if isinstance(meshOptions, str):
            meshOptions = self._parse_mesh(meshOptions)
        opts = defaultMeshOptions()
        opts.update(meshOptions)
        coordsys = int(opts.get("coordsys", 0))
        if coordsys not in (0, 1, 2, 3, 4):
            raise ValueError("coordsys %d is not one of pyranda's coordinate systems 0-4" % coordsys)
        # pyrandaMPI.py:101-131: a symmetric end of a non-periodic direction is SYMM, else NONE
        sym = opts["symmetric"]
        bc = tuple(tuple("SYMM" if (sym[d][e] and not opts["periodic"][d]) else "NONE" for e in range(2))
                   for d in range(3))
        self.meshOptions = opts
        self.mesh.options = opts
        self.mesh.coordsys = coordsys
        nx, ny, nz = [int(v) for v in opts["nn"]]
        self.nx, self.ny, self.nz = nx, ny, nz
        self.npts = nx * ny * nz
        self.dx = (opts["xn"][0] - opts["x1"][0]) / max(nx - 1, 1)
        self.dy = (opts["xn"][1] - opts["x1"][1]) / max(ny - 1, 1)
        self.dz = (opts["xn"][2] - opts["x1"][2]) / max(nz - 1, 1)
        self.precision = precision
        self.grid = Grid((nx, ny, nz), opts["periodic"], opts["x1"], opts["xn"], precision=precision, device=device,
                         bc=bc, coordsys=coordsys)
        self.PyMPI = pyrandaGPU(self)
        self.mesh.PyMPI = self.PyMPI
        self._make_mesh()
        self.zero = self.grid.zeros()
        self.equations = []
        self.conserved = []
        self.variables = {}
        self.initial_conditions = []
        self.nPDE = self.nALG = self.nELP = 0
        self.packages = {}
        self.userDefined = {}
        self.time = 0.0
        self.cycle = 0
        self.deltat = 0.0
        self._phi = None
        self._graph = None
        self._graphs_enabled = False
        self._fuse = None
        self._fuse_wanted = False
        self._fuse_arith = "fp64"
        self.get_sMap()

    # ------------------------------------------------------------ mesh set-up
    def _parse_mesh(self, mesh_str):
        """pyrandaMesh.makeMeshStr / set_options (pyranda/pyrandaMesh.py:33-49)."""
        opts = defaultMeshOptions()

        def set_options(ind, x1, xn, nn, periodic=False):
            opts["x1"][ind] = x1
            opts["xn"][ind] = xn
            opts["nn"][ind] = nn
            opts["periodic"][ind] = periodic

        smap = {"xdom=(": "set_options(0,", "ydom=(": "set_options(1,", "zdom=(": "set_options(2,"}
        ns = {"set_options": set_options, "numpy": numpy, "pi": math.pi}
        for line in splitLines(mesh_str):
            exec(fortran3d(line, dict(smap)), ns, ns)
        return opts

    def _curvilinear_coords(self):
        """pyrandaMesh.py:92-131: node coordinates numpy.linspace(x1, xn, nn) per
        direction, replaced point by point by meshOptions['function'](i, j, k)."""
        opts = self.meshOptions
        lin = [numpy.linspace(opts["x1"][d], opts["xn"][d], num=[self.nx, self.ny, self.nz][d]) for d in range(3)]
        x, y, z = numpy.meshgrid(*lin, indexing="ij")
        fn = opts.get("function")
        if fn:
            for i in range(self.nx):
                for j in range(self.ny):
                    for k in range(self.nz):
                        x[i, j, k], y[i, j, k], z[i, j, k] = fn(i, j, k)
        return x, y, z

    def _set_curvilinear(self, x, y, z):
        """setup_mesh_x3 with these coordinates, then the mesh quantities of the simulation."""
        g = self.grid
        g.set_mesh_coords(x, y, z, self.meshOptions.get("periodicGrid", True))
        if self.mesh.coords is not None:
            for i, c in enumerate(self.mesh.coords):
                c.data = g.mesh(i)
            self.mesh.d1, self.mesh.d2, self.mesh.d3 = g.mesh(3), g.mesh(4), g.mesh(5)
            self.mesh.GridLen, self.mesh.CellVol = g.mesh(6), g.mesh(7)

    def _make_mesh(self):
        g = self.grid
        if self.mesh.coordsys == 3:
            x, y, z = self._curvilinear_coords()
            self._set_curvilinear(x, y, z)
        self.mesh.coords = [pyrandaVar("x", "mesh"), pyrandaVar("y", "mesh"), pyrandaVar("z", "mesh")]
        for i, c in enumerate(self.mesh.coords):
            c.sim = self
            c.allocated = True
            c.data = g.mesh(i)
        # pyrandaMesh.py:151-191: coordinates in x-y-z space, the native ones kept beside them
        self.mesh.coordsNative = None
        if self.mesh.coordsys in (1, 2, 4):
            native = [g.mesh(i) for i in range(3)]
            self.mesh.coordsNative = native
            r, a, b = native
            if self.mesh.coordsys == 1:
                xyz = (r * torch.cos(a), r * torch.sin(a), b)
            else:
                xyz = (r * torch.sin(a) * torch.cos(b), r * torch.sin(a) * torch.sin(b), r * torch.cos(a))
            for c, v in zip(self.mesh.coords, xyz):
                c.data = g.field(v)
        self.mesh.shape = [self.nx, self.ny, self.nz]
        self.mesh.nn = self.meshOptions["nn"]
        self.mesh.d1 = g.mesh(3)
        self.mesh.d2 = g.mesh(4)
        self.mesh.d3 = g.mesh(5)
        self.mesh.GridLen = g.mesh(6)
        self.mesh.CellVol = g.mesh(7)
        ii = torch.arange(self.nx, dtype=torch.float64, device=g.device).view(-1, 1, 1)
        jj = torch.arange(self.ny, dtype=torch.float64, device=g.device).view(1, -1, 1)
        kk = torch.arange(self.nz, dtype=torch.float64, device=g.device).view(1, 1, -1)
        self.mesh.indices = []
        for name, a in (("iloc", ii), ("jloc", jj), ("kloc", kk)):
            v = pyrandaVar(name, "mesh")
            v.sim = self
            v.allocated = True
            v.data = g.field(a.expand(self.nx, self.ny, self.nz))
            self.mesh.indices.append(v)

    # ------------------------------------------------------------------- sMap
    def get_sMap(self):
        """pyranda.py:812-869 with the same keys; targets run on the device."""
        s = {}
        s["div("] = "self.div("
        s["divT("] = "self.divT("
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
        s["lap("] = "self.laplacian("
        s["ring("] = "self.ring("
        s["ringV("] = "self.ringV("
        s["dd4x("] = "self.dd4x("
        s["dd4y("] = "self.dd4y("
        s["dd4z("] = "self.dd4z("
        s["dd8x("] = "self.dd8x("
        s["dd8y("] = "self.dd8y("
        s["dd8z("] = "self.dd8z("
        s["sum("] = "self.PyMPI.sum3D("
        s["mean("] = "1.0/float(self.npts) * self.PyMPI.sum3D("
        s["mean3D("] = "self.PyMPI.mean3D("
        s["sign("] = "numpy.sign("
        s["dot("] = "numpy.dot("
        s["abs("] = "numpy.abs("
        s["sqrt("] = "numpy.sqrt("
        s["sin("] = "numpy.sin("
        s["cos("] = "numpy.cos("
        s["tanh("] = "numpy.tanh("
        s["exp("] = "numpy.exp("
        s["where("] = "numpy.where("
        s["max("] = "self.PyMPI.max3D("
        s["min("] = "self.PyMPI.min3D("
        s["3d("] = "self.emptyScalar("
        s["pi"] = "numpy.pi"
        s["gridLen"] = "self.mesh.GridLen"
        s["random3D()"] = "self.random3D()"
        s["erf("] = "scipy.special.erf("
        s["meshx"] = "self.mesh.coords[0].data"
        s["meshy"] = "self.mesh.coords[1].data"
        s["meshz"] = "self.mesh.coords[2].data"
        s["meshi"] = "self.mesh.indices[0].data"
        s["meshj"] = "self.mesh.indices[1].data"
        s["meshk"] = "self.mesh.indices[2].data"
        self.sMap = s

    def addPackage(self, package):
        self.packages[package.name] = package
        self.packagesRestart = getattr(self, "packagesRestart", [])
        base = type(package).__module__.rsplit(".", 1)[-1]
        self.packagesRestart.append("pyranda." + base)   # the reference's module name (pyranda.py:152)
        package.get_sMap()
        self.sMap.update(package.sMap)

    def addUserDefinedFunction(self, name, equation):
        self.userDefined[name] = equation
        self.sMap.update({"%s(" % name: "self.userDefined['%s'](self," % name})

    # -------------------------------------------------------------- variables
    def iprint(self, sprnt, wpm=0):
        if not self.silent:
            print(sprnt, flush=True)

    def allocate(self):
        for v in self.variables.values():
            v.__allocate__(self)

    def var(self, name):
        if name in self.variables:
            return self.variables[name]
        raise ValueError("Error: variable name: %s not found in database" % name)

    def x(self):
        return self.mesh.coords[0]

    def y(self):
        return self.mesh.coords[1]

    def z(self):
        return self.mesh.coords[2]

    def emptyScalar(self, val=0.0):
        t = self.grid.zeros()
        if val != 0.0:
            t.fill_(val)
        return t

    def random3D(self):
        t = self.grid.empty()
        t.uniform_()
        return t

    def eval(self, expression):
        return eval(fortran3d(expression, self.sMap), EVAL_GLOBALS, {"self": self})

    def parse(self, expression, parseDict=None):
        if parseDict:
            expression = self.updateStringFromDictionary(expression, parseDict, "parse")
        exec(fortran3d(expression, self.sMap), EVAL_GLOBALS, {"self": self})

    def addVar(self, name, kind=None, rank="scalar"):
        if name not in self.variables:
            self.variables[name] = pyrandaVar(name, kind, rank)

    def addEqu(self, equation):
        peq = pyrandaEq(equation, self.sMap)
        self.equations.append(peq)
        if peq.kind == "PDE":
            self.nPDE += 1
            self.conserved.append(peq.LHS[0])
            if len(peq.LHS) > 1:
                raise ValueError("only single return values for PDEs allowed")
        else:
            self.nALG += 1

    def updateStringFromDictionary(self, string, dictionary, handle):
        for item in dictionary:
            if item in string:
                string = string.replace(item, str(dictionary[item]))
        return string

    def EOM(self, eom, eomDict=False):
        """pyranda.py:231-285"""
        if eomDict:
            eom = self.updateStringFromDictionary(eom, eomDict, "EOM")
        self.eom = eom
        lines = [el for el in eom.split("\n") if el]
        lines = [el for el in lines if el.strip() and el.strip()[0] != "#"]
        names = []
        for eq in lines:
            names += findVar(eq, "scalar")
        for v in sorted(set(names)):
            self.addVar(v, kind="conserved")
        for eq in lines:
            self.addEqu(eq)
        self.allocate()
        self.variables["meshx"] = self.mesh.coords[0]
        self.variables["meshy"] = self.mesh.coords[1]
        self.variables["meshz"] = self.mesh.coords[2]

    def checkForNan(self, names=None):
        """Names of variables holding NaN (pyranda.py:287-303)."""
        names = names or list(self.variables)
        bad = []
        for n in names:
            d = self.variables[n].data
            if isinstance(d, torch.Tensor):
                if d.is_floating_point() and bool(torch.isnan(d).any()):
                    bad.append(n)
            elif isinstance(d, float) and math.isnan(d):
                bad.append(n)
        return " ".join(bad)

    def setIC(self, ics, icDict=False, addOnly=False, verbose=False):
        """pyranda.py:305-370"""
        if icDict:
            ics = self.updateStringFromDictionary(ics, icDict, "ICs")
        self.ics = ics
        lines = splitLines(ics)
        names = []
        for eq in lines:
            names += findVar(eq, "scalar")
        for v in sorted(set(names)):
            self.addVar(v, kind="conserved")
        self.allocate()
        self.initial_conditions += lines
        if addOnly:
            return
        ns = {"self": self}
        for ic in lines:
            exec(fortran3d(ic, self.sMap), EVAL_GLOBALS, ns)
        self._unalias()
        bad = self.checkForNan(sorted(set(names)))
        if bad:
            raise FloatingPointError("Found some nans in inits: %s" % bad)
        self.updateVars()
        bad = self.checkForNan()
        if bad:
            raise FloatingPointError("Found some nans in Update after init: %s" % bad)

    # -------------------------------------------------------------- operators
    # pyranda.py:607-736; a direction of one point returns 0.0 as the reference
    def ddx(self, val):
        return 0.0 if self.nx <= 1 else self.grid.ddx(val)

    def ddy(self, val):
        return 0.0 if self.ny <= 1 else self.grid.ddy(val)

    def ddz(self, val):
        return 0.0 if self.nz <= 1 else self.grid.ddz(val)

    def dd4x(self, val):
        return self.grid.d4(0, val)

    def dd4y(self, val):
        return self.grid.d4(1, val)

    def dd4z(self, val):
        return self.grid.d4(2, val)

    def laplacian(self, val):
        return self.grid.laplacian(val)

    def divT(self, fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz):
        return self.grid.divT(fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz)

    def dd8x(self, val):
        return self.grid.d8(0, val)

    def dd8y(self, val):
        return self.grid.d8(1, val)

    def dd8z(self, val):
        return self.grid.d8(2, val)

    def div(self, f1, f2=None, f3=None):
        z = self.zero
        g = self.grid
        if f2 is None and f3 is None:
            if self.nx > 1:
                return g.div(f1, z, z)
            if self.ny > 1:
                return g.div(z, f1, z)
            if self.nz > 1:
                return g.div(z, z, f1)
            return 0.0
        if f3 is None:
            if self.nx > 1 and self.ny > 1:
                return g.div(f1, f2, z)
            if self.nz > 1 and self.ny > 1:
                return g.div(z, f1, f2)
            if self.nz > 1 and self.nx > 1:
                return g.div(f1, z, f2)
            if self.nx > 1:
                return g.div(f1, z, z)
            if self.ny > 1:
                return g.div(z, f1, z)
            if self.nz > 1:
                return g.div(z, z, f1)
            return 0.0
        return g.div(f1, f2, f3)

    def grad(self, val):
        return self.grid.grad(val)

    def ring(self, val):
        return self.grid.ring(val)

    def ringV(self, vx, vy, vz):
        return self.grid.ringv(vx, vy, vz)

    def filter(self, val):
        return self.grid.filter("spectral", val, PG_DIR_ALL)

    def gfilter(self, val):
        return self.grid.filter("gaussian", val, PG_DIR_ALL)

    def gfilterx(self, val):
        return self.grid.filter("gaussian", val, 0)

    def gfiltery(self, val):
        return self.grid.filter("gaussian", val, 1)

    def gfilterz(self, val):
        return self.grid.filter("gaussian", val, 2)

    def filterx(self, val):
        return self.grid.filter("spectral", val, 0)

    def filtery(self, val):
        return self.grid.filter("spectral", val, 1)

    def filterz(self, val):
        return self.grid.filter("spectral", val, 2)

    # parcop.f90:84-128 getVar: native coordinates, spacings, det J and the inverse Jacobian
    _MESH_VARS = {"x": 0, "y": 1, "z": 2, "d1": 3, "d2": 4, "d3": 5, "dtJ": 10, "dAx": 11, "dAy": 12,
                  "dAz": 13, "dBx": 14, "dBy": 15, "dBz": 16, "dCx": 17, "dCy": 18, "dCz": 19}

    def getVar(self, vname):
        if vname not in self._MESH_VARS:
            raise ValueError("mesh variable %s is not one of %s" % (vname, sorted(self._MESH_VARS)))
        return self.grid.mesh(self._MESH_VARS[vname])

    # -------------------------------------------------------------- viz dumps
    def write(self, wVars=None):
        """pyranda.py:431-470: a visualisation dump in pyranda's VTK format (pyranda_gb300.vtk).

        ``<name>/vis<cycle>/proc-000000.<cycle>.vtk`` holds the variables of
        wVars (default: the conserved ones) on the mesh coordinates, BINARY or
        ASCII after ``self.ioformat``; ``<name>/pyranda.visit`` lists every
        dump written so far.  Returns the file's path.
        """
        from . import vtk
        wVars = list(wVars) if wVars else list(self.conserved)
        path = vtk.dump_path(self.name, self.cycle)
        os.makedirs(os.path.dirname(path), exist_ok=True)
        shape = (self.nx, self.ny, self.nz)

        def host(v):
            a = v.numpy()
            return numpy.broadcast_to(numpy.asarray(a, dtype=numpy.float64), shape) if numpy.ndim(a) < 3 else a

        coords = [host(c) for c in self.mesh.coords]
        fields = {n: host(self.variables[n]) for n in wVars}
        t = _num(self.time)
        if getattr(self, "ioformat", "BINARY") == "ASCII":
            vtk.write_ascii(path, coords, fields, wVars, int(self.cycle), t)
        else:
            vtk.write_binary(path, coords, fields, wVars, int(self.cycle), t)
        if not hasattr(self, "vizDumpHistory"):
            self.vizDumpHistory = []
        self.vizDumpHistory.append([self.cycle, t])
        vtk.write_visit(self.name, self.vizDumpHistory)
        return path + ".vtk"

    # ---------------------------------------------------------------- restart
    def writeRestart(self, ivars=None, suffix=None, wVars=None):
        """pyranda.py:475-589: the simulation state in pyranda's restart format (pyranda_gb300.restart).

        The directory is ``<name>/restart_<cycle>``; ivars (a dict) adds
        numbers, strings, lists and numpy arrays of the caller to the restart.
        """
        from . import restart
        wVars = list(wVars) if wVars else list(self.variables)
        dump = restart.restart_dir(self.name, self.cycle, suffix)
        os.makedirs(dump, exist_ok=True)
        serial = {}
        if ivars:
            serial["local_vars"] = {"numpyArrays": {}}
            for k, v in ivars.items():
                if isinstance(v, numpy.ndarray):
                    fn = os.path.join(dump, k)
                    serial["local_vars"]["numpyArrays"][k] = fn
                    numpy.save(fn, v)
                elif v is None or isinstance(v, (str, int, float, bool, list, dict)):
                    serial["local_vars"][k] = v
        mesh = dict(self.meshOptions)
        mesh["function"] = None
        nx, ny, nz = self.nx, self.ny, self.nz
        serial.update({
            "mesh": mesh, "EOM": getattr(self, "eom", ""), "ICs": getattr(self, "ics", ""),
            "decomp": [1, 1, 1],
            "procMap": {"0-g1": numpy.zeros(3, dtype=numpy.int32),
                        "0-gn": numpy.array([nx - 1, ny - 1, nz - 1], dtype=numpy.int32)},
            "packages": list(getattr(self, "packagesRestart", [])),
            "time": _num(self.time), "deltat": _num(self.deltat), "cycle": int(self.cycle),
            "vizDumpHistory": list(getattr(self, "vizDumpHistory", [])), "sMap": dict(self.sMap)})
        arrays = {}
        for n in wVars:
            d = self.variables[n].data
            arrays[n] = self.variables[n].numpy() if isinstance(d, torch.Tensor) and d.dim() > 0 else _num(d)
        # which variables were single numbers, and which of those Python numbers rather than
        # device scalars (extra keys; the reference's reader ignores them): torch divides by a
        # Python number as a multiplication by its reciprocal, so a restart keeps the type
        serial["scalars"] = sorted(n for n in wVars if not isinstance(arrays[n], numpy.ndarray))
        serial["pyscalars"] = sorted(n for n in serial["scalars"] if not isinstance(self.variables[n].data,
                                                                                     torch.Tensor))
        restart.write_files(dump, serial, arrays, (nx, ny, nz))
        return dump

    # --------------------------------------------------------------- stepping
    def _unalias(self):
        """Give every variable its own storage (the RK update works in place)."""
        seen = {}
        for v in self.variables.values():
            d = v.data
            if isinstance(d, torch.Tensor) and d.dim() > 0:
                key = d.data_ptr()
                if key in seen and seen[key] is not v:
                    v.data = d.clone()
                else:
                    seen[key] = v

    def updateFlux(self):
        flux = {}
        for eq in self.equations:
            if eq.kind == "PDE":
                flux[eq.LHS[0]] = eq.RHS(self)
        return flux

    def updateVars(self, verbose=False):
        """pyranda.py:393-428: evaluate every ALG line in order."""
        skip = 0
        for eq in self.equations:
            if skip:
                skip -= 1
                continue
            if not eq.active or eq.kind != "ALG":
                continue
            grp = getattr(eq, "_fused_group", None) if self._fuse is not None else None
            if grp is not None:
                outs = grp.run(self, self._fuse)
                if outs is not None:   # one kernel for the whole run of equations
                    for e, o in zip(grp.eqs, outs):
                        self._assign(e.LHS[0], o)
                    skip = len(grp.eqs) - 1
                    continue
            rhs = eq.RHS(self)
            if not eq.LHS:
                continue
            if eq.rank == 1:
                self._assign(eq.LHS[0], rhs)
            else:
                for ii in range(len(rhs)):
                    self._assign(eq.LHS[ii], rhs[ii])

    def _assign(self, name, value):
        var = self.variables[name]
        if isinstance(value, torch.Tensor):
            for other in self.variables.values():
                if other is not var and other.data is value:
                    value = value.clone()
                    break
        var.data = value

    def _field_of(self, name):
        v = self.variables[name]
        d = v.data
        if not (isinstance(d, torch.Tensor) and tuple(d.shape) == self.grid.n and self.grid._fortran_ok(d)
                and d.dtype == torch.float64):
            v.data = self.grid.field(d)
        return v.data

    def rk4(self, time, dt):
        """One LSRK(5,4) step (pyranda.py:758-810), ALG update after every stage."""
        if self._fuse_wanted and self._fuse is None:
            from .fuse import Fuser
            self._fuse = Fuser(self, arith=self._fuse_arith)
            self._fuse.install(EVAL_GLOBALS)
        if self._graphs_enabled:
            t = self._rk4_graph(time, dt)
        else:
            t = self._rk4_eager(time, dt)
        if self._fuse is not None and self._fuse.lib is None:
            self._fuse.build()   # after the recording step, before any capture
        return t

    def use_fusion(self, enable=True, arithmetic="fp64"):
        """Evaluate the EOM's elementwise arithmetic in generated CUDA kernels.

        Each maximal elementwise subtree of every equation becomes one kernel
        (pyranda_gb300.fuse).  The next rk4 step records the kernels' argument
        kinds and runs unfused; the kernels are then compiled once (nvcc,
        cached by source hash) and used from the following step on.  With
        arithmetic='fp64' the results equal the unfused ones bit for bit;
        arithmetic='fp32' evaluates the expressions in FP32 between FP64
        fields (FP32 rounding error per line); arithmetic='df64' in
        double-float FP32 pairs (~48 bits).
        """
        if arithmetic not in ("fp64", "fp32", "df64"):
            raise ValueError("arithmetic must be 'fp64', 'fp32' or 'df64'")
        self._fuse_arith = arithmetic
        self._fuse_wanted = bool(enable)
        if self._fuse is not None and (not enable or self._fuse.arith != arithmetic):
            self._fuse = None
            for eq in self.equations:
                eq.RHS = eval("lambda self: " + eq.sRHS, EVAL_GLOBALS)

    def _dt_tensor(self, dt):
        """The time step as a device scalar (a field -- e.g. a reference restart's dt -- gives its first value)."""
        if isinstance(dt, torch.Tensor):
            return dt.to(device=self.grid.device, dtype=torch.float64).reshape(-1)[0].reshape(())
        if isinstance(dt, numpy.ndarray):
            return torch.full((), float(dt.flat[0]), dtype=torch.float64, device=self.grid.device)
        return torch.full((), float(dt), dtype=torch.float64, device=self.grid.device)

    def _time_tensor(self, time):
        return time

    def _time_buffer(self):
        """Device storage of the simulation time read by a recorded step."""
        return torch.zeros((), dtype=torch.float64, device=self.grid.device)

    def _load_time(self, buf, time):
        if isinstance(time, torch.Tensor):
            buf.copy_(time)
        else:
            buf.fill_(float(time))

    def _stage_time(self, time_i, eta, dt, dt_dev):
        """t = t0 + eta_k dt (pyranda.py:805)."""
        return time_i + eta * dt

    def _rk4_eager(self, time, dt, dt_dev=None):
        names = self.conserved
        if self._phi is None or set(self._phi) != set(names):
            self._phi = {U: self.grid.empty() for U in names}
        for U in names:
            self._phi[U].zero_()
        if dt_dev is None:
            dt_dev = self._dt_tensor(dt)
        time_i = self._time_tensor(time)
        self.deltat = dt
        fused_rk = self._fuse is not None and self._fuse.lib is not None
        for ii in range(5):
            if fused_rk:   # PDE kernels that own their variable's stage update apply it themselves
                self._fuse.rk_ctx = {"A": ARK[ii], "B": BRK[ii], "dt": dt_dev, "phi": self._phi}
            try:
                flux = self.updateFlux()
            finally:
                if fused_rk:
                    self._fuse.rk_ctx = None
            rest = [n for n in names if flux[n] is not RK_DONE]
            if rest:
                U = [self._field_of(n) for n in rest]
                F = [self.grid.field(flux[n]) for n in rest]
                PHI = [self._phi[n] for n in rest]
                self.grid.rk_stage(U, PHI, F, dt_dev, ARK[ii], BRK[ii])
            time = self._stage_time(time_i, ETA[ii], dt, dt_dev)
            self.time = time
            self.updateVars()
        self.cycle += 1
        return time

    # ----------------------------------------------------------- CUDA graphs
    def use_graphs(self, enable=True):
        """Record one whole rk4 step in a CUDA graph and replay it afterwards.

        The EOM must not read ``simtime`` as a Python number and must keep the
        same set of conserved variables.  The first rk4 call after enabling
        runs eagerly (allocating every variable), the second records the graph.
        """
        self._graphs_enabled = bool(enable)
        self._graph = None
        self._graph_warm = False

    def _rk4_graph(self, time, dt):
        if not getattr(self, "_graph_warm", False):
            self._graph_warm = True
            return self._rk4_eager(time, dt)
        if self._graph is None:
            self._capture(time, dt)
        self._g_dt.copy_(self._dt_tensor(dt))
        self._load_time(self._g_t0, time)
        self._graph.replay()
        self.cycle += 1
        self.deltat = dt
        t = self._stage_time(self._time_tensor(time), 1.0, dt, self._g_dt)
        self.time = t
        return t

    def _capture(self, time, dt):
        self._unalias()
        for n in self.conserved:
            self._field_of(n)
        before = {n: v.data for n, v in self.variables.items()}
        self._g_dt = self._dt_tensor(dt).clone()
        self._g_t0 = self._time_buffer()
        self._phi = {U: self.grid.empty() for U in self.conserved}
        stream = torch.cuda.Stream(device=self.grid.device)
        stream.wait_stream(torch.cuda.current_stream())
        g = torch.cuda.CUDAGraph()
        # Python's cyclic collector may finalise an older simulation at any
        # allocation; destroying its graph or its library handle calls CUDA
        # APIs that are not allowed while a stream is being captured.
        gc_was_enabled = gc.isenabled()
        gc.collect()
        gc.disable()
        try:
            with torch.cuda.stream(stream):
                with torch.cuda.graph(g, stream=stream, capture_error_mode="thread_local"):
                    self._capture_body(before)
        finally:
            if gc_was_enabled:
                gc.enable()
        torch.cuda.current_stream().wait_stream(stream)
        flush_pending()
        self.cycle -= 1
        for n, old in before.items():
            if isinstance(old, torch.Tensor):
                self.variables[n].data = old
        self._g_storage = {n: t for n, t in before.items() if isinstance(t, torch.Tensor)}
        self._graph = g
        # the capture itself did not advance the state: replay once for this step

    def sync_graph_storage(self):
        """After eager work on a graph-recorded simulation: put every variable back into the storage the graph reads."""
        for n, t in getattr(self, "_g_storage", {}).items():
            v = self.variables.get(n)
            if v is None or v.data is t:
                continue
            if isinstance(v.data, torch.Tensor) and (v.data.shape == t.shape or t.dim() == 0):
                t.copy_(v.data.reshape(t.shape) if t.dim() == 0 else v.data)
            elif not isinstance(v.data, torch.Tensor):
                t.fill_(float(v.data))
            v.data = t

    def _capture_body(self, before):
        """The recorded work: one eager step, then the rebound variables copied back into the replay's storage."""
        self._rk4_eager(self._g_t0, self._g_dt, dt_dev=self._g_dt)
        for n, v in self.variables.items():
            old = before.get(n)
            new = v.data
            if isinstance(old, torch.Tensor) and isinstance(new, torch.Tensor) and old is not new:
                if old.shape == new.shape or old.dim() == 0:
                    old.copy_(new)
