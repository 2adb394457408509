"""Ensembles: many independent pyranda simulations advanced as one.

pyranda runs one simulation per process (one parcop patch per
``pyrandaSim``, pyranda/pyrandaMPI.py:151-155).  Here M independent grids of
any sizes that share their periodicity and null directions are stored back to
back in one flat FP64 device buffer; member m owns points
``[offsets[m], offsets[m+1])`` in its own Fortran order.  Every compact
operator is one launch over the lines of all members (``pg_ens_*`` in
``libpyranda_gpu.so``), so small 2-D members fill the GPU together, and a
whole RK step of the ensemble records into one CUDA graph.

Semantics that differ from a single simulation, all per member:
  * ``sum``/``max``/``min``/``mean`` and ``dt.courant``/``dt.diff`` give one
    value per member, broadcast to that member's points (a field), so
    expressions and the RK update use them pointwise;
  * the time step is a field (each member's dt on its points) and
    ``rk4(time, dt)`` takes and returns the M members' times as a device
    tensor;
  * ``var(name).sum()`` returns a numpy array of M values.
"""
import ctypes

import numpy
import torch

from . import _lib
from .grid import _ptr, _stream, flush_pending, release
from .pyranda import defaultMeshOptions, pyrandaGPU, pyrandaSim, pyrandaVar

_AX = {"x": 0, "y": 1, "z": 2}


class EnsembleGrid:
    """M Cartesian grids in one flat field layout (the ``Grid`` interface)."""

    def __init__(self, members, precision="fp64", device=None):
        """members: sequence of (n, periodic, x1, xn), each a 3-sequence."""
        if not torch.cuda.is_available():
            raise RuntimeError("pyranda_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = _lib.load()
        flush_pending()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.m = len(members)
        if self.m < 1:
            raise ValueError("an ensemble needs at least one member")
        arr = (_lib.pg_grid * self.m)()
        self.members = []
        for i, (n, periodic, x1, xn) in enumerate(members):
            n = tuple(int(v) for v in n)
            self.members.append(n)
            for d in range(3):
                arr[i].n[d] = n[d]
                arr[i].periodic[d] = 1 if periodic[d] else 0
                arr[i].x1[d] = float(x1[d])
                arr[i].xn[d] = float(xn[d])
            arr[i].precision = _lib.precision_code(precision)
        self.periodic = tuple(bool(p) for p in members[0][1])
        self.precision = precision
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.pg_ens_create(self.m, arr, ctypes.byref(h)), "pg_ens_create")
        self.h = h
        offs = (ctypes.c_int64 * (self.m + 1))()
        self.npts = int(self.lib.pg_ens_points(self.h, offs))
        self.offsets = numpy.array(list(offs), dtype=numpy.int64)
        self.n = (self.npts,)
        self.shape = self.n
        counts = numpy.diff(self.offsets)
        self.member_points = counts.astype(numpy.float64)
        self.patch_d, self.mesh_d = [], []
        for i in range(self.m):
            pd = (ctypes.c_double * 3)()
            md = (ctypes.c_double * 3)()
            _lib.check(self.lib.pg_ens_spacing(self.h, i, pd, md), "pg_ens_spacing")
            self.patch_d.append(list(pd))
            self.mesh_d.append(list(md))
        dev = self.device
        self.starts = torch.as_tensor(self.offsets[:-1], dtype=torch.int64, device=dev)
        self.member_id = torch.as_tensor(numpy.repeat(numpy.arange(self.m), counts), dtype=torch.int64, device=dev)
        self.counts_field = self.member_field(self.member_points)
        self._planes = {}

    def __del__(self):
        try:
            if getattr(self, "h", None):
                release(self.lib, "pg_ens_destroy", self.h)
                self.h = None
        except Exception:
            pass

    def set_precision(self, precision):
        self.precision = precision
        _lib.check(self.lib.pg_ens_set_precision(self.h, _lib.precision_code(precision)),
                   "pg_ens_set_precision")

    def set_line_split(self, on):
        """Banded line solves split across the threads of a CTA (see Grid.set_line_split)."""
        _lib.check(self.lib.pg_ens_set_line_split(self.h, 1 if on else 0), "pg_ens_set_line_split")

    # ------------------------------------------------------------------ fields
    def empty(self):
        return torch.empty(self.npts, dtype=torch.float64, device=self.device)

    def zeros(self):
        return torch.zeros(self.npts, dtype=torch.float64, device=self.device)

    def _fortran_ok(self, t):
        return t.dim() == 1 and t.shape[0] == self.npts and t.stride(0) == 1

    def field(self, v):
        """v as a flat device field: a field, a per-member array of M values, or a constant."""
        if isinstance(v, torch.Tensor) and v.dtype == torch.float64 and v.device == self.device \
                and tuple(v.shape) == self.n and v.is_contiguous():
            return v
        if isinstance(v, torch.Tensor):
            t = v.to(device=self.device, dtype=torch.float64)
            if t.dim() == 1 and t.shape[0] == self.m and self.m != self.npts:
                return self.member_field(t)
            out = self.empty()
            out.copy_(t.expand(self.n))
            return out
        a = numpy.asarray(v, dtype=numpy.float64)
        if a.ndim == 1 and a.shape[0] == self.m and self.m != self.npts:
            return self.member_field(a)
        out = self.empty()
        if a.ndim == 0:
            out.fill_(float(a))
        else:
            out.copy_(torch.from_numpy(numpy.ascontiguousarray(numpy.broadcast_to(a, self.n))).to(self.device))
        return out

    def member_field(self, values):
        """A field holding values[m] on every point of member m."""
        v = torch.as_tensor(values, dtype=torch.float64).to(self.device)
        return v.index_select(0, self.member_id)

    def member_values(self, f):
        """The value of a per-member field at each member's first point (M values, on the device)."""
        return f.index_select(0, self.starts)

    def member_view(self, f, m):
        """Member m of a flat field as an (nx, ny, nz) Fortran-ordered view."""
        nx, ny, nz = self.members[m]
        return f[int(self.offsets[m]):int(self.offsets[m + 1])].view(nz, ny, nx).permute(2, 1, 0)

    def from_members(self, arrays):
        """A flat field from one (nx, ny, nz) array or tensor per member."""
        out = self.empty()
        for m, a in enumerate(arrays):
            self.member_view(out, m).copy_(torch.as_tensor(numpy.asarray(a) if not isinstance(a, torch.Tensor)
                                                           else a, dtype=torch.float64))
        return out

    def plane(self, axis, k):
        """Index of plane k (negative counts from the end) of every member along an axis."""
        key = (axis, k)
        if key not in self._planes:
            d = _AX[axis] if isinstance(axis, str) else int(axis)
            idx = []
            for m, (nx, ny, nz) in enumerate(self.members):
                n = (nx, ny, nz)[d]
                kk = k % n
                ii, jj, ll = numpy.meshgrid(numpy.arange(nx), numpy.arange(ny), numpy.arange(nz), indexing="ij")
                sel = (ii, jj, ll)[d] == kk
                flat = (ii + nx * (jj + ny * ll))[sel]
                idx.append(numpy.sort(flat.ravel()) + self.offsets[m])
            self._planes[key] = torch.as_tensor(numpy.concatenate(idx), dtype=torch.int64, device=self.device)
        return self._planes[key]

    def get_plane(self, a, axis, k):
        return a.index_select(0, self.plane(axis, k))

    def set_plane(self, a, axis, k, value):
        """Plane k of every member := value (a number or get_plane's layout); graph-safe."""
        idx = self.plane(axis, k)
        if isinstance(value, torch.Tensor) and value.dim() > 0:
            a.index_copy_(0, idx, value)
        else:
            a.index_fill_(0, idx, float(value))

    def _out(self, out):
        if out is None:
            return self.empty()
        if not self._fortran_ok(out):
            raise ValueError("output field must be a contiguous float64 vector of the ensemble's points")
        return out

    # --------------------------------------------------------------- operators
    def d1(self, direction, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_d1(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_ens_d1")
        return out

    def ddx(self, v, out=None):
        return self.d1(0, v, out)

    def ddy(self, v, out=None):
        return self.d1(1, v, out)

    def ddz(self, v, out=None):
        return self.d1(2, v, out)

    def d8(self, direction, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_d8(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_ens_d8")
        return out

    def filter(self, kind, v, direction=_lib.PG_DIR_ALL, out=None):
        v = self.field(v)
        out = self._out(out)
        k = _lib.PG_SPECTRAL if kind == "spectral" else _lib.PG_GAUSSIAN
        _lib.check(self.lib.pg_ens_filter(self.h, k, direction, _ptr(v), _ptr(out), _stream()), "pg_ens_filter")
        return out

    def ring(self, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_ring(self.h, _ptr(v), _ptr(out), _stream()), "pg_ens_ring")
        return out

    def d2(self, direction, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_d2(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_ens_d2")
        return out

    def d4(self, direction, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_d4(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_ens_d4")
        return out

    def laplacian(self, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_laplacian(self.h, _ptr(v), _ptr(out), _stream()), "pg_ens_laplacian")
        return out

    def divT(self, fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz):
        return [self.div(fxx, fyx, fzx), self.div(fxy, fyy, fzy), self.div(fxz, fyz, fzz)]

    def ringv(self, vx, vy, vz, out=None):
        vx, vy, vz = self.field(vx), self.field(vy), self.field(vz)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_ringv(self.h, _ptr(vx), _ptr(vy), _ptr(vz), _ptr(out), _stream()),
                   "pg_ens_ringv")
        return out

    def grad(self, v):
        v = self.field(v)
        gx, gy, gz = self.empty(), self.empty(), self.empty()
        _lib.check(self.lib.pg_ens_grad(self.h, _ptr(v), _ptr(gx), _ptr(gy), _ptr(gz), _stream()), "pg_ens_grad")
        return [gx, gy, gz]

    def div(self, fx, fy, fz, out=None):
        fx, fy, fz = self.field(fx), self.field(fy), self.field(fz)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_div(self.h, _ptr(fx), _ptr(fy), _ptr(fz), _ptr(out), _stream()), "pg_ens_div")
        return out

    def mesh(self, which):
        out = self.empty()
        _lib.check(self.lib.pg_ens_mesh(self.h, which, _ptr(out), _stream()), "pg_ens_mesh")
        return out

    # ---------------------------------------------------- time step and reductions
    def courant(self, u, v, w, c, out=None):
        u, c = self.field(u), self.field(c)
        vp, vc = (None, 0.0)
        wp, wc = (None, 0.0)
        if isinstance(v, torch.Tensor) and v.dim() > 0:
            v = self.field(v)
            vp = _ptr(v)
        else:
            vc = float(v)
        if isinstance(w, torch.Tensor) and w.dim() > 0:
            w = self.field(w)
            wp = _ptr(w)
        else:
            wc = float(w)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_courant(self.h, _ptr(u), vp, wp, _ptr(c), vc, wc, _ptr(out), _stream()),
                   "pg_ens_courant")
        return out

    def diff(self, bulk, rho, out=None):
        bulk, rho = self.field(bulk), self.field(rho)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_diff(self.h, _ptr(bulk), _ptr(rho), _ptr(out), _stream()), "pg_ens_diff")
        return out

    def reduce(self, op, v, out=None):
        """op 0 sum, 1 max, 2 min over each member; returned as a field."""
        if not isinstance(v, torch.Tensor) or v.dim() == 0:
            x = v if not isinstance(v, torch.Tensor) else v.to(self.device, torch.float64)
            return x * self.counts_field if op == 0 else self.field(x)
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ens_reduce(self.h, op, _ptr(v), _ptr(out), None, _stream()), "pg_ens_reduce")
        return out

    def reduce_members(self, op, v):
        """op 0 sum, 1 max, 2 min over each member: M values on the device."""
        out = torch.empty(self.m, dtype=torch.float64, device=self.device)
        if not isinstance(v, torch.Tensor) or v.dim() == 0:
            x = float(v)
            out.fill_(x)
            return out * torch.as_tensor(self.member_points, device=self.device) if op == 0 else out
        v = self.field(v)
        _lib.check(self.lib.pg_ens_reduce(self.h, op, _ptr(v), None, _ptr(out), _stream()), "pg_ens_reduce")
        return out

    def reduce_value(self, op, v):
        """Host values of a per-member reduction (numpy array of M)."""
        return self.reduce_members(op, v).cpu().numpy()

    def rk_stage(self, U, PHI, F, dt, A, B):
        n = len(U)
        arr = ctypes.c_void_p * n
        u = arr(*[t.data_ptr() for t in U])
        p = arr(*[t.data_ptr() for t in PHI])
        f = arr(*[t.data_ptr() for t in F])
        _lib.check(self.lib.pg_ens_rk_stage(self.h, n, u, p, f, _ptr(dt), float(A), float(B), _stream()),
                   "pg_ens_rk_stage")

    def check_finite(self, v, flag):
        _lib.check(self.lib.pg_check_finite(_ptr(v), v.numel(), _ptr(flag), _stream()), "pg_check_finite")


class pyrandaEnsembleGPU(pyrandaGPU):
    """Per-member reductions (broadcast to fields) for an ensemble."""

    def __init__(self, sim):
        pyrandaGPU.__init__(self, sim)

    def sum3D(self, data):
        return self.grid.reduce(0, data)

    def max3D(self, data):
        return self.grid.reduce(1, data)

    def min3D(self, data):
        return self.grid.reduce(2, data)

    def mean3D(self, data):
        return self.grid.reduce(0, data) / self.grid.counts_field

    def _axis_sum(self, data, axis):
        raise NotImplementedError("line and plane sums are per member: use EnsembleGrid.member_view")


class pyrandaEnsemble(pyrandaSim):
    """M independent pyrandaSims (one mesh string or option dict each) advanced together.

    The EOM, IC and packages are shared: one ``EOM``/``setIC`` call defines
    every member.  ``precision`` and ``device`` are as for ``pyrandaSim``.
    """

    def __init__(self, name, meshes, silent=False, precision="fp64", device=None):
        self.name = name
        self.silent = silent
        opts_list = []
        for mo in meshes:
            if isinstance(mo, str):
                mo = self._parse_mesh(mo)
            opts = defaultMeshOptions()
            opts.update(mo)
            if opts.get("coordsys", 0) != 0:
                raise ValueError("only Cartesian meshes (coordsys=0) are supported")
            if any(any(s) for s in opts["symmetric"]):
                raise ValueError("SYMM boundaries are not supported; use periodic or one-sided (NONE)")
            opts_list.append(opts)
        self.member_options = opts_list
        from .pyranda import _Mesh
        self.mesh = _Mesh()
        self.meshOptions = opts_list[0]
        self.mesh.options = opts_list[0]
        self.mesh.coordsys = 0
        specs = [([int(v) for v in o["nn"]], o["periodic"], o["x1"], o["xn"]) for o in opts_list]
        self.precision = precision
        self.grid = EnsembleGrid(specs, precision=precision, device=device)
        n0 = specs[0][0]
        # only "is this direction null" is read from nx/ny/nz; all members agree on it
        self.nx, self.ny, self.nz = n0
        self.npts = self.grid.npts
        self.M = self.grid.m
        self.PyMPI = pyrandaEnsembleGPU(self)
        self.mesh.PyMPI = self.PyMPI
        self._make_mesh()
        self.dx = self.grid.member_field([(o["xn"][0] - o["x1"][0]) / max(int(o["nn"][0]) - 1, 1) for o in opts_list])
        self.dy = self.grid.member_field([(o["xn"][1] - o["x1"][1]) / max(int(o["nn"][1]) - 1, 1) for o in opts_list])
        self.dz = self.grid.member_field([(o["xn"][2] - o["x1"][2]) / max(int(o["nn"][2]) - 1, 1) for o in opts_list])
        self.zero = self.grid.zeros()
        self.equations = []
        self.conserved = []
        self.variables = {}
        self.initial_conditions = []
        self.nPDE = self.nALG = self.nELP = 0
        self.packages = {}
        self.userDefined = {}
        self.time = torch.zeros(self.M, dtype=torch.float64, device=self.grid.device)
        self.cycle = 0
        self.deltat = 0.0
        self._phi = None
        self._graph = None
        self._graphs_enabled = False
        self._fuse = None
        self._fuse_wanted = False
        self._fuse_arith = "fp64"
        self.get_sMap()

    def _make_mesh(self):
        g = self.grid
        self.mesh.coords = [pyrandaVar("x", "mesh"), pyrandaVar("y", "mesh"), pyrandaVar("z", "mesh")]
        for i, c in enumerate(self.mesh.coords):
            c.sim = self
            c.allocated = True
            c.data = g.mesh(i)
        self.mesh.shape = [g.npts]
        self.mesh.nn = [o["nn"] for o in self.member_options]
        self.mesh.d1 = g.mesh(3)
        self.mesh.d2 = g.mesh(4)
        self.mesh.d3 = g.mesh(5)
        self.mesh.GridLen = g.mesh(6)
        self.mesh.CellVol = g.mesh(7)
        self.mesh.indices = []
        for d, name in enumerate(("iloc", "jloc", "kloc")):
            parts = []
            for (nx, ny, nz) in g.members:
                a = numpy.meshgrid(numpy.arange(nx), numpy.arange(ny), numpy.arange(nz), indexing="ij")[d]
                parts.append(a.ravel(order="F").astype(numpy.float64))
            v = pyrandaVar(name, "mesh")
            v.sim = self
            v.allocated = True
            v.data = torch.as_tensor(numpy.concatenate(parts), device=g.device)
            self.mesh.indices.append(v)

    def get_sMap(self):
        pyrandaSim.get_sMap(self)
        self.sMap["mean("] = "self.PyMPI.mean3D("

    def emptyScalar(self, val=0.0):
        t = self.grid.zeros()
        if val != 0.0:
            t.fill_(val)
        return t

    # --------------------------------------------------------------- stepping
    def _dt_tensor(self, dt):
        """The time step as a field: from a field, M per-member values or one number."""
        return self.grid.field(dt)

    def _time_tensor(self, time):
        if isinstance(time, torch.Tensor) and time.dim() == 1:
            return time.to(device=self.grid.device, dtype=torch.float64)
        t = torch.empty(self.M, dtype=torch.float64, device=self.grid.device)
        if isinstance(time, torch.Tensor):
            t.copy_(time.expand(self.M))
        else:
            t.copy_(torch.from_numpy(numpy.array(numpy.broadcast_to(numpy.asarray(time, dtype=numpy.float64),
                                                                    (self.M,)))))
        return t

    def _time_buffer(self):
        return torch.zeros(self.M, dtype=torch.float64, device=self.grid.device)

    def _load_time(self, buf, time):
        buf.copy_(self._time_tensor(time))

    def _stage_time(self, time_i, eta, dt, dt_dev):
        """Each member's t0 + eta_k dt (pyranda.py:805), dt read from the dt field."""
        return time_i + eta * self.grid.member_values(dt_dev)
