"""Device-side grid: one pg_handle plus the field conventions of pyranda.

Fields are torch float64 tensors of shape (nx, ny, nz) laid out in Fortran
order (x fastest, strides (1, nx, nx*ny)) on the current CUDA device, which is
the memory layout of the F-ordered numpy arrays pyranda hands to parcop
(pyranda/pyrandaMPI.py:249-250).  Every operator here is one or more calls
into ``libpyranda_gpu.so`` on the current torch stream; outputs are allocated
by torch's caching allocator (or passed in), never by the library.
"""
import ctypes
import json
import os

import torch

from . import _lib

_DIRS = {"x": 0, "y": 1, "z": 2}


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


# Handles whose owner was collected while a CUDA graph was being recorded.
# Destroying a handle frees device memory, which is not allowed during stream
# capture, and Python's cyclic collector can finalise an old grid at any
# allocation -- also inside another simulation's capture.  Such handles wait
# here until the next safe point (a new grid, or the end of a capture).
_PENDING = []


def _capturing():
    try:
        return torch.cuda.is_available() and torch.cuda.is_current_stream_capturing()
    except Exception:
        return True


def release(lib, destroy, h):
    """Destroy a handle now, or later when a capture is in progress."""
    if _capturing():
        _PENDING.append((destroy, h))
        return
    getattr(lib, destroy)(h)


def flush_pending():
    """Destroy the handles deferred during a capture (call outside captures)."""
    if _capturing():
        return
    from . import _lib
    lib = _lib.load()
    while _PENDING:
        destroy, h = _PENDING.pop()
        getattr(lib, destroy)(h)


PLAN_CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "sweep_plans.json")


def _plan_cache_enabled():
    return os.environ.get("PYRANDA_GB300_PLAN_CACHE", "1") != "0"


def _plan_cache_get(key, path=None):
    """The cached autotuned plan (18 ints, pg_sweep_plan's layout) for key, or None."""
    if not _plan_cache_enabled():
        return None
    try:
        with open(path or PLAN_CACHE) as f:
            plan = json.load(f).get(key)
    except (OSError, ValueError):
        return None
    if isinstance(plan, list) and len(plan) == 18 and all(v in (0, 1, 2) for v in plan):
        return plan
    return None


def _plan_cache_put(key, plan, path=None):
    """Adds key -> plan to the cache file (written to a temporary file and renamed into place)."""
    if not _plan_cache_enabled():
        return
    path = path or PLAN_CACHE
    try:
        with open(path) as f:
            data = json.load(f)
        if not isinstance(data, dict):
            data = {}
    except (OSError, ValueError):
        data = {}
    data[key] = [int(v) for v in plan]
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = "%s.%d.tmp" % (path, os.getpid())
        with open(tmp, "w") as f:
            json.dump(data, f)
        os.replace(tmp, path)
    except OSError:
        pass


class Grid:
    """A pyranda patch on one GPU (parcop.f90:23-81 setup + setup_mesh / setup_mesh_x3)."""

    def __init__(self, n, periodic, x1, xn, precision="fp64", device=None, line_split=False, bc=None,
                 coordsys=0):
        """bc: per direction the (lower, upper) end codes of non-periodic directions,
        'NONE' (one-sided closures), 'SYMM' (symmetry plane) or 'XTND' (extended data);
        coordsys: 0 Cartesian, 1 cylindrical (x = radius), 2 spherical (x = radius,
        y = polar angle, z = azimuth), 3 curvilinear (coordinates by set_mesh_coords),
        4 spherical with ratio-zoned radii."""
        if not torch.cuda.is_available():
            raise RuntimeError("pyranda_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = _lib.load()
        flush_pending()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.n = tuple(int(v) for v in n)
        self.shape = self.n
        self.npts = self.n[0] * self.n[1] * self.n[2]
        self.periodic = tuple(bool(p) for p in periodic)
        g = _lib.pg_grid()
        for d in range(3):
            g.n[d] = self.n[d]
            g.periodic[d] = 1 if self.periodic[d] else 0
            g.x1[d] = float(x1[d])
            g.xn[d] = float(xn[d])
        codes = {"NONE": _lib.PG_BC_NONE, "SYMM": _lib.PG_BC_SYMM, "XTND": _lib.PG_BC_XTND}
        self.bc = tuple(tuple(b) for b in (bc or (("NONE", "NONE"),) * 3))
        for d in range(3):
            for e in range(2):
                g.bc[d][e] = codes[self.bc[d][e]]
        g.coordsys = int(coordsys)
        self.coordsys = int(coordsys)
        self.symmetric = tuple((not self.periodic[d]) and "SYMM" in self.bc[d] for d in range(3))
        self.precision = precision
        # the autotuned path reuses a plan measured before for the same grid, GPU and library build
        cached = _plan_cache_get(self._plan_key()) if precision == "auto" else None
        g.precision = _lib.precision_code("fp32" if cached is not None else precision)
        h = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.pg_create(ctypes.byref(g), ctypes.byref(h)), "pg_create")
        self.h = h
        self.plan_from_cache = False
        if cached is not None:
            plan = (ctypes.c_int * len(cached))(*cached)
            with torch.cuda.device(self.device):
                _lib.check(self.lib.pg_set_sweep_plan(self.h, plan), "pg_set_sweep_plan")
            self.plan_from_cache = True
        elif precision == "auto":
            raw = (ctypes.c_int * 18)()
            _lib.check(self.lib.pg_sweep_plan(self.h, raw), "pg_sweep_plan")
            _plan_cache_put(self._plan_key(), list(raw))
        pd = (ctypes.c_double * 3)()
        md = (ctypes.c_double * 3)()
        self.lib.pg_get_spacing(self.h, pd, md)
        self.patch_d = list(pd)  # dx, dy, dz of the d1 metric
        self.mesh_d = list(md)   # mesh d1, d2, d3
        self.gridlen = min(self.mesh_d)
        self._scalar_pool = []
        self.line_split = False
        if line_split:
            self.set_line_split(True)

    def _plan_key(self):
        """What an autotuned plan depends on: the operators (extents, periodicity, ends,
        coordinates), the GPU and the library build."""
        lib = _lib.lib_path()
        st = os.stat(lib)
        return json.dumps([list(self.n), list(self.periodic), [list(b) for b in self.bc], self.coordsys,
                           torch.cuda.get_device_name(self.device), st.st_size, int(st.st_mtime)])

    def __del__(self):
        try:
            if getattr(self, "h", None):
                release(self.lib, "pg_destroy", self.h)
                self.h = None
        except Exception:
            pass

    def dense_plan(self):
        """{(operator, direction): True where the dense kernel runs} (operators 'd1', 'd8', 'sf', 'gf')."""
        plan = (ctypes.c_int * 12)()
        _lib.check(self.lib.pg_dense_plan(self.h, plan), "pg_dense_plan")
        return {(op, "xyz"[d]): bool(plan[k * 3 + d]) for k, op in enumerate(("d1", "d8", "sf", "gf"))
                for d in range(3)}

    def sweep_plan(self):
        """{(operator, direction): 'banded' | 'dense' | 'split'} (operators 'd1', 'd8', 'sf', 'gf', 'd2', 'd4')."""
        plan = (ctypes.c_int * 18)()
        _lib.check(self.lib.pg_sweep_plan(self.h, plan), "pg_sweep_plan")
        names = ("banded", "dense", "split")
        return {(op, "xyz"[d]): names[plan[k * 3 + d]] for k, op in enumerate(("d1", "d8", "sf", "gf", "d2", "d4"))
                for d in range(3)}

    def set_precision(self, precision):
        self.precision = precision
        _lib.check(self.lib.pg_set_precision(self.h, _lib.precision_code(precision)),
                   "pg_set_precision")

    def set_line_split(self, on):
        """Banded line solves split across the threads of a CTA (segments of 32
        points joined by the reduced system) instead of one thread per line."""
        _lib.check(self.lib.pg_set_line_split(self.h, 1 if on else 0), "pg_set_line_split")
        self.line_split = bool(on)

    # ------------------------------------------------------------------ fields
    def empty(self):
        nx, ny, nz = self.n
        return torch.empty((nz, ny, nx), dtype=torch.float64, device=self.device).permute(2, 1, 0)

    def zeros(self):
        t = self.empty()
        t.zero_()
        return t

    def _fortran_ok(self, t):
        # a tensor whose storage order is x-fastest (any size-1 dims may carry odd strides)
        nx, ny, nz = self.n
        exp = (1, nx, nx * ny)
        for d in range(3):
            if self.n[d] > 1 and t.stride(d) != exp[d]:
                return False
        return True

    def field(self, v):
        """Return v as a device field in the library layout (copying only if needed)."""
        if isinstance(v, torch.Tensor) and v.dtype == torch.float64 and v.device == self.device \
                and tuple(v.shape) == self.n and self._fortran_ok(v):
            return v
        out = self.empty()
        if isinstance(v, torch.Tensor):
            out.copy_(v.to(device=self.device, dtype=torch.float64).expand(self.n))
        else:
            import numpy
            a = numpy.asarray(v, dtype=numpy.float64)
            if a.ndim == 0:
                out.fill_(float(a))
            else:
                out.copy_(torch.from_numpy(numpy.array(numpy.broadcast_to(a, self.n), order="C")).to(self.device))
        return out

    def _out(self, out):
        if out is None:
            return self.empty()
        if not self._fortran_ok(out):
            raise ValueError("output field must be float64 (nx,ny,nz) in Fortran order")
        return out

    # --------------------------------------------------------------- operators
    def d1(self, direction, v, out=None, sym=1):
        """sym = -1: the variant for a field antisymmetric about a symmetry plane."""
        v = self.field(v)
        out = self._out(out)
        if sym == 1:
            _lib.check(self.lib.pg_d1(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_d1")
        else:
            _lib.check(self.lib.pg_d1_sym(self.h, direction, sym, _ptr(v), _ptr(out), _stream()), "pg_d1_sym")
        return out

    def ddx(self, v, out=None):
        return self.d1(0, v, out)

    def ddy(self, v, out=None):
        return self.d1(1, v, out)

    def ddz(self, v, out=None):
        return self.d1(2, v, out)

    def d8(self, direction, v, out=None, sym=1):
        v = self.field(v)
        out = self._out(out)
        if sym == 1:
            _lib.check(self.lib.pg_d8(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_d8")
        else:
            _lib.check(self.lib.pg_d8_sym(self.h, direction, sym, _ptr(v), _ptr(out), _stream()), "pg_d8_sym")
        return out

    def d2(self, direction, v, out=None):
        """Compact 10th-order second derivative (c10d2), divided by the spacing squared."""
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_d2(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_d2")
        return out

    def d4(self, direction, v, out=None):
        """Explicit 4th-order fourth derivative (e4d4), no metric."""
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_d4(self.h, direction, _ptr(v), _ptr(out), _stream()), "pg_d4")
        return out

    def laplacian(self, v, out=None):
        """The Laplacian (operators.f90:513-559): d2x + d2y + d2z on Cartesian grids,
        the cylindrical and spherical forms on those grids."""
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_laplacian(self.h, _ptr(v), _ptr(out), _stream()), "pg_laplacian")
        return out

    def divT(self, fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz):
        """Divergence of a tensor (operators.f90:97-181, every coordinate system)."""
        f = [self.field(x) for x in (fxx, fxy, fxz, fyx, fyy, fyz, fzx, fzy, fzz)]
        out = [self.empty() for _ in range(3)]
        fp = (ctypes.c_void_p * 9)(*[x.data_ptr() for x in f])
        op = (ctypes.c_void_p * 3)(*[x.data_ptr() for x in out])
        _lib.check(self.lib.pg_divt(self.h, fp, op, _stream()), "pg_divt")
        return out

    def filter(self, kind, v, direction=_lib.PG_DIR_ALL, out=None, sym=None):
        """kind 'spectral' (c8ff8, fbar) or 'gaussian' (cgfs4, gbar); sym: per direction +1 / -1
        (the variant for antisymmetric fields at a symmetry plane)."""
        v = self.field(v)
        out = self._out(out)
        k = _lib.PG_SPECTRAL if kind == "spectral" else _lib.PG_GAUSSIAN
        if sym is None:
            _lib.check(self.lib.pg_filter(self.h, k, direction, _ptr(v), _ptr(out), _stream()), "pg_filter")
        else:
            s3 = (ctypes.c_int * 3)(*[int(x) for x in sym])
            _lib.check(self.lib.pg_filter_sym(self.h, k, direction, s3, _ptr(v), _ptr(out), _stream()),
                       "pg_filter_sym")
        return out

    def ring(self, v, out=None):
        v = self.field(v)
        out = self._out(out)
        _lib.check(self.lib.pg_ring(self.h, _ptr(v), _ptr(out), _stream()), "pg_ring")
        return out

    def ringv(self, vx, vy, vz, out=None):
        vx, vy, vz = self.field(vx), self.field(vy), self.field(vz)
        out = self._out(out)
        _lib.check(self.lib.pg_ringv(self.h, _ptr(vx), _ptr(vy), _ptr(vz), _ptr(out), _stream()), "pg_ringv")
        return out

    def grad(self, v):
        v = self.field(v)
        gx, gy, gz = self.empty(), self.empty(), self.empty()
        _lib.check(self.lib.pg_grad(self.h, _ptr(v), _ptr(gx), _ptr(gy), _ptr(gz), _stream()), "pg_grad")
        return [gx, gy, gz]

    def div(self, fx, fy, fz, out=None):
        fx, fy, fz = self.field(fx), self.field(fy), self.field(fz)
        out = self._out(out)
        _lib.check(self.lib.pg_div(self.h, _ptr(fx), _ptr(fy), _ptr(fz), _ptr(out), _stream()), "pg_div")
        return out

    def mesh(self, which):
        """pg_mesh_var: 0-2 native coordinates, 3-5 d1 d2 d3, 6 GridLen, 7 CellVol,
        8-9 the filtered cell volumes, 10 det J, 11-19 dA/dx .. dC/dz (curvilinear)."""
        out = self.empty()
        _lib.check(self.lib.pg_mesh(self.h, which, _ptr(out), _stream()), "pg_mesh")
        return out

    def set_mesh_coords(self, x, y, z, mesh_periodic=True):
        """setup_mesh_x3 (parcop.f90:73-81): the coordinates of a curvilinear grid and
        its metrics; mesh_periodic is pyranda's 'periodicGrid' option."""
        x, y, z = self.field(x), self.field(y), self.field(z)
        _lib.check(self.lib.pg_set_mesh_coords(self.h, _ptr(x), _ptr(y), _ptr(z), 1 if mesh_periodic else 0,
                                               _stream()), "pg_set_mesh_coords")

    # ---------------------------------------------------- time step and reductions
    def scalar(self):
        return torch.empty((), dtype=torch.float64, device=self.device)

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
        out = self.scalar() if out is None else out
        _lib.check(self.lib.pg_courant(self.h, _ptr(u), vp, wp, _ptr(c), vc, wc, _ptr(out), _stream()),
                   "pg_courant")
        return out

    def diff(self, bulk, rho, out=None):
        bulk, rho = self.field(bulk), self.field(rho)
        out = self.scalar() if out is None else out
        _lib.check(self.lib.pg_diff(self.h, _ptr(bulk), _ptr(rho), _ptr(out), _stream()), "pg_diff")
        return out

    def reduce(self, op, v, out=None):
        """op: 0 sum, 1 max, 2 min over a field (or any float64 device tensor)."""
        if not isinstance(v, torch.Tensor):
            return float(v)
        if v.dtype != torch.float64 or v.device != self.device or not v.is_contiguous():
            if not (tuple(v.shape) == self.n and self._fortran_ok(v) and v.dtype == torch.float64):
                v = v.to(device=self.device, dtype=torch.float64).contiguous()
        out = self.scalar() if out is None else out
        _lib.check(self.lib.pg_reduce(self.h, op, _ptr(v), v.numel(), _ptr(out), _stream()), "pg_reduce")
        return out

    @property
    def member_points(self):
        return float(self.npts)

    def reduce_value(self, op, v):
        """Host value of a global reduction (a number times npts for sums of constants)."""
        if not isinstance(v, torch.Tensor):
            return float(v) * self.npts if op == 0 else float(v)
        return float(self.reduce(op, v))

    def plane(self, axis, k):
        """Index of plane k (negative counts from the end) along an axis."""
        idx = [slice(None)] * 3
        idx[_DIRS[axis] if isinstance(axis, str) else int(axis)] = k
        return tuple(idx)

    def get_plane(self, a, axis, k):
        return a[self.plane(axis, k)]

    def set_plane(self, a, axis, k, value):
        """a[plane] = value (a number or a plane of values); no host copies, so it records in a CUDA graph."""
        a[self.plane(axis, k)] = value

    def rk_stage(self, U, PHI, F, dt, A, B):
        n = len(U)
        arr = ctypes.c_void_p * n
        u = arr(*[t.data_ptr() for t in U])
        p = arr(*[t.data_ptr() for t in PHI])
        f = arr(*[t.data_ptr() for t in F])
        _lib.check(self.lib.pg_rk_stage(self.h, n, u, p, f, _ptr(dt), float(A), float(B), _stream()),
                   "pg_rk_stage")

    def check_finite(self, v, flag):
        _lib.check(self.lib.pg_check_finite(_ptr(v), v.numel(), _ptr(flag), _stream()), "pg_check_finite")
