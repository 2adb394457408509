"""Learned LAD closure: an MLP standing in for the artificial bulk viscosity
beta and conductivity kappa of the LAD method, trained on the GPU by this
library's own kernels.

The plain closure (examples/ISSW_cyl.py:101-104 with the shock problem's
coefficients) is
    beta  = gbar( |ring(div u)| rho ) * 7e-2
    kappa = gbar( ring(T) rho cv / (T dt) ) * 1e-3,
which costs two ring operators (six 8th-derivative sweeps) and two Gaussian
filters (six sweeps) per RK stage.  The learned closure replaces them with one
pass for |grad rho| (second-order central differences,
``pg_lad_grad_magnitude``) and one fused feature-gather + MLP kernel
(``pg_lad_closure``).  The plain closure stays
both the reference for the learned one's error and its fallback: the kernel raises
a flag when a prediction leaves the training range, and
``pyrandaLearnedLAD.step`` then re-runs that RK step with the plain closure
from the step's conserved state.

Network inputs, outputs and normalisation are documented with the C ABI
(include/pyranda_gpu.h, ``pg_lad_*``).
"""
import ctypes
import math
import os

import numpy
import torch

from . import _lib
from .grid import _ptr, _stream
from .pyrandaPackage import pyrandaPackage

NIN, NK, NH, NOUT = _lib.PG_LAD_IN, _lib.PG_LAD_K, _lib.PG_LAD_HIDDEN, _lib.PG_LAD_OUT
NW, NP = _lib.PG_LAD_NWEIGHT, _lib.PG_LAD_NPARAM
# offsets of the parameter layout
OFF = {"w1": (0, NH * NK), "w2": (NH * NK, NH * NH), "w3": (NH * NK + NH * NH, NH * NH),
       "w4": (NH * NK + 2 * NH * NH, NOUT * NH), "b1": (NW, NH), "b2": (NW + NH, NH), "b3": (NW + 2 * NH, NH),
       "b4": (NW + 3 * NH, NOUT)}
BETA_COEF, KAPPA_COEF = 7.0e-2, 1.0e-3


class LadModel:
    """Parameters and normalisation of the closure network (all on the device)."""

    def __init__(self, device="cuda", seed=0):
        self.device = torch.device(device)
        g = numpy.random.default_rng(seed)
        p = numpy.zeros(NP, dtype=numpy.float32)
        for name, fan_in in (("w1", NK), ("w2", NH), ("w3", NH), ("w4", NH)):
            o, n = OFF[name]
            p[o:o + n] = g.standard_normal(n) * math.sqrt(2.0 / fan_in)   # He initialisation
        self.params = torch.from_numpy(p).to(self.device)
        self.wbf16 = self.params[:NW].to(torch.bfloat16).contiguous()
        self.xmean = torch.zeros(NK, dtype=torch.float32, device=self.device)
        self.xinvstd = torch.ones(NK, dtype=torch.float32, device=self.device)
        self.ym, self.ys = [0.0, 0.0], [1.0, 1.0]
        self.ylo, self.yhi = [-1e30, -1e30], [1e30, 1e30]

    def struct(self):
        m = _lib.pg_lad_model()
        m.wbf16 = self.wbf16.data_ptr()
        m.params = self.params.data_ptr()
        m.xmean = self.xmean.data_ptr()
        m.xinvstd = self.xinvstd.data_ptr()
        for i in range(2):
            m.ym[i], m.ys[i], m.ylo[i], m.yhi[i] = self.ym[i], self.ys[i], self.ylo[i], self.yhi[i]
        return m

    def sync_bf16(self):
        self.wbf16.copy_(self.params[:NW].to(torch.bfloat16))

    def save(self, path):
        numpy.savez(path, params=self.params.cpu().numpy(), xmean=self.xmean.cpu().numpy(),
                    xinvstd=self.xinvstd.cpu().numpy(), ym=numpy.array(self.ym), ys=numpy.array(self.ys),
                    ylo=numpy.array(self.ylo), yhi=numpy.array(self.yhi))

    @classmethod
    def load(cls, path, device="cuda"):
        z = numpy.load(path)
        m = cls(device)
        m.params.copy_(torch.from_numpy(z["params"].astype(numpy.float32)))
        m.sync_bf16()
        m.xmean.copy_(torch.from_numpy(z["xmean"].astype(numpy.float32)))
        m.xinvstd.copy_(torch.from_numpy(z["xinvstd"].astype(numpy.float32)))
        m.ym, m.ys = [float(v) for v in z["ym"]], [float(v) for v in z["ys"]]
        m.ylo, m.yhi = [float(v) for v in z["ylo"]], [float(v) for v in z["yhi"]]
        return m


# ------------------------------------------------------------------ features
def grad_magnitude(grid, rho):
    """|grad rho| by second-order central differences (pg_lad_grad_magnitude): one pass over rho."""
    out = grid.empty()
    _lib.check(grid.lib.pg_lad_grad_magnitude(grid.h, _ptr(grid.field(rho)), _ptr(out), _stream()),
               "pg_lad_grad_magnitude")
    return out


def raw_features(grid, div, gmag, pts):
    """Raw feature rows [len(pts), NK] (float32, device) of flat point indices pts."""
    pts = pts.to(device=grid.device, dtype=torch.int64).contiguous()
    raw = torch.empty((pts.numel(), NK), dtype=torch.float32, device=grid.device)
    _lib.check(grid.lib.pg_lad_features(grid.h, _ptr(grid.field(div)), _ptr(grid.field(gmag)), _ptr(pts),
                                        pts.numel(), _ptr(raw), _stream()), "pg_lad_features")
    return raw


def normalize(raw, model):
    X = torch.empty((raw.shape[0], NK), dtype=torch.bfloat16, device=raw.device)
    _lib.check(_lib.load().pg_lad_normalize(_ptr(raw), raw.shape[0], _ptr(model.xmean), _ptr(model.xinvstd),
                                            _ptr(X), _stream()), "pg_lad_normalize")
    return X


def targets(beta, kappa, rho, dt, cv, delta):
    """Normalised targets of the plain closure: beta/(rho D), kappa dt/(rho cv D^2)."""
    y0 = beta / (rho * delta)
    y1 = kappa * dt / (rho * cv * delta * delta)
    return torch.stack([y0.reshape(-1), y1.reshape(-1)], dim=1)


def _flat(f):
    """A Fortran-ordered (nx, ny, nz) field as the vector of its points in memory order."""
    return f.permute(2, 1, 0).reshape(-1)


# ------------------------------------------------------------------ training
class Trainer:
    """Adam on the MSE of the normalised targets, with the library's kernels."""

    def __init__(self, model, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        self.model = model
        self.lib = _lib.load()
        dev = model.device
        self.m = torch.zeros(NP, dtype=torch.float32, device=dev)
        self.v = torch.zeros(NP, dtype=torch.float32, device=dev)
        self.grad = torch.zeros(NP, dtype=torch.float32, device=dev)
        self.loss = torch.zeros(1, dtype=torch.float32, device=dev)
        self.lr, self.betas, self.eps = lr, betas, eps
        self.t = 0

    def gradient(self, X, T, Y=None):
        """Zero, then accumulate dL/dparams of one batch; returns the device loss."""
        self.grad.zero_()
        self.loss.zero_()
        m = self.model.struct()
        rows = X.shape[0]
        _lib.check(self.lib.pg_lad_train_step(ctypes.byref(m), _ptr(X), _ptr(T), rows, 1.0 / (rows * NOUT),
                                              _ptr(self.grad), _ptr(self.loss), _ptr(Y) if Y is not None else None,
                                              _stream()), "pg_lad_train_step")
        return self.loss

    def step(self, X, T):
        loss = self.gradient(X, T)
        self.t += 1
        _lib.check(self.lib.pg_lad_adam(_ptr(self.model.params), _ptr(self.m), _ptr(self.v), _ptr(self.grad), NP,
                                        self.lr, self.betas[0], self.betas[1], self.eps, self.t,
                                        _ptr(self.model.wbf16), NW, _stream()), "pg_lad_adam")
        return loss


def fit_normalisation(model, raw, T, margin=0.25):
    """Input and output statistics of a training set; columns constant over it are switched off."""
    xm = raw.mean(dim=0)
    xs = raw.std(dim=0)
    inv = torch.where(xs > 1e-9 * xm.abs().clamp(min=1e-30), 1.0 / xs.clamp(min=1e-30), torch.zeros_like(xs))
    model.xmean.copy_(xm)
    model.xinvstd.copy_(inv)
    tm, ts = T.mean(dim=0), T.std(dim=0).clamp(min=1e-12)
    model.ym, model.ys = [float(v) for v in tm], [float(v) for v in ts]
    Tn = (T - tm) / ts
    lo, hi = Tn.min(dim=0).values, Tn.max(dim=0).values
    span = hi - lo
    model.ylo = [float(v) for v in lo - margin * span]
    model.yhi = [float(v) for v in hi + margin * span]
    return Tn.contiguous()


def train(model, X, Tn, iters=3000, batch=8192, lr=1e-3, seed=0, log_every=0, cosine=False):
    """Adam over random batches of (X, Tn); returns the loss history (host floats, one per log point).

    cosine: the learning rate follows lr (1 + cos(pi it / iters)) / 2 down to zero."""
    tr = Trainer(model, lr=lr)
    gen = torch.Generator(device=X.device).manual_seed(seed)
    hist = []
    for it in range(iters):
        if cosine:
            tr.lr = lr * 0.5 * (1.0 + math.cos(math.pi * it / iters))
        idx = torch.randint(0, X.shape[0], (min(batch, X.shape[0]),), device=X.device, generator=gen)
        loss = tr.step(X.index_select(0, idx).contiguous(), Tn.index_select(0, idx).contiguous())
        if log_every and (it % log_every == 0 or it == iters - 1):
            hist.append(float(loss.item()))
    return hist


def shock_training_set(runs=20, snapshots_per_run=100, shape=(128, 64, 64), points=2048, seed=1,
                       steps_between=1, precision="fp32"):
    """Snapshots of seeded shock-interface runs with the plain closure.

    The default grid is 128 x 64 x 64 on [0, 4] x [0, 1)^2 (spacing 4/128 in x,
    1/64 in y and z); 256 x 64 x 64 has equal spacings, like the 512 x 128 x 128
    shock problem the closure serves.
    Mach ~ U[1.2, 3.0] and amplitude ~ U[0.01, 0.1] from default_rng(seed);
    each snapshot contributes `points` points, half where beta is largest
    (shock and interface) and half uniformly at random.  Returns
    (raw features [S, NK] float32, targets [S, 2] float64) on the device.
    """
    from . import problems
    from .pyranda import pyrandaSim
    from .pyrandaBC import pyrandaBC
    from .pyrandaTimestep import pyrandaTimestep

    def packs(s):
        s.addPackage(pyrandaBC(s))
        s.addPackage(pyrandaTimestep(s))

    rng = numpy.random.default_rng(seed)
    raws, tgts, meta = [], [], []
    for r in range(runs):
        mach, amp = float(rng.uniform(1.2, 3.0)), float(rng.uniform(0.01, 0.1))
        ss = problems.build_shock(pyrandaSim, *shape, packs, mach=mach, amp=amp, silent=True, precision=precision)
        ss.use_graphs(True)
        g = ss.grid
        delta = max(g.mesh_d)      # the closure's length scale (pg_lad_closure)
        gen = torch.Generator(device=g.device).manual_seed(int(rng.integers(1 << 30)))
        t = 0.0
        for s in range(snapshots_per_run):
            for _ in range(steps_between):
                t = ss.rk4(t, ss.variables["dt"].data)
            V = ss.variables
            div, rho, beta, kappa = V["div"].data, V["rho"].data, V["beta"].data, V["kappa"].data
            if not bool(torch.isfinite(rho).all()):
                break
            gmag = grad_magnitude(g, rho)
            # flat point index p = i + nx (j + ny k), the kernels' order
            top = torch.topk(_flat(beta), points // 2).indices
            rnd = torch.randint(0, g.npts, (points - points // 2,), device=g.device, generator=gen)
            pts = torch.cat([top, rnd])
            raws.append(raw_features(g, div, gmag, pts))
            pick = lambda f: _flat(f).index_select(0, pts)  # noqa: E731
            tgts.append(targets(pick(beta), pick(kappa), pick(rho), V["dt"].data, problems.CV, delta))
        meta.append((mach, amp, s + 1))
        del ss
    return torch.cat(raws), torch.cat(tgts).to(torch.float32), meta


# --------------------------------------------------------------- simulation
LEARNED_LAD = ("[:beta:,:kappa:] = lad.closure(:div:,:rho:,:T:,:dt:)")


class pyrandaLearnedLAD(pyrandaPackage):
    """``lad.closure(div, rho, T, dt)`` -> [beta, kappa], learned or plain.

    mode 'learned' evaluates the network (the fallback flag accumulates on
    the device), 'plain' the LAD operators, 'off' returns zeros (the method
    without a closure, for comparison).
    """

    def __init__(self, pysim, model, cv, mode="learned"):
        pyrandaPackage.__init__(self, "LAD", pysim)
        self.model = model
        self.cv = float(cv)
        self.mode = mode
        self.flag = torch.zeros(1, dtype=torch.int32, device=pysim.grid.device)
        self.fallbacks = 0
        self._m = model.struct()

    def get_sMap(self):
        self.sMap = {"lad.closure(": "self.packages['LAD'].closure("}

    def closure(self, div, rho, T, dt):
        ss, g = self.pyranda, self.pyranda.grid
        if self.mode == "plain":
            beta = g.filter("gaussian", torch.abs(g.ring(div)) * rho) * BETA_COEF
            kappa = g.filter("gaussian", g.ring(T) * rho * self.cv / (T * dt)) * KAPPA_COEF
            return [beta, kappa]
        if self.mode == "off":
            return [ss.emptyScalar(), ss.emptyScalar()]
        rho = g.field(rho)
        gmag = grad_magnitude(g, rho)
        beta, kappa = g.empty(), g.empty()
        dtd = dt if isinstance(dt, torch.Tensor) else torch.full((), float(dt), dtype=torch.float64,
                                                                  device=g.device)
        _lib.check(g.lib.pg_lad_closure(g.h, ctypes.byref(self._m), _ptr(g.field(div)), _ptr(gmag), _ptr(rho),
                                        _ptr(dtd), self.cv, _ptr(beta), _ptr(kappa), _ptr(self.flag), _stream()),
                   "pg_lad_closure")
        return [beta, kappa]

    def _state_names(self):
        """The state a step reads before writing: the conserved variables, the
        variables the PDE right-hand sides read (the first stage uses them as
        the previous step left them), and the variables the algebraic
        equations read before writing or never write (e.g. :dt: in kappa)."""
        if getattr(self, "_state", None) is None:
            from .pyrandaUtils import findVar
            ss = self.pyranda
            need = set(ss.conserved)
            written = set()
            for eq in ss.equations:
                rhs = eq.eqstr.split("=", 1)[1] if eq.LHS else eq.eqstr
                if eq.kind == "PDE":
                    need.update(findVar(rhs, "scalar"))
                    continue
                need.update(v for v in findVar(rhs, "scalar") if v not in written)
                written.update(eq.LHS or [])
            self._state = sorted(v for v in need if v in ss.variables)
        return self._state

    def step(self, time, dt):
        """One rk4 step with the learned closure; if the flag was raised, redo it with the plain closure.

        What the step reads before writing is kept (``_state_names``).  On a
        fallback it is restored and the step runs again with the plain
        closure (eagerly; a recorded graph's storage is refreshed afterwards),
        so the result equals a plain-closure step from the same state.
        """
        ss = self.pyranda
        saved = {n: ss.variables[n].data.clone() for n in self._state_names()
                 if isinstance(ss.variables[n].data, torch.Tensor)}
        dt_saved = dt.clone() if isinstance(dt, torch.Tensor) else dt
        self.flag.zero_()
        t = ss.rk4(time, dt)
        if int(self.flag.item()) == 0:
            return t
        self.fallbacks += 1
        for n, d in saved.items():   # in place: a recorded graph keeps reading the same storage
            v = ss.variables[n]
            if isinstance(v.data, torch.Tensor) and v.data.shape == d.shape:
                v.data.copy_(d)
            else:
                v.data = d
        graphs = ss._graphs_enabled
        ss._graphs_enabled = False
        self.mode = "plain"
        try:
            t = ss.rk4(time, dt_saved)
        finally:
            self.mode = "learned"
            ss._graphs_enabled = graphs
            if graphs:
                ss.sync_graph_storage()
        return t


def learned_shock_eom():
    """The shock problem's EOM with the learned closure in place of the plain one."""
    from . import problems
    return problems.SHOCK_EOM.replace(problems.PLAIN_LAD.replace("CV", repr(problems.CV)), LEARNED_LAD)


DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "lad_shock.npz")
