"""Throughput of the 256^3 compressible Taylor-Green RK step on GB300.

Metric: Mpoint-RK-steps/s = nx*ny*nz*steps / seconds / 1e6 for the
compressible Taylor-Green vortex at Mach 0.1 and Re 1600 (the EOM of pyranda's
examples/TaylorGreen.py -- Navier-Stokes with LAD artificial viscosity,
compact filters, 10th-order Pade derivatives, LSRK(5,4) with the ALG update
after every stage -- plus the physical viscosity) on a periodic 256^3 grid.

Headline (``value``): the fastest split-precision path -- dense split-TF32
or FP32 banded compact sweeps (exact fixed-point d8 RHS) on FP64 fields,
FP64 RK state and reductions, fused FP64 EOM arithmetic, the whole step
recorded in a CUDA graph.  The same line reports the plain FP64 path
(reference arithmetic) and the field L2 error of every fast path against it,
after the timed steps and after --err-steps steps (200: the configuration's
run length).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
Under torchrun each rank runs an independent replica (the path does not shard:
one grid per GPU), value = all ranks' points*steps / max-over-ranks time.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpoint-RK-steps/s at 256³ TGV on 1 GB300: plain FP64 vs split-FP32+graphs, at L2 err"
UNIT = "Mpoint-RK-steps/s"
CFL = 0.5


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--n", type=int, default=256, help="grid points per direction")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    p.add_argument("--err-steps", type=int, default=200,
                   help="steps after which the headline path's field error against FP64 is reported again "
                        "(0: only after the timed steps)")
    p.add_argument("--no-fusion", action="store_true", help="fast paths without the fused EOM kernels")
    p.add_argument("--fusion-arith", default="fp64", choices=["fp32", "fp64", "df64"],
                   help="arithmetic of the fast paths' fused EOM kernels (fp64: bit-exact with unfused; "
                        "fp32: FP32 arithmetic between FP64 fields; df64: double-float FP32 pairs, ~48 bits)")
    p.add_argument("--mode", default="step", choices=["step", "sweeps", "profile", "peaks", "shock", "ensemble",
                                                      "shock-learned", "kernels", "lad"],
                   help="sweeps: time every directional sweep kernel alone on one n^3 field; "
                        "profile: one eager RK step between cudaProfilerStart/Stop (for ncu); "
                        "peaks: HBM copy, FP64 and FP32 GEMM rates; "
                        "shock: throughput of the 512x128x128 shock-interface problem; "
                        "ensemble: 64 Kelvin-Helmholtz 2-D runs of seeded sizes advanced together; "
                        "shock-learned: 512x128x128 shock-interface with the learned LAD closure against "
                        "the plain one (trains the closure first when no trained model is found); "
                        "kernels: d1, compact-filter and d8 sweeps on one periodic n^3 field at --precision "
                        "(a light target for profilers); "
                        "lad: the learned-closure kernel alone on a 512x128x128 grid (a light target for profilers)")
    p.add_argument("--model", default=None, help="shock-learned: trained closure (.npz); default: the packaged one")
    p.add_argument("--train-runs", type=int, default=20, help="shock-learned: training runs when training")
    p.add_argument("--train-iters", type=int, default=3000, help="shock-learned: Adam iterations when training")
    p.add_argument("--train-cosine", action="store_true", help="shock-learned: cosine learning-rate decay")
    p.add_argument("--train-shape", default="128,64,64", help="shock-learned: grid of the training runs")
    p.add_argument("--save-model", default=None, help="shock-learned: where a newly trained closure is saved "
                                                      "(default pyranda_gb300/_build/lad_shock_trained.npz)")
    p.add_argument("--members", type=int, default=64, help="ensemble mode: number of members")
    p.add_argument("--precision", default="fp32",
                   choices=["fp32", "fp64", "dense", "auto", "fp32-only", "fp32-split", "fp64-split"],
                   help="profile mode: arithmetic of the profiled step; step mode: 'fp32-only' skips the dense run; "
                        "kernels mode: '-split' runs the split-line banded sweeps")
    p.add_argument("--reps", type=int, default=20)
    p.add_argument("--no-subconfigs", action="store_true",
                   help="step mode: skip the short ensemble (64 Kelvin-Helmholtz members) and learned-closure "
                        "sub-lines")
    p.add_argument("--sub-steps", type=int, default=5, help="step mode: timed steps of each sub-line")
    return p.parse_args()


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        rows = []
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------- CPU baseline
def _cpu_worker(args):
    """One oracle process: TGV on its own sub-grid, single-threaded OpenMP."""
    shape, steps, warmup = args
    os.environ["OMP_NUM_THREADS"] = "1"
    sys.path.insert(0, ROOT)
    from oracle import oracle
    from pyranda_gb300 import problems
    oracle.set_threads(1)
    import numpy

    mesh = "\n".join("%sdom = (0.0, %r, %d, periodic=True)" % (ax, 2 * math.pi * (n - 1) / n, n)
                     for ax, n in zip("xyz", shape))
    ss = oracle.OracleSim("TG", mesh)
    ss.addPackage("Timestep")
    ss.EOM(problems.TGV_EOM_NS)
    ss.setIC(problems.TGV_IC_NS)
    dt = ss.variables["dt"].data * CFL
    t = 0.0
    for _ in range(warmup):
        t = ss.rk4(t, dt)
        dt = ss.variables["dt"].data * CFL
    t0 = time.perf_counter()
    for _ in range(steps):
        t = ss.rk4(t, dt)
        dt = ss.variables["dt"].data * CFL
    wall = time.perf_counter() - t0
    return int(numpy.prod(shape)), steps, wall


def cpu_baseline(steps, warmup, shape=(128, 128, 64)):
    """The oracle (a CPU port of parcop + pyranda's driver) on every host core.

    One single-threaded process per core, each on its own periodic sub-grid
    of the Taylor-Green problem (the per-point work of a decomposed run
    without its halo exchange).  Returns (Mpoint-RK-steps/s, cores, sample).
    """
    import multiprocessing as mp
    from oracle import oracle
    oracle.build()
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        res = pool.map(_cpu_worker, [(shape, steps, warmup)] * cores)
    pts = sum(r[0] * r[1] for r in res)
    wall = max(r[2] for r in res)
    sample = ("%d processes x TGV %dx%dx%d periodic, %d timed RK steps each after %d warm-up, "
              "oracle (CPU port of parcop, FP64), 1 thread per process" % (cores, *shape, steps, warmup))
    return pts / wall / 1e6, cores, sample, wall


# --------------------------------------------------------------------------- distributed
def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def run_reference(args):
    world, rank, _ = dist_setup()
    if rank != 0:
        return 0
    k = max(1, args.steps)
    w = max(0, args.warmup)
    # size the per-step sample so the whole run stays within a few minutes
    est_us_per_pt_step = 6.0
    budget_s = 150.0 / (k + w)
    shapes = [(128, 128, 64), (96, 96, 64), (64, 64, 64), (64, 64, 32), (32, 32, 32)]
    shape = shapes[-1]
    for s in shapes:
        if s[0] * s[1] * s[2] * est_us_per_pt_step * 1e-6 <= budget_s:
            shape = s
            break
    v, cores, sample, wall = cpu_baseline(k, w, shape)
    line = {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "n_gpus": args.gpus, "steps": k, "warmup": w,
            "ms_per_step": round(wall / k * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (Taylor-Green initial condition, Mach 0.1)",
            "impl": "reference",
            "config": {"workload": "compressible Taylor-Green vortex, Mach 0.1, Re 1600, periodic, LAD + compact "
                                   "filters, LSRK(5,4)",
                       "grid": [args.n] * 3, "cpu_sample_grid": list(shape)},
            "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------------------------------ GPU
def make_sim(n, precision, graphs, fusion=False, arith="fp64"):
    from pyranda_gb300 import pyrandaSim, pyrandaTimestep, problems
    ss = problems.build_tgv(pyrandaSim, n, lambda s: s.addPackage(pyrandaTimestep(s)), ns=True, silent=True,
                            precision=precision)
    if graphs:
        ss.use_graphs(True)
    if fusion:
        ss.use_fusion(True, arithmetic=arith)
    return ss


def run_steps(ss, k, t0=0.0):
    t = t0
    for _ in range(k):
        dt = ss.variables["dt"].data * CFL
        t = ss.rk4(t, dt)
    return t


def max_over_ranks(seconds, dist_on, device=None):
    """Largest per-rank time (the job's time) under torch.distributed, else itself."""
    if not dist_on:
        return float(seconds)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(npts, steps, world, seconds):
    """Whole-job Mpoint-RK-steps/s: every rank advances its own replica."""
    return npts * steps * world / seconds / 1e6


def time_steps(ss, k, torch, dist_on):
    """CUDA-event time of k steps on the current stream, barrier + sync around."""
    if dist_on:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    run_steps(ss, k)
    e.record()
    torch.cuda.synchronize()
    if dist_on:
        dist.barrier()
    return s.elapsed_time(e) / 1e3


def sweep_roofline(ss, torch, reps=20):
    """Average CUDA-event duration of each sweep kernel class on one 256^3 field."""
    g = ss.grid
    v = ss.variables["rho"].data
    out = g.empty()
    res = {}
    cases = {
        "d1": lambda d: g.d1(d, v, out=out),
        "sfilter": lambda d: g.filter("spectral", v, d, out=out),
        "d8": lambda d: g.d8(d, v, out=out),
        "gfilter": lambda d: g.filter("gaussian", v, d, out=out),
    }
    for name, f in cases.items():
        for d in range(3):
            f(d)
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            for _ in range(reps):
                f(d)
            e.record()
            torch.cuda.synchronize()
            res["%s_%s" % (name, "xyz"[d])] = s.elapsed_time(e) / reps / 1e3
    return res


# DRAM bytes (ncu dram__bytes_read.sum + dram__bytes_write.sum) of one launch
# of each sweep kernel class at 256^3, from the captures summarised in
# profiles/ (carried over: measured on the kernel build named in the file, not
# re-measured by this run).  Key: (operator, direction, dense or banded).
NCU_TRAFFIC_256 = {
    ("sf", "y", "dense"): (136362752 + 88161280, "profiles/roofline_traffic_256.md"),
    ("sf", "y", "banded"): (275878656 + 163471872, "profiles/roofline_traffic_256.md"),
    ("d1", "x", "split"): (134330112 + 96838400, "profiles/seg_sweeps_256.md"),
    ("d1", "z", "split"): (134425600 + 98427648, "profiles/seg_sweeps_256.md"),
}


def sweep_counts(prec, arith, fusion):
    """Directional sweeps per RK step of the TGV problem, per (operator,
    direction), counted at the Grid API of an eager 32^3 copy of the problem
    (the counts do not depend on the grid size): ddx/ddy/ddz = one d1 sweep,
    fbar / gbar = three filter sweeps, ring = three d8 sweeps, grad and div =
    three d1 sweeps."""
    import collections
    ss = make_sim(32, prec, graphs=False, fusion=fusion, arith=arith)
    run_steps(ss, 1)
    g = ss.grid
    cnt = collections.Counter()
    all3 = (0, 1, 2)

    def wrap(name, sweeps):
        orig = getattr(g, name)

        def counted(*a, **kw):
            for key in sweeps(*a, **kw):
                cnt[key] += 1
            return orig(*a, **kw)
        setattr(g, name, counted)

    wrap("d1", lambda d, *a, **k: [("d1", d)])
    wrap("d8", lambda d, *a, **k: [("d8", d)])
    wrap("filter", lambda kind, v, direction=3, **k: [("sf" if kind == "spectral" else "gf", dd)
                                                       for dd in (all3 if direction == 3 else (direction,))])
    wrap("ring", lambda *a, **k: [("d8", d) for d in all3])
    wrap("ringv", lambda *a, **k: [("d8", d) for d in all3 for _ in range(3)])
    wrap("grad", lambda *a, **k: [("d1", d) for d in all3])
    wrap("div", lambda *a, **k: [("d1", d) for d in all3])
    run_steps(ss, 1)
    del ss
    return dict(cnt)


def l2_errors(a, b, names):
    out = {}
    for n in names:
        x, y = a.variables[n].data, b.variables[n].data
        out[n] = float(((x - y).norm() / y.norm()).item())
    return out


def linf_errors(a, b, names):
    """max |a - b| / max |b| per field."""
    out = {}
    for n in names:
        x, y = a.variables[n].data, b.variables[n].data
        out[n] = float(((x - y).abs().max() / y.abs().max()).item())
    return out


def momentum_error(a, b, names=("rhou", "rhov", "rhow")):
    """Relative L2 error of the momentum vector field (rho u, rho v, rho w) of `a` against `b`."""
    num = sum(float((a.variables[n].data - b.variables[n].data).norm()) ** 2 for n in names)
    den = sum(float(b.variables[n].data.norm()) ** 2 for n in names)
    return (num / den) ** 0.5


def sweeps_only(args):
    """Per-sweep CUDA-event timings on one periodic n^3 TGV field: FP32 banded (one thread per line and split
    lines), dense split-TF32 and FP64 banded."""
    import torch
    torch.cuda.set_device(0)
    npts = args.n ** 3
    out = {"n": args.n}
    for prec in ("fp32", "fp32-split", "dense", "fp64"):
        ss = make_sim(args.n, prec.split("-")[0], graphs=False)
        if prec.endswith("split"):
            ss.grid.set_line_split(True)
        sw = sweep_roofline(ss, torch, reps=args.reps)
        out[prec] = {k: {"ms": round(v * 1e3, 4), "GB/s": round(16.0 * npts / v / 1e9, 1)} for k, v in sw.items()}
        del ss
        torch.cuda.empty_cache()
    print(json.dumps(out), flush=True)
    return 0


def kernel_sweeps(args):
    """d1, compact-filter and d8 sweeps in x, y, z on one periodic n^3 field (two fields on the device)."""
    import torch
    from pyranda_gb300.grid import Grid
    torch.cuda.set_device(0)
    n = args.n
    g = Grid((n, n, n), (True, True, True), (0, 0, 0), (2 * math.pi * (n - 1) / n,) * 3,
             precision=args.precision.split("-")[0], line_split=args.precision.endswith("split"))
    v = g.mesh(0)
    v.copy_(torch.sin(v) + 2.0)
    out = g.empty()
    res = {}
    for name, f in (("d1", lambda d: g.d1(d, v, out=out)), ("sfilter", lambda d: g.filter("spectral", v, d, out=out)),
                    ("d8", lambda d: g.d8(d, v, out=out))):
        for d in range(3):
            f(d)
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            for _ in range(args.reps):
                f(d)
            e.record()
            torch.cuda.synchronize()
            ms = s.elapsed_time(e) / args.reps
            res["%s_%s" % (name, "xyz"[d])] = {"ms": round(ms, 4), "GB/s": round(16.0 * n ** 3 / ms / 1e6, 1)}
    print(json.dumps({"n": n, "precision": args.precision, "sweeps": res}), flush=True)
    return 0


def lad_kernel(args):
    """pg_lad_closure alone on a 512x128x128 grid with seeded fields and an untrained network."""
    import ctypes
    import torch
    from pyranda_gb300.grid import Grid, _ptr, _stream
    from pyranda_gb300 import learned_lad as LL
    torch.cuda.set_device(0)
    g = Grid((512, 128, 128), (False, True, True), (0, 0, 0), (4.0, 127 / 128, 127 / 128), precision="fp32")
    gen = torch.Generator(device="cuda").manual_seed(0)
    div, gm, rho = (g.empty() for _ in range(3))
    for t in (div, gm, rho):
        t.copy_(torch.rand(t.shape, generator=gen, device="cuda", dtype=torch.float64).permute(0, 1, 2))
    rho += 1.0
    dt = torch.full((), 1e-3, dtype=torch.float64, device="cuda")
    m = LL.LadModel("cuda", seed=0)
    mm = m.struct()
    beta, kappa = g.empty(), g.empty()
    flag = torch.zeros(1, dtype=torch.int32, device="cuda")

    def call():
        return g.lib.pg_lad_closure(g.h, ctypes.byref(mm), _ptr(div), _ptr(gm), _ptr(rho), _ptr(dt), 2.5, _ptr(beta),
                                    _ptr(kappa), _ptr(flag), _stream())
    assert call() == 0
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.reps):
        call()
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / args.reps
    print(json.dumps({"lad_kernel_ms": round(ms, 4), "points": g.npts, "ns_per_point": round(ms * 1e6 / g.npts, 3)}),
          flush=True)
    return 0


def profile_step(args):
    """One eager TGV RK step inside a profiler range, after 2 warm-up steps."""
    import torch
    torch.cuda.set_device(0)
    ss = make_sim(args.n, args.precision, graphs=False, fusion=not args.no_fusion and args.precision != "fp64",
                  arith=args.fusion_arith)
    run_steps(ss, 2)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStart()
    run_steps(ss, 1)
    torch.cuda.synchronize()
    torch.cuda.cudart().cudaProfilerStop()
    return 0


def measure_peaks():
    """Device ceilings measured with library routines (copy, DGEMM, SGEMM)."""
    import torch
    torch.cuda.set_device(0)
    torch.backends.cuda.matmul.allow_tf32 = False
    out = {}

    def best(f, reps=10):
        f()
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            f()
            e.record()
            torch.cuda.synchronize()
            ts.append(s.elapsed_time(e) / 1e3)
        return min(ts)

    a = torch.empty(1 << 28, dtype=torch.float64, device="cuda")
    b = torch.empty_like(a)
    a.fill_(1.0)
    out["hbm_copy_GBps"] = round(2 * a.numel() * 8 / best(lambda: b.copy_(a)) / 1e9, 1)
    del a, b
    for dt, key, n in ((torch.float64, "fp64_gemm_TFLOPs", 8192), (torch.float32, "fp32_gemm_TFLOPs", 8192)):
        x = torch.randn(n, n, dtype=dt, device="cuda")
        y = torch.randn(n, n, dtype=dt, device="cuda")
        out[key] = round(2 * n ** 3 / best(lambda: torch.mm(x, y), 5) / 1e12, 2)
        del x, y
    out["device"] = torch.cuda.get_device_name(0)
    print(json.dumps(out), flush=True)
    return 0


def shock_throughput(args):
    """Mpoint-RK-steps/s of the 512x128x128 shock-interface problem (FP64 and fast path)."""
    import torch
    from pyranda_gb300 import pyrandaSim, pyrandaBC, pyrandaTimestep, problems
    torch.cuda.set_device(0)

    def packs(s):
        s.addPackage(pyrandaBC(s))
        s.addPackage(pyrandaTimestep(s))

    out = {"workload": "shock-interface 512x128x128, x one-sided, y/z periodic, LAD", "steps": args.steps}
    npts = 512 * 128 * 128
    for prec, graphs in (("fp64", False), ("fp32", True), ("auto", True)):
        ss = problems.build_shock(pyrandaSim, 512, 128, 128, packs, silent=True, precision=prec)
        if graphs:
            ss.use_graphs(True)
            ss.use_fusion(True, arithmetic=args.fusion_arith)
        run_steps(ss, max(3, args.warmup))
        sec = time_steps(ss, args.steps, torch, False)
        key = prec + ("+graphs+fusion(%s)" % args.fusion_arith if graphs else "")
        out[key] = {"value": round(job_value(npts, args.steps, 1, sec), 3), "unit": UNIT,
                    "ms_per_step": round(sec / args.steps * 1e3, 3)}
        if prec == "auto":
            out[key]["dense_plan"] = {"%s_%s" % k: v for k, v in ss.grid.dense_plan().items()}
        del ss
        torch.cuda.empty_cache()
    print(json.dumps(out), flush=True)
    return 0


def ensemble_throughput(args):
    """The ensemble mode: print ensemble_result() as one JSON line."""
    print(json.dumps(ensemble_result(args)), flush=True)
    return 0


def ensemble_result(args, one_at_a_time=True):
    """Mpoint-RK-steps/s of 64 Kelvin-Helmholtz runs (n^2, n from {128..512}, seeded) in one ensemble.

    Runs the FP64 ensemble eagerly and the fast path (FP32 sweeps, CUDA graph
    per step), the fast path's field error against FP64 after the same steps,
    the average duration of one x and one y derivative sweep over all members,
    and the members one at a time (one graph-captured simulation per distinct
    size, times its count) for comparison.
    """
    import torch
    from pyranda_gb300 import pyrandaSim, pyrandaBC, pyrandaTimestep, problems
    from pyranda_gb300.ensemble import pyrandaEnsemble
    torch.cuda.set_device(0)

    def packs(s):
        s.addPackage(pyrandaTimestep(s))
        s.addPackage(pyrandaBC(s))

    sizes = problems.kh_sizes(args.members)
    npts = sum(n * n for n in sizes)
    k, w = args.steps, max(3, args.warmup)
    out = {"workload": "Kelvin-Helmholtz 2-D ensemble, %d members n^2 with n from %s (default_rng(0))"
                       % (len(sizes), list(problems.KH_SIZES)),
           "points": npts, "steps": k}

    def run(ens, nsteps, dt):
        t = torch.zeros(ens.M, dtype=torch.float64, device="cuda")
        for _ in range(nsteps):
            t = ens.rk4(t, dt)
            dt = torch.minimum(ens.variables["dt"].data, 1.1 * dt)
        return dt

    res = {}
    for prec, graphs in (("fp64", False), ("fp32", True), ("auto", True)):
        ens = problems.build_kh_ensemble(pyrandaEnsemble, sizes, packs, silent=True, precision=prec)
        if graphs:
            ens.use_graphs(True)
            ens.use_fusion(True, arithmetic=args.fusion_arith)
        dt0 = ens.variables["dt"].data.clone()
        dt = run(ens, w, dt0.clone())
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        run(ens, k, dt)
        e.record()
        torch.cuda.synchronize()
        sec = s.elapsed_time(e) / 1e3
        out[prec + ("+graphs+fusion(%s)" % args.fusion_arith if graphs else "")] = {"value": round(npts * k / sec / 1e6, 3), "unit": UNIT,
                                                            "ms_per_step": round(sec / k * 1e3, 3)}
        res[prec] = ens
    # every precision took the same number of steps from the same IC
    for p in ("fp32", "auto"):
        out["%s_vs_fp64_rel_l2" % p] = {n: float(((res[p].variables[n].data - res["fp64"].variables[n].data).norm()
                                                 / res["fp64"].variables[n].data.norm()).item())
                                       for n in ("rho", "rhou", "rhov", "Et")}
    del res["auto"]
    g = res["fp32"].grid
    v = res["fp32"].variables["rho"].data
    o = g.empty()
    for d in (0, 1):
        g.d1(d, v, out=o)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(args.reps):
            g.d1(d, v, out=o)
        e.record()
        torch.cuda.synchronize()
        ms = s.elapsed_time(e) / args.reps
        out["d1_%s_fp32" % "xy"[d]] = {"ms": round(ms, 4), "GB/s": round(16.0 * npts / (ms * 1e-3) / 1e9, 1)}
    del res, g, v, o
    torch.cuda.empty_cache()
    if not one_at_a_time:
        return out
    # one member at a time: every distinct size once, weighted by its count
    seq = 0.0
    for n in sorted(set(sizes)):
        ss = problems.build_kh(pyrandaSim, n, packs, silent=True, precision="fp32")
        ss.use_graphs(True)
        dt = ss.variables["dt"].data.clone()
        t = 0.0
        for _ in range(w):
            t = ss.rk4(t, dt)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(k):
            t = ss.rk4(t, dt)
        e.record()
        torch.cuda.synchronize()
        seq += s.elapsed_time(e) / 1e3 * sizes.count(n)
        del ss
    out["one_at_a_time_fp32+graphs"] = {"value": round(npts * k / seq / 1e6, 3), "unit": UNIT,
                                        "ms_per_step": round(seq / k * 1e3, 3)}
    return out


def shock_learned(args):
    """The shock-learned mode: print shock_learned_result() as one JSON line."""
    print(json.dumps(shock_learned_result(args)), flush=True)
    return 0


def shock_learned_result(args, train_if_missing=True):
    """C5: the learned LAD closure on the 512x128x128 shock-interface problem.

    Both runs use the fast path (FP32 sweeps, FP64 state, one CUDA graph per
    RK step); each takes its own CFL/diffusion steps, and the learned run is
    advanced to the time the plain run reached, where the densities are
    compared.  Without a trained model the closure is
    first trained here: 2000 snapshots of 20 seeded 128x64x64 runs (Mach in
    [1.2, 3], amplitude in [0.01, 0.1], default_rng(1)), then Adam.
    """
    import torch
    from pyranda_gb300 import pyrandaSim, pyrandaBC, pyrandaTimestep, problems
    from pyranda_gb300 import learned_lad as LL
    torch.cuda.set_device(0)
    out = {"workload": "shock-interface 512x128x128 (Mach 1.5, amplitude 0.05), learned vs plain LAD closure",
           "steps": args.steps}
    path = args.model or LL.DEFAULT_MODEL
    if os.path.exists(path):
        model = LL.LadModel.load(path)
        out["model"] = os.path.relpath(path, ROOT)
    elif not train_if_missing:
        out["skipped"] = "no trained closure at %s" % os.path.relpath(path, ROOT)
        return out
    else:
        t0 = time.time()
        shape = tuple(int(x) for x in args.train_shape.split(","))
        raw, T, meta = LL.shock_training_set(runs=args.train_runs, snapshots_per_run=2000 // args.train_runs,
                                             shape=shape)
        t1 = time.time()
        model = LL.LadModel("cuda", seed=0)
        Tn = LL.fit_normalisation(model, raw, T)
        X = LL.normalize(raw, model)
        hist = LL.train(model, X, Tn, iters=args.train_iters, batch=8192, lr=1e-3,
                        log_every=max(1, args.train_iters // 8), cosine=args.train_cosine)
        torch.cuda.synchronize()
        t2 = time.time()
        save = args.save_model or os.path.join(ROOT, "pyranda_gb300", "_build", "lad_shock_trained.npz")
        os.makedirs(os.path.dirname(os.path.abspath(save)), exist_ok=True)
        model.save(save)
        out["training"] = {"shape": list(shape), "iters": args.train_iters, "cosine": args.train_cosine,
                           "samples": int(raw.shape[0]), "snapshots": sum(m[2] for m in meta),
                           "runs": [[round(a, 4), round(b, 4), c] for a, b, c in meta],
                           "data_s": round(t1 - t0, 1), "train_s": round(t2 - t1, 1), "loss": hist}
        del raw, T, X, Tn
    npts = 512 * 128 * 128
    k, w = args.steps, max(3, args.warmup)

    def build(mode):
        def packs(ss):
            ss.addPackage(pyrandaBC(ss))
            ss.addPackage(pyrandaTimestep(ss))
            ss.addPackage(LL.pyrandaLearnedLAD(ss, model, problems.CV, mode="plain"))
        # the initial state always comes from the plain closure; the run then uses `mode`
        ss = problems.build_shock(pyrandaSim, 512, 128, 128, packs, eom=LL.learned_shock_eom(), silent=True,
                                  precision="auto")
        ss.packages["LAD"].mode = mode
        ss.use_graphs(True)
        ss.use_fusion(True, arithmetic=args.fusion_arith)
        return ss

    def advance(ss, step, t, t_end=None, nmax=None):
        """Own CFL/diffusion steps (the reference scripts' loop); up to t_end or nmax steps."""
        n = 0
        while (nmax is None or n < nmax) and (t_end is None or t < t_end - 1e-12):
            dt = ss.variables["dt"].data
            if t_end is not None:
                dt = torch.clamp(dt, max=t_end - t)
            t = float(step(t, dt))
            n += 1
        return t, n

    plain = build("plain")
    t, _ = advance(plain, plain.rk4, 0.0, nmax=w)
    t_w = t
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    t_end, k_plain = advance(plain, plain.rk4, t, nmax=k)
    e.record()
    torch.cuda.synchronize()
    t_plain = s.elapsed_time(e) / 1e3
    rho_plain = plain.variables["rho"].data.clone()
    del plain
    torch.cuda.empty_cache()
    learned = build("learned")
    lad = learned.packages["LAD"]
    t, _ = advance(learned, lad.step, 0.0, nmax=w)
    t_wl = t
    torch.cuda.synchronize()
    s.record()
    t, k_learn = advance(learned, lad.step, t, t_end=t_end, nmax=20 * k)
    e.record()
    torch.cuda.synchronize()
    t_learn = s.elapsed_time(e) / 1e3
    rho = learned.variables["rho"].data
    l1 = float(((rho - rho_plain).abs().sum() / rho_plain.abs().sum()).item())
    # the closure alone on the final state: learned (|grad rho| + fused gather/MLP) vs plain (2 rings + 2 filters)
    V = learned.variables
    closure_ms = {}
    for mode in ("learned", "plain"):
        lad.mode = mode
        lad.closure(V["div"].data, V["rho"].data, V["T"].data, V["dt"].data)
        torch.cuda.synchronize()
        s.record()
        for _ in range(args.reps):
            lad.closure(V["div"].data, V["rho"].data, V["T"].data, V["dt"].data)
        e.record()
        torch.cuda.synchronize()
        closure_ms[mode] = round(s.elapsed_time(e) / args.reps, 4)
    # both closures on the same (final) state: their extremes set the diffusive time step
    diag = {}
    tsp = learned.packages["Timestep"]
    for mode in ("plain", "learned"):
        lad.mode = mode
        b, kp = lad.closure(V["div"].data, V["rho"].data, V["T"].data, V["dt"].data)
        bs = b.flatten()[::7].float()
        diag[mode] = {"beta_max": float(b.max()), "beta_p999": float(torch.quantile(bs, 0.999)),
                      "beta_mean": float(b.mean()), "kappa_max": float(kp.max()),
                      "dt_beta_limit": 0.2 * float(tsp.diff(b, V["rho"].data))}
        if mode == "plain":
            beta_ref, kappa_ref = b.clone(), kp.clone()
        else:
            diag["beta_rel_l1"] = float((b - beta_ref).abs().sum() / beta_ref.abs().sum())
            diag["kappa_rel_l1"] = float((kp - kappa_ref).abs().sum() / kappa_ref.abs().sum())
    out["closure_on_final_state"] = diag
    lad.mode = "learned"
    # its parts: |grad rho| (one central-difference pass) and the fused feature-gather + network kernel
    g = learned.grid
    gm = LL.grad_magnitude(g, V["rho"].data)
    beta, kappa = g.empty(), g.empty()
    import ctypes
    from pyranda_gb300.grid import _ptr, _stream
    parts = {"grad_magnitude": lambda: LL.grad_magnitude(g, V["rho"].data),
             "lad_kernel": lambda: g.lib.pg_lad_closure(g.h, ctypes.byref(lad._m), _ptr(V["div"].data), _ptr(gm),
                                                       _ptr(V["rho"].data), _ptr(V["dt"].data.reshape(())),
                                                       problems.CV, _ptr(beta), _ptr(kappa), _ptr(lad.flag),
                                                       _stream())}
    for name, f in parts.items():
        f()
        torch.cuda.synchronize()
        s.record()
        for _ in range(args.reps):
            f()
        e.record()
        torch.cuda.synchronize()
        closure_ms[name] = round(s.elapsed_time(e) / args.reps, 4)
    out["closure_ms_per_call"] = closure_ms
    out["precision"] = learned.precision
    out["t_end"] = t_end
    out["plain_lad"] = {"value": round(npts * k_plain / t_plain / 1e6, 3), "unit": UNIT, "steps": k_plain,
                        "ms_per_step": round(t_plain / k_plain * 1e3, 3),
                        "sim_time_per_s": (t_end - t_w) / t_plain}
    out["learned_lad"] = {"value": round(npts * k_learn / t_learn / 1e6, 3), "unit": UNIT, "steps": k_learn,
                          "ms_per_step": round(t_learn / k_learn * 1e3, 3),
                          "sim_time_per_s": (t_end - t_wl) / t_learn, "fallback_steps": lad.fallbacks}
    out["speedup_per_step"] = round((t_plain / k_plain) / (t_learn / k_learn), 3)
    out["speedup_time_to_solution"] = round(out["learned_lad"]["sim_time_per_s"] / out["plain_lad"]["sim_time_per_s"], 3)
    out["density_l1_vs_plain"] = l1
    out["note"] = ("each closure takes its own CFL/diffusion steps to the same time t_end; the learned "
                   "closure's timing includes its per-step state snapshot and fallback-flag read")
    return out


def main():
    args = parse()
    if args.mode == "peaks":
        return measure_peaks()
    if args.mode == "shock":
        return shock_throughput(args)
    if args.mode == "ensemble":
        return ensemble_throughput(args)
    if args.mode == "shock-learned":
        return shock_learned(args)
    if args.mode == "kernels":
        return kernel_sweeps(args)
    if args.mode == "lad":
        return lad_kernel(args)
    if args.impl == "reference":
        return run_reference(args)
    if args.mode == "sweeps":
        return sweeps_only(args)
    if args.mode == "profile":
        return profile_step(args)
    import torch
    world, rank, local = dist_setup()
    dist_on = world > 1
    if dist_on:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()

    # CPU baseline before any forked process could inherit a CUDA context
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, sample, _ = cpu_baseline(2, 1)
        cpu = {"value": round(v, 4), "unit": UNIT, "cores": cores, "kind": "port", "sample": sample}

    from pyranda_gb300 import _lib
    n = args.n
    npts = n ** 3
    k, w = args.steps, max(3, args.warmup)

    # ---- split-precision paths, each with one CUDA graph per RK step:
    # FP32 banded sweeps, and dense split-TF32 operators on the tensor cores
    fast_runs = {}
    runs = ([("fp32", args.fusion_arith)] if args.precision == "fp32-only" else
            [("fp32", args.fusion_arith), ("dense", args.fusion_arith), ("auto", args.fusion_arith)])
    if args.precision != "fp32-only" and not args.no_fusion:
        for other in ("fp64", "df64", "fp32"):   # the same path with the other EOM arithmetics, for comparison only
            if other != args.fusion_arith:
                runs.append(("auto", other))
    for prec, arith in runs:
        sim = make_sim(n, prec, graphs=True, fusion=not args.no_fusion, arith=arith)
        run_steps(sim, 1)             # eager step (records the fused kernels, then compiles them)
        c0 = _lib.launch_count()
        f0 = sim._fuse.fused_calls if sim._fuse is not None else 0
        run_steps(sim, 1)             # records the step's graph (counts this library's and the fused launches)
        lps = _lib.launch_count() - c0 + ((sim._fuse.fused_calls - f0) if sim._fuse is not None else 0)
        run_steps(sim, w - 2)         # capture + replays
        clocks = ClockSampler(dev)
        clocks.start()
        t = time_steps(sim, k, torch, dist_on)
        ck_ = clocks.stop()
        t = max_over_ranks(t, dist_on, "cuda")
        key = prec if arith == args.fusion_arith else "%s+%s-eom" % (prec, arith)
        fast_runs[key] = {"sim": sim, "t": t, "launches": lps, "clocks": ck_, "arith": arith, "prec": prec,
                           "plan": {"%s_%s" % k: v for k, v in sim.grid.sweep_plan().items()}}
    # the headline is the fastest path with the requested EOM arithmetic
    best = min((p for p in fast_runs if fast_runs[p]["arith"] == args.fusion_arith), key=lambda p: fast_runs[p]["t"])
    fast, t_fast = fast_runs[best]["sim"], fast_runs[best]["t"]
    best_prec, best_arith = fast_runs[best]["prec"], fast_runs[best]["arith"]
    launches_per_step, ck = fast_runs[best]["launches"], fast_runs[best]["clocks"]
    value = job_value(npts, k, world, t_fast)

    # ---- plain FP64 path, same IC, same number of steps (no graph)
    extra = {"fast_paths": {p: {"value": round(job_value(npts, k, world, r["t"]), 4), "unit": UNIT,
                                "ms_per_step": round(r["t"] / k * 1e3, 3), "dense_plan": r["plan"],
                                "eom_arith": r["arith"] if not args.no_fusion else "unfused fp64"}
                            for p, r in fast_runs.items()}}
    if not args.no_fp64:
        plain = make_sim(n, "fp64", graphs=False)
        run_steps(plain, w)
        t64 = time_steps(plain, k, torch, dist_on)
        t64 = max_over_ranks(t64, dist_on, "cuda")
        extra["fp64_plain"] = {"value": round(job_value(npts, k, world, t64), 4), "unit": UNIT,
                               "ms_per_step": round(t64 / k * 1e3, 3), "form": "eager, unfused EOM arithmetic"}
        # the plain FP64 form with its EOM arithmetic fused into generated FP64
        # kernels and the whole step in one CUDA graph (bit-identical results)
        plain_fg = make_sim(n, "fp64", graphs=True, fusion=True, arith="fp64")
        run_steps(plain_fg, w)
        t64g = max_over_ranks(time_steps(plain_fg, k, torch, dist_on), dist_on, "cuda")
        same = all(torch.equal(plain_fg.variables[nm].data, plain.variables[nm].data)
                   for nm in ("rho", "rhou", "rhov", "rhow", "Et"))
        extra["fp64_fused_graph"] = {"value": round(job_value(npts, k, world, t64g), 4), "unit": UNIT,
                                     "ms_per_step": round(t64g / k * 1e3, 3),
                                     "form": "fused FP64 EOM kernels, CUDA graph per RK step",
                                     "bit_identical_to_fp64_plain": bool(same)}
        extra["speedup"] = {"vs_fp64_plain_eager": round(t64 / t_fast, 3),
                            "vs_fp64_fused_graph": round(t64g / t_fast, 3)}
        del plain_fg
        torch.cuda.empty_cache()
        # accuracy of each fast path: every sim advanced w + k steps from the same IC
        for p, r in fast_runs.items():
            errs = l2_errors(r["sim"], plain, ["rho", "rhou", "rhov", "rhow", "Et"])
            extra["fast_paths"][p]["l2_err_vs_fp64"] = {kk: float("%.3e" % vv) for kk, vv in errs.items()}
            errs = linf_errors(r["sim"], plain, ["rho", "rhou", "rhov", "rhow", "Et"])
            extra["fast_paths"][p]["linf_err_vs_fp64"] = {kk: float("%.3e" % vv) for kk, vv in errs.items()}
            extra["fast_paths"][p]["l2_err_vs_fp64"]["momentum_vector"] = float("%.3e" % momentum_error(r["sim"], plain))
        extra["l2_err_vs_fp64"] = extra["fast_paths"][best]["l2_err_vs_fp64"]
        extra["linf_err_vs_fp64"] = extra["fast_paths"][best]["linf_err_vs_fp64"]
        extra["l2_err_steps"] = w + k
        if args.err_steps > w + k:   # the headline path and the plain one continued to the configuration's length
            more = args.err_steps - (w + k)
            run_steps(plain, more)
            run_steps(fast, more)
            errs = l2_errors(fast, plain, ["rho", "rhou", "rhov", "rhow", "Et"])
            errs = {kk: float("%.3e" % vv) for kk, vv in errs.items()}
            errs["momentum_vector"] = float("%.3e" % momentum_error(fast, plain))
            linf = {kk: float("%.3e" % vv)
                    for kk, vv in linf_errors(fast, plain, ["rho", "rhou", "rhov", "rhow", "Et"]).items()}
            extra["l2_err_vs_fp64_long"] = {"steps": args.err_steps, "path": best, "rel_l2": errs, "rel_linf": linf}
        del plain
        torch.cuda.empty_cache()

    # ---- dominant-kernel roofline (sweeps on one 256^3 field, FP32 arithmetic)
    import json as _json
    peaks = {}
    try:
        peaks = _json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    for p, r in fast_runs.items():
        if r["sim"] is not fast:
            del r["sim"]
    torch.cuda.empty_cache()
    sw = sweep_roofline(fast, torch)
    # the dominant sweep kernel: largest share of the step (launches per step x
    # CUDA-event duration per launch / step time)
    counts = sweep_counts(fast_runs[best]["prec"], fast_runs[best]["arith"], not args.no_fusion)
    cls = {"d1": "d1", "d8": "d8", "sf": "sfilter", "gf": "gfilter"}
    step_s = t_fast / k
    shares = {}
    for (op, d), c in counts.items():
        key = "%s_%s" % (cls[op], "xyz"[d])
        shares[key] = {"launches_per_step": c, "ms_per_launch": round(sw[key] * 1e3, 4),
                       "share_of_step": round(c * sw[key] / step_s, 4)}
    dom = max(shares, key=lambda kk: shares[kk]["share_of_step"])
    dom_op = {v: kk for kk, v in cls.items()}[dom.split("_")[0]]
    dom_dir = dom.split("_")[1]
    dur = sw[dom]
    achieved = 16.0 * npts / dur / 1e9
    form = fast.grid.sweep_plan()[(dom_op, dom_dir)]
    dense_dom = form == "dense"
    dirn = {"x": 0, "y": 1, "z": 2}[dom_dir]
    if dense_dom:
        kname = ("dense_kernel (tcgen05 kind::tf32, 3 products, TMEM accumulator), %s sweep along %s"
                 % (dom_op, dom_dir) + ("; after d8_rhs_kernel (exact fixed-point RHS)" if dom_op == "d8" else ""))
        # the tensor-core work of the same launch: 3 TF32 products of 2n flops per point
        roof_extra = {"tensor_tflops": round(3 * 2 * n * npts / dur / 1e12, 1),
                      "tensor_peak_note": "TF32 dense nominal ~1100 TFLOP/s (no measured TF32 peak in "
                                          "MEASURED_PEAKS.json)"}
    elif form == "split" and n % 32 == 0:
        kname = ("seg_kernel<%s, dir=%d> (FP32 split-line banded solve: 32-row segments unrolled in registers, "
                 "joined by the reduced system; %s)" % (dom_op, dirn, "tile staged through shared memory" if dirn == 0
                                                        else "lines read and written straight from global memory"))
        roof_extra = {}
    elif form == "split":
        kname = ("split_kernel<float, %s, dir=%d> (split-line banded solve: 32-point segments joined by the "
                 "reduced system, tile of lines in shared memory)" % (dom_op, dirn))
        roof_extra = {}
    else:
        kname = "sweep_kernel<float, %s, dir=%d> (FP32 banded line solve, one thread per line)" % (dom_op, dirn)
        roof_extra = {}
    tr = NCU_TRAFFIC_256.get((dom_op, dom_dir, form)) if n == 256 else None
    roof = {"bound": "hbm", "kernel": kname, "kernel_class": dom,
            "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
            "traffic": tr[0] if tr else None,
            "traffic_source": ("carried over from %s: ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                               "launch at 256^3 of the kernel build profiled there (not re-measured in this run)"
                               % tr[1]) if tr else "no ncu capture of this kernel class at this size",
            "algorithmic_bytes_per_launch": 16 * npts,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6800 GB/s",
            "selection": "largest share of the step among the sweep kernel classes",
            "kernel_shares": shares,
            "sweep_ms": {kk: round(vv * 1e3, 4) for kk, vv in sw.items()}}
    roof.update(roof_extra)

    # ---- end to end: host state in pinned memory, copied in and out every step
    names = fast.conserved
    host = {nm: torch.empty((n, n, n), dtype=torch.float64).pin_memory() for nm in names}
    for nm in names:
        host[nm].copy_(fast.variables[nm].data.permute(2, 1, 0))
    torch.cuda.synchronize()
    # one copy stream per field, so the fields' copies run on the copy engines side by side: a field's
    # copy-in waits for its previous copy-out (same host buffer), the step waits for every copy-in,
    # and the copy-outs wait for the step
    comp = torch.cuda.current_stream()
    cstreams = {nm: torch.cuda.Stream() for nm in names}
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for nm in names:
        cstreams[nm].wait_stream(comp)
    for _ in range(k):
        for nm in names:
            with torch.cuda.stream(cstreams[nm]):
                fast.variables[nm].data.permute(2, 1, 0).copy_(host[nm], non_blocking=True)
            comp.wait_stream(cstreams[nm])
        run_steps(fast, 1)
        for nm in names:
            cstreams[nm].wait_stream(comp)
            with torch.cuda.stream(cstreams[nm]):
                host[nm].copy_(fast.variables[nm].data.permute(2, 1, 0), non_blocking=True)
    for nm in names:
        comp.wait_stream(cstreams[nm])
    e.record()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(s.elapsed_time(e) / 1e3, dist_on, "cuda")
    nbytes = len(names) * npts * 8
    e2e_line = {"value": round(job_value(npts, k, world, t_e2e), 4), "unit": UNIT,
                "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes}
    final_dense_plan = fast_runs[best]["plan"]
    uses_dense = best_prec == "dense" or (best_prec == "auto" and "dense" in fast.grid.sweep_plan().values())
    del fast, fast_runs
    torch.cuda.empty_cache()

    # ---- short sub-lines of the other configurations, measured in the same run
    if not args.no_subconfigs and world == 1:
        ns = argparse.Namespace(members=64, steps=args.sub_steps, warmup=3, reps=5, fusion_arith=args.fusion_arith)
        try:
            extra["subconfig_ensemble_kh64"] = ensemble_result(ns, one_at_a_time=False)
        except Exception as ex:  # reported, never hides the headline
            extra["subconfig_ensemble_kh64"] = {"error": repr(ex)[:300]}
        torch.cuda.empty_cache()
        ns = argparse.Namespace(model=None, steps=args.sub_steps, warmup=3, reps=5, fusion_arith=args.fusion_arith)
        try:
            extra["subconfig_learned_lad_shock"] = shock_learned_result(ns, train_if_missing=False)
        except Exception as ex:
            extra["subconfig_learned_lad_shock"] = {"error": repr(ex)[:300]}
        torch.cuda.empty_cache()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": world, "steps": k, "warmup": w,
            "ms_per_step": round(t_fast / k * 1e3, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": ("tf32x3 (f32 accumulate) / f32 sweeps, f64 state" if uses_dense
                                           else "f32 sweeps (RHS differences from f32 hi + lo pairs), f64 state"),
            "data": "synthetic (Taylor-Green initial condition, Mach 0.1)",
            "config": {"workload": "compressible Taylor-Green vortex %d^3 periodic, Mach 0.1, Re 1600, LAD + compact filters, "
                                   "LSRK(5,4), CFL 0.5" % n,
                       "grid": [n, n, n],
                       "path": {"dense": "dense split-TF32 tensor-core operators (d1, compact and Gaussian "
                                         "filters), d8 as A^-1 on its exact fixed-point RHS",
                                "auto": "per operator and direction the fastest of dense split-TF32, FP32 banded "
                                        "(one thread per line) and FP32 split-line banded (autotuned on the grid)",
                                "fp32": "fp32 banded sweeps"}[best_prec]
                               + ", FP64 state, fused EOM arithmetic in %s, CUDA graph per RK step"
                               % best_arith.upper(),
                       "sweep_plan": final_dense_plan,
                       "l2": "inputs larger than L2 (~40 fields of %d MiB)" % (npts * 8 >> 20),
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": roof,
            "cpu_baseline": cpu,
            "e2e": e2e_line,
            "gpu_launches": int(launches_per_step * k),
            "clocks": ck,
        }
        line.update(extra)
        print(json.dumps(line), flush=True)
    if dist_on:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
