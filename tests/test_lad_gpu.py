"""Learned LAD closure kernels against the oracle, and what training buys.

* pg_lad_train_step's gradient equals the oracle's (oracle/lad_mlp.py) on
  the same BF16 parameters and inputs to relative L2 <= 2e-3 (FP32 against
  FP64 accumulation; a hidden activation can land on the other side of a
  BF16 rounding boundary);
* pg_lad_closure's outputs equal the oracle forward on the oracle's own
  27-point feature gather: differences <= 1e-4 (median) and 1e-2 (99th
  percentile) of the field's scale;
* Adam on the FP32 master weights matches the textbook update;
* training reduces the loss; out-of-range predictions raise the fallback
  flag and the step is re-run with the plain closure;
* on a held-out shock state the trained network's beta and kappa are much
  closer to the plain operators' than the untrained network's, and a run
  with the trained closure stays close to the plain run while the run
  without a closure does not survive.
"""
import ctypes

import numpy
import pytest

from tests.helpers import to_dev, to_host

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _model(seed=0):
    from pyranda_gb300.learned_lad import LadModel
    return LadModel("cuda", seed=seed)


def test_train_step_gradient_matches_oracle():
    from oracle import lad_mlp as L
    from pyranda_gb300.learned_lad import Trainer
    m = _model(1)
    r = numpy.random.default_rng(5)
    X = torch.from_numpy(r.standard_normal((300, L.NK)).astype(numpy.float32)).cuda().to(torch.bfloat16)
    T = torch.from_numpy(r.standard_normal((300, 2)).astype(numpy.float32)).cuda()
    tr = Trainer(m)
    loss = float(tr.gradient(X, T).item())
    lo, go = L.loss_and_grad(m.params.cpu().numpy(), X.float().cpu().numpy(), T.cpu().numpy())
    g = tr.grad.cpu().numpy().astype(numpy.float64)
    assert abs(loss - lo) <= 1e-4 * abs(lo)
    assert numpy.linalg.norm(g - go) <= 2e-3 * numpy.linalg.norm(go)
    for name, (o, n) in L.OFF.items():
        assert numpy.linalg.norm(g[o:o + n] - go[o:o + n]) <= 5e-3 * max(numpy.linalg.norm(go[o:o + n]), 1e-12), name


def test_closure_inference_matches_oracle():
    from oracle import lad_mlp as L
    from pyranda_gb300.grid import Grid
    from pyranda_gb300.learned_lad import fit_normalisation
    n, per = (24, 20, 12), (True, False, True)
    g = Grid(n, per, (0, 0, 0), (1.0, 1.0, 0.5), precision="fp64")
    r = numpy.random.default_rng(7)
    div = numpy.asfortranarray(r.standard_normal(n))
    gm = numpy.asfortranarray(numpy.abs(r.standard_normal(n)))
    rho = numpy.asfortranarray(1.0 + r.random(n))
    m = _model(2)
    delta = max(g.mesh_d)
    raw = L.features(div, gm, per, delta)
    fit_normalisation(m, torch.from_numpy(raw.astype(numpy.float32)).cuda(),
                      torch.from_numpy(r.random((raw.shape[0], 2)).astype(numpy.float32)).cuda())
    dt = torch.full((), 2e-3, dtype=torch.float64, device="cuda")
    beta, kappa, flag = g.empty(), g.empty(), torch.zeros(1, dtype=torch.int32, device="cuda")
    mm = m.struct()
    d, gg, rr = to_dev(div, torch), to_dev(gm, torch), to_dev(rho, torch)
    from pyranda_gb300.grid import _ptr, _stream
    rc = g.lib.pg_lad_closure(g.h, ctypes.byref(mm), _ptr(d), _ptr(gg), _ptr(rr), _ptr(dt), 2.5, _ptr(beta),
                              _ptr(kappa), _ptr(flag), _stream())
    assert rc == 0
    Xn = (raw - m.xmean.cpu().numpy()) * m.xinvstd.cpu().numpy()
    y, _ = L.forward(m.params.cpu().numpy(), Xn)
    rf = rho.ravel(order="F")
    b_ref = numpy.maximum(0.0, y[:, 0] * m.ys[0] + m.ym[0]) * rf * delta
    k_ref = numpy.maximum(0.0, y[:, 1] * m.ys[1] + m.ym[1]) * rf * 2.5 * delta ** 2 / 2e-3
    b = to_host(beta).ravel(order="F")
    k = to_host(kappa).ravel(order="F")
    # relative to the field's scale: clamped points are zero in both
    rb = numpy.abs(b - b_ref) / max(numpy.abs(b_ref).max(), 1e-300)
    rk = numpy.abs(k - k_ref) / max(numpy.abs(k_ref).max(), 1e-300)
    assert numpy.median(rb) < 1e-4 and numpy.median(rk) < 1e-4
    assert numpy.quantile(rb, 0.99) < 1e-2 and numpy.quantile(rk, 0.99) < 1e-2


def test_adam_matches_textbook_update():
    from pyranda_gb300.learned_lad import NP, NW, Trainer
    m = _model(3)
    tr = Trainer(m, lr=1e-2)
    p0 = m.params.clone()
    g = torch.randn(NP, device="cuda", dtype=torch.float32)
    tr.grad.copy_(g)
    tr.t = 1
    from pyranda_gb300.grid import _ptr, _stream
    rc = tr.lib.pg_lad_adam(_ptr(m.params), _ptr(tr.m), _ptr(tr.v), _ptr(tr.grad), NP, 1e-2, 0.9, 0.999, 1e-8, 1,
                            _ptr(m.wbf16), NW, _stream())
    assert rc == 0
    mh = (0.1 * g) / (1 - 0.9)
    vh = (0.001 * g * g) / (1 - 0.999)
    ref = p0 - 1e-2 * mh / (torch.sqrt(vh) + 1e-8)
    assert float((m.params - ref).abs().max()) < 1e-6
    assert torch.equal(m.wbf16, m.params[:NW].to(torch.bfloat16))


def test_training_reduces_loss():
    from pyranda_gb300.learned_lad import fit_normalisation, normalize, train
    r = numpy.random.default_rng(9)
    raw = torch.from_numpy(r.standard_normal((20000, 64)).astype(numpy.float32)).cuda()
    raw[:, 55:] = 0
    T = torch.stack([torch.relu(raw[:, 13]) + 0.5 * raw[:, 40], torch.tanh(raw[:, 5] - raw[:, 30])], 1)
    m = _model(4)
    Tn = fit_normalisation(m, raw, T)
    X = normalize(raw, m)
    hist = train(m, X, Tn, iters=400, batch=4096, lr=3e-3, log_every=50)
    assert hist[-1] < 0.2 * hist[0], hist


def _packs(ss):
    from pyranda_gb300 import pyrandaBC, pyrandaTimestep
    ss.addPackage(pyrandaBC(ss))
    ss.addPackage(pyrandaTimestep(ss))


def _shock(eom, mode, model, shape=(64, 32, 32), mach=1.8, amp=0.05):
    from pyranda_gb300 import problems, pyrandaSim
    from pyranda_gb300.learned_lad import pyrandaLearnedLAD

    def packs(ss):
        _packs(ss)
        ss.addPackage(pyrandaLearnedLAD(ss, model, problems.CV, mode=mode))

    return problems.build_shock(pyrandaSim, *shape, packs, mach=mach, amp=amp, eom=eom, silent=True,
                                precision="fp64")


@pytest.mark.parametrize("graphs", [False, True])
def test_fallback_flag_reruns_the_step_with_the_plain_closure(graphs):
    from pyranda_gb300.learned_lad import learned_shock_eom
    m = _model(5)
    m.ylo, m.yhi = [1e9, 1e9], [2e9, 2e9]   # every prediction is out of range
    # both start from the plain closure's initial state; a then predicts
    a = _shock(learned_shock_eom(), "plain", m)
    b = _shock(learned_shock_eom(), "plain", m)
    lad = a.packages["LAD"]
    lad.mode = "learned"
    if graphs:
        a.use_graphs(True)
    ta, tb = 0.0, 0.0
    for _ in range(3):
        dt = b.variables["dt"].data.clone()
        ta = lad.step(ta, dt)
        tb = b.rk4(tb, dt)
    assert lad.fallbacks == 3
    for name in ("rho", "rhou", "Et", "beta", "kappa"):
        assert torch.equal(a.variables[name].data, b.variables[name].data), name


@pytest.mark.slow
def test_trained_closure_beats_untrained_and_none():
    """Train on snapshots of small seeded runs; evaluate on an unseen state and an unseen run.

    * On a held-out plain-LAD state (Mach and amplitude outside the training
      seeds' draws), the trained network's beta and kappa are much closer to
      the plain operators' than the same network untrained.
    * A run with the trained closure stays finite and close to the plain run
      (density L1), while the run without a closure does not survive.
    """
    from pyranda_gb300.learned_lad import (fit_normalisation, learned_shock_eom, normalize, shock_training_set,
                                           train)
    raw, T, _ = shock_training_set(runs=4, snapshots_per_run=25, shape=(64, 32, 32), points=4096, seed=1,
                                   precision="fp64")
    m = _model(6)
    Tn = fit_normalisation(m, raw, T)
    X = normalize(raw, m)
    train(m, X, Tn, iters=1500, batch=8192, lr=2e-3)
    untrained = _model(7)
    untrained.xmean.copy_(m.xmean)
    untrained.xinvstd.copy_(m.xinvstd)
    untrained.ym, untrained.ys = m.ym, m.ys
    # a held-out state: the plain closure's beta and kappa against each network's
    ss = _shock(learned_shock_eom(), "plain", m, mach=2.2, amp=0.07)
    t = 0.0
    for _ in range(30):
        t = float(ss.rk4(t, ss.variables["dt"].data))
    V = ss.variables
    lad = ss.packages["LAD"]
    args = (V["div"].data, V["rho"].data, V["T"].data, V["dt"].data)
    ref_b, ref_k = lad.closure(*args)
    errs = {}
    for name, model in (("trained", m), ("untrained", untrained)):
        lad.model, lad._m, lad.mode = model, model.struct(), "learned"
        b, k = lad.closure(*args)
        errs[name] = (float((b - ref_b).norm() / ref_b.norm()), float((k - ref_k).norm() / ref_k.norm()))
    print("closure relative L2 error (beta, kappa):", errs)
    assert errs["trained"][0] < 0.5 * errs["untrained"][0], errs
    assert errs["trained"][1] < 0.5 * errs["untrained"][1], errs
    # whole runs to the same time, each with its own CFL / diffusion steps
    t_end = 0.35
    runs = {}
    for name, mode in (("plain", "plain"), ("learned", "learned"), ("off", "off")):
        ss = _shock(learned_shock_eom(), "plain", m, mach=2.2, amp=0.07)
        ss.packages["LAD"].mode = mode
        t, n = 0.0, 0
        while t < t_end - 1e-12 and n < 2000:
            dt = min(float(ss.variables["dt"].data), t_end - t)
            t = float(ss.rk4(t, dt))
            n += 1
            if not bool(torch.isfinite(ss.variables["rho"].data).all()):
                break
        runs[name] = ss.variables["rho"].data
    ref = runs["plain"]
    err = {k: float((v - ref).abs().sum() / ref.abs().sum()) if bool(torch.isfinite(v).all()) else float("inf")
           for k, v in runs.items() if k != "plain"}
    print("density L1 error vs plain LAD:", err)
    assert err["learned"] < 0.05, err               # the learned run stays close to the plain one
    assert err["learned"] < err["off"], err         # while no closure at all does not survive


@pytest.mark.parametrize("per", [(True, False, True), (False, True, False)], ids=["PNP", "NPN"])
def test_grad_magnitude_matches_oracle(per):
    from oracle import lad_mlp as L
    from pyranda_gb300.grid import Grid
    from pyranda_gb300.learned_lad import grad_magnitude
    n = (24, 20, 12)
    g = Grid(n, per, (0, 0, 0), (1.0, 2.0, 0.5), precision="fp64")
    r = numpy.random.default_rng(11)
    rho = numpy.asfortranarray(1.0 + r.random(n))
    got = to_host(grad_magnitude(g, to_dev(rho, torch)))
    want = L.grad_magnitude(rho, per, g.mesh_d)
    assert numpy.abs(got - want).max() <= 1e-6 * numpy.abs(want).max()
    flat = Grid((16, 1, 8), (True, False, True), (0, 0, 0), (1.0, 1.0, 1.0), precision="fp64")
    f = numpy.asfortranarray(1.0 + r.random((16, 1, 8)))
    got = to_host(grad_magnitude(flat, to_dev(f, torch)))
    assert numpy.abs(got - L.grad_magnitude(f, (True, False, True), flat.mesh_d)).max() <= 1e-6 * got.max()
