"""Fused EOM arithmetic reproduces the unfused steps bit for bit.

The fused kernels round every operation as torch does, so fields after
several RK steps must be identical with and without fusion, eagerly and
with the step recorded in a CUDA graph, for the Taylor-Green, Kelvin-Helmholtz
(walls, 2-D) and shock (one-sided x, LAD + conductivity) problems.
"""
import numpy
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _packs(ss):
    from pyranda_gb300 import pyrandaBC, pyrandaTimestep
    ss.addPackage(pyrandaTimestep(ss))
    ss.addPackage(pyrandaBC(ss))


def _build(kind, precision):
    from pyranda_gb300 import problems, pyrandaSim
    if kind == "tgv":
        return problems.build_tgv(pyrandaSim, 32, lambda s: _packs(s), silent=True, precision=precision)
    if kind == "kh":
        return problems.build_kh(pyrandaSim, 48, _packs, silent=True, precision=precision)
    return problems.build_shock(pyrandaSim, 64, 16, 16, _packs, silent=True, precision=precision)


def _run(ss, steps):
    t = 0.0
    for _ in range(steps):
        t = ss.rk4(t, ss.variables["dt"].data.clone())
    return ss


@pytest.mark.parametrize("kind", ["tgv", "kh", "shock"])
@pytest.mark.parametrize("graphs", [False, True])
def test_fused_equals_unfused(kind, graphs):
    a = _build(kind, "fp32")
    b = _build(kind, "fp32")
    b.use_fusion(True)
    if graphs:
        b.use_graphs(True)
    _run(a, 4)
    _run(b, 4)
    assert b._fuse is not None and b._fuse.lib is not None
    assert b._fuse.fused_calls > 0 or graphs
    for name, v in a.variables.items():
        x, y = v.data, b.variables[name].data
        if isinstance(x, torch.Tensor):
            assert torch.equal(x, y), (kind, name, float((x - y).abs().max()))


@pytest.mark.parametrize("kind", ["tgv", "kh", "shock"])
def test_fp32_arithmetic_stays_close_to_unfused(kind):
    """FP32 EOM arithmetic between FP64 fields.

    Every line then carries FP32 rounding (2**-24 relative), which the
    derivatives of large-mean fluxes (pressure) amplify: after 4 steps the
    conserved fields stay within 1e-5 relative L2 of the FP64-arithmetic run
    (momentum components measured against the momentum vector's norm, since a
    component may start at zero).
    """
    a = _build(kind, "fp32")
    b = _build(kind, "fp32")
    b.use_fusion(True, arithmetic="fp32")
    b.use_graphs(True)
    _run(a, 4)
    _run(b, 4)
    assert b._fuse is not None and b._fuse.arith == "fp32" and b._fuse.lib is not None
    mom = [n for n in ("rhou", "rhov", "rhow") if n in b.conserved]
    mnorm = sum(float(torch.linalg.vector_norm(a.variables[n].data)) ** 2 for n in mom) ** 0.5
    for name in b.conserved:
        x, y = a.variables[name].data, b.variables[name].data
        assert torch.isfinite(y).all(), (kind, name)
        ref = mnorm if name in mom else float(torch.linalg.vector_norm(x))
        err = float(torch.linalg.vector_norm(x - y)) / max(ref, 1e-300)
        assert err <= 1e-5, (kind, name, err)


@pytest.mark.parametrize("kind", ["tgv", "kh", "shock"])
def test_df64_arithmetic_stays_close_to_fp64(kind):
    """Double-float EOM arithmetic (FP32 hi + lo pairs, ~48 bits): after 4
    steps the conserved fields stay within 1e-6 relative L2 of the
    FP64-arithmetic run (momentum components against the momentum norm),
    10x inside the FP32 arithmetic's bar.  The operations themselves agree
    with FP64 to 2e-13 (test_df64_operations_against_fp64); what reaches the
    fields is the LAD bulk viscosity beta = gbar(|ring(div)| rho): where the
    dilatation div = ux + vy + wz cancels (the Taylor-Green flow, the smooth
    regions of the shock problem) it is rounding noise, and ring takes its 8th
    derivative, so 48-bit and 53-bit arithmetic give different noise; the
    shear viscosity mu = gbar(|ring(S)|) rho of the Taylor-Green flow likewise.
    (Measured: TGV 32^3 rhou 2.6e-7, shock 4.6e-8, KH 1.6e-14.)"""
    a = _build(kind, "fp32")
    b = _build(kind, "fp32")
    b.use_fusion(True, arithmetic="df64")
    b.use_graphs(True)
    _run(a, 4)
    _run(b, 4)
    assert b._fuse is not None and b._fuse.arith == "df64" and b._fuse.lib is not None
    mom = [n for n in ("rhou", "rhov", "rhow") if n in b.conserved]
    mnorm = sum(float(torch.linalg.vector_norm(a.variables[n].data)) ** 2 for n in mom) ** 0.5
    for name in b.conserved:
        x, y = a.variables[name].data, b.variables[name].data
        assert torch.isfinite(y).all(), (kind, name)
        ref = mnorm if name in mom else float(torch.linalg.vector_norm(x))
        err = float(torch.linalg.vector_norm(x - y)) / max(ref, 1e-300)
        print(kind, name, "df64 vs fp64 EOM arithmetic: %.2e" % err)
        assert err <= 1e-6, (kind, name, err)


def test_df64_operations_against_fp64():
    """Each double-float operation on random operands (signs and magnitudes
    from 1e-3 to 1e3) against the FP64 result: relative error <= 2e-13
    (add / subtract relative to the larger operand)."""
    import ctypes
    from pyranda_gb300 import fuse
    src = fuse.PRELUDE_DF64 + r"""
extern "C" __global__ void ops(int64_t n, const double* a, const double* b, double* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const real x = PG_LOAD(a[i]), y = PG_LOAD(b[i]);
    out[7 * i + 0] = PG_STORE(x);
    out[7 * i + 1] = PG_STORE(PG_ADD(x, y));
    out[7 * i + 2] = PG_STORE(PG_SUB(x, y));
    out[7 * i + 3] = PG_STORE(PG_MUL(x, y));
    out[7 * i + 4] = PG_STORE(PG_DIV(x, y));
    out[7 * i + 5] = PG_STORE(PG_SQRT(PG_ABS(x)));
    out[7 * i + 6] = PG_STORE(pg_max(x, (-y)));
  }
}
extern "C" int ops_launch(int64_t n, const double* a, const double* b, double* out, void* stream) {
  ops<<<64, 256, 0, (cudaStream_t)stream>>>(n, a, b, out);
  return (int)cudaGetLastError();
}
"""
    lib = ctypes.CDLL(fuse.compile_source(src, fmad=True))
    r = numpy.random.default_rng(3)
    n = 100000
    a = r.choice([-1.0, 1.0], n) * 10.0 ** r.uniform(-3, 3, n)
    b = r.choice([-1.0, 1.0], n) * 10.0 ** r.uniform(-3, 3, n)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    out = torch.empty(7 * n, dtype=torch.float64, device="cuda")
    assert lib.ops_launch(ctypes.c_int64(n), ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()),
                          ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(0)) == 0
    o = out.cpu().numpy().reshape(n, 7)
    big = numpy.maximum(numpy.abs(a), numpy.abs(b))
    checks = [(o[:, 0], a, numpy.abs(a)), (o[:, 1], a + b, big), (o[:, 2], a - b, big), (o[:, 3], a * b, numpy.abs(a * b)),
              (o[:, 4], a / b, numpy.abs(a / b)), (o[:, 5], numpy.sqrt(numpy.abs(a)), numpy.sqrt(numpy.abs(a))),
              (o[:, 6], numpy.maximum(a, -b), big)]
    for k, (got, want, scale) in enumerate(checks):
        err = float(numpy.max(numpy.abs(got - want) / scale))
        assert err <= 2e-13, (k, err)


def test_fp32_load_and_store_conversions():
    """The integer FP64<->FP32 conversions of the FP32 kernels: nearest-even rounding, inf/NaN kept,
    magnitudes below 2**-126 flushed to zero, FP32 -> FP64 exact."""
    import ctypes
    from pyranda_gb300 import fuse
    src = fuse.PRELUDE_FP32 + r"""
extern "C" __global__ void conv(int64_t n, const double* in, float* f, double* back) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    f[i] = pg_d2f(in[i]);
    back[i] = pg_f2d(f[i]);
  }
}
extern "C" int conv_launch(int64_t n, const double* in, float* f, double* back, void* stream) {
  conv<<<64, 256, 0, (cudaStream_t)stream>>>(n, in, f, back);
  return (int)cudaGetLastError();
}
"""
    lib = ctypes.CDLL(fuse.compile_source(src, fmad=True))
    g = torch.Generator().manual_seed(3)
    vals = torch.cat([
        torch.randn(20000, generator=g, dtype=torch.float64) * torch.exp2(torch.randint(-140, 130, (20000,), generator=g).double()),
        torch.tensor([0.0, -0.0, 1.0, -1.0, 2.0 ** -126, 2.0 ** -127, -(2.0 ** -130), 3.4028234663852886e38,
                      3.4028235677973366e38, 1e39, -1e300, float("inf"), float("-inf"), float("nan"),
                      1.0 + 2.0 ** -24, 1.0 + 3 * 2.0 ** -24, 1.0 + 2.0 ** -24 + 2.0 ** -50], dtype=torch.float64)])
    x = vals.cuda()
    f = torch.empty(x.numel(), dtype=torch.float32, device="cuda")
    back = torch.empty_like(x)
    assert lib.conv_launch(ctypes.c_int64(x.numel()), ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(f.data_ptr()),
                           ctypes.c_void_p(back.data_ptr()), ctypes.c_void_p(0)) == 0
    torch.cuda.synchronize()
    want = vals.float()                       # round to nearest even, denormals kept
    tiny = vals.abs() < 2.0 ** -126
    want = torch.where(tiny, torch.zeros_like(want).copysign(want), want)
    got = f.cpu()
    nan = torch.isnan(vals)
    assert torch.isnan(got[nan]).all()
    assert torch.equal(got[~nan].view(torch.int32), want[~nan].view(torch.int32))
    assert torch.equal(back.cpu()[~nan], got[~nan].double())
    assert torch.isnan(back.cpu()[nan]).all()
