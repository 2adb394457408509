"""Fused EOM arithmetic reproduces the unfused steps bit for bit.

The fused kernels round every operation as torch does, so fields after
several RK steps must be identical with and without fusion, eagerly and
with the step recorded in a CUDA graph, for the Taylor-Green, Kelvin-Helmholtz
(walls, 2-D) and shock (one-sided x, LAD + conductivity) problems.
"""
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
