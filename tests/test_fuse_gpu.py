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
