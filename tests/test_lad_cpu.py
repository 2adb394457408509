"""The learned-closure oracle's gradient against finite differences (CPU).

The oracle (oracle/lad_mlp.py) is what the GPU training kernel's gradients
are checked against, so its own backward pass is pinned here: without BF16
rounding the network is piecewise linear, and central differences of the
loss reproduce the analytic gradient to ~1e-7 relative.
"""
import numpy

from oracle import lad_mlp as L


def test_oracle_gradient_matches_finite_differences():
    rng = numpy.random.default_rng(3)
    p = rng.standard_normal(L.NP) * 0.2
    X = rng.standard_normal((40, L.NK))
    T = rng.standard_normal((40, L.NOUT))
    loss, g = L.loss_and_grad(p, X, T, rounding=False)
    idx = numpy.concatenate([rng.choice(L.NW, 40, replace=False), numpy.arange(L.NW, L.NP)[::7]])
    h = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += h
        lp, _ = L.loss_and_grad(q, X, T, rounding=False)
        q[i] -= 2 * h
        lm, _ = L.loss_and_grad(q, X, T, rounding=False)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    x = numpy.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -2.5, 0.0], dtype=numpy.float32)
    r = L.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 * 2.0 ** -7 and r[3] == -2.5 and r[4] == 0.0


def test_feature_layout():
    div = numpy.arange(24, dtype=float).reshape(4, 3, 2, order="F")
    gm = -div
    F = L.features(div, gm, (True, False, True), 0.5)
    assert F.shape == (24, L.NK)
    # centre of the stencil (s = 13) is the point itself
    assert numpy.allclose(F[:, 13], div.ravel(order="F") * 0.5)
    assert numpy.allclose(F[:, 27 + 13], gm.ravel(order="F") * 0.5)
    assert numpy.all(F[:, L.NIN - 1] == 0.5) and numpy.all(F[:, L.NIN:] == 0)
