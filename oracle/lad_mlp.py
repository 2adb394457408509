"""Test infrastructure: numpy restatement of the learned LAD closure network.

CPU oracle for pyranda_gb300's pg_lad_* kernels (pg_lad.cu); only the tests
use it.  It restates, in FP64 with BF16 rounding at the kernels' rounding
points (inputs, weights, hidden activations), the network
  64 -> 64 -> 64 -> 64 -> 2 (ReLU hidden), parameters in the PG_LAD_NPARAM
  layout [w1 | w2 | w3 | w4 | b1 | b2 | b3 | b4] (weight rows = output unit),
its mean-squared-error loss over rows x outputs and the gradient of that loss
with respect to every parameter, and the 27-point feature gather:
  features of point (i, j, k) = f32(div)*f32(D) (an FP32 product) at the 27
  neighbours (di, dj, dk in
  {-1, 0, 1}, index s = (di+1) + 3 (dj+1) + 9 (dk+1)), then |grad rho|*D at
  the same neighbours, then D (the largest mesh spacing), then zeros up to
  64; periodic directions wrap,
  one-sided directions clamp, a direction of one point repeats the point.
The reference has no learned closure; parity here is between the CUDA
kernels and this restatement of their stated arithmetic, plus a
finite-difference check of the restated gradient.
"""
import numpy

NK, NH, NOUT, NIN = 64, 64, 2, 55
NW = 3 * NH * NH + NOUT * NH
NP = NW + 3 * NH + NOUT
OFF = {"w1": (0, NH * NK), "w2": (NH * NK, NH * NH), "w3": (NH * NK + NH * NH, NH * NH),
       "w4": (NH * NK + 2 * NH * NH, NOUT * NH), "b1": (NW, NH), "b2": (NW + NH, NH), "b3": (NW + 2 * NH, NH),
       "b4": (NW + 3 * NH, NOUT)}


def bf16(x):
    """Round to BF16 (nearest, ties to even), returned as float64."""
    a = numpy.asarray(x, dtype=numpy.float32)
    u = a.view(numpy.uint32).astype(numpy.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(numpy.uint32).view(numpy.float32).astype(numpy.float64)


def unpack(params, round_weights=True):
    """Weights (BF16-rounded FP32 values, or the exact FP64 values) and FP32 biases."""
    p = numpy.asarray(params, dtype=numpy.float64)
    W = {}
    for name, shape in (("w1", (NH, NK)), ("w2", (NH, NH)), ("w3", (NH, NH)), ("w4", (NOUT, NH))):
        o, n = OFF[name]
        w = bf16(p[o:o + n].astype(numpy.float32)) if round_weights else p[o:o + n]
        W[name] = w.reshape(shape)
    for name in ("b1", "b2", "b3", "b4"):
        o, n = OFF[name]
        W[name] = p[o:o + n].astype(numpy.float32).astype(numpy.float64) if round_weights else p[o:o + n]
    return W


def forward(params, X, rounding=True):
    """Outputs [rows, 2] and the hidden activations."""
    W = unpack(params, rounding)
    r = bf16 if rounding else (lambda v: v)
    x = r(X)
    h1 = r(numpy.maximum(x @ W["w1"].T + W["b1"], 0.0))
    h2 = r(numpy.maximum(h1 @ W["w2"].T + W["b2"], 0.0))
    h3 = r(numpy.maximum(h2 @ W["w3"].T + W["b3"], 0.0))
    y = h3 @ W["w4"].T + W["b4"]
    return y, (x, h1, h2, h3)


def loss_and_grad(params, X, T, rounding=True):
    """mean((y - T)^2) over rows x outputs, and its gradient in the parameter layout."""
    W = unpack(params, rounding)
    y, (x, h1, h2, h3) = forward(params, X, rounding)
    T = numpy.asarray(T, dtype=numpy.float64)
    n = y.size
    e = y - T
    loss = float((e * e).sum() / n)
    dy = 2.0 * e / n
    g = numpy.zeros(NP)

    def put(name, v):
        o, m = OFF[name]
        g[o:o + m] = numpy.asarray(v).ravel()

    put("w4", dy.T @ h3)
    put("b4", dy.sum(axis=0))
    d3 = (dy @ W["w4"]) * (h3 > 0)
    put("w3", d3.T @ h2)
    put("b3", d3.sum(axis=0))
    d2 = (d3 @ W["w3"]) * (h2 > 0)
    put("w2", d2.T @ h1)
    put("b2", d2.sum(axis=0))
    d1 = (d2 @ W["w2"]) * (h1 > 0)
    put("w1", d1.T @ x)
    put("b1", d1.sum(axis=0))
    return loss, g


def grad_magnitude(rho, periodic, d):
    """|grad rho| of pg_lad_grad_magnitude: FP32 central differences (f32(rho_hi) - f32(rho_lo)) * s with
    s = f32(1/d) / 2 (one-sided ends of non-periodic lines: f32(1/d), neighbour clamped), squares summed
    over x, y, z, FP32 sqrt; F-ordered (nx, ny, nz) FP64 in and out."""
    r = numpy.asarray(rho, dtype=numpy.float64).astype(numpy.float32)
    g2 = numpy.zeros(r.shape, dtype=numpy.float64)
    for ax in range(3):
        n = r.shape[ax]
        if n == 1:
            continue
        i = numpy.arange(n)
        if periodic[ax]:
            lo, hi = (i - 1) % n, (i + 1) % n
            sc = numpy.full(n, numpy.float32(numpy.float32(1.0 / d[ax]) * numpy.float32(0.5)), dtype=numpy.float32)
        else:
            lo, hi = numpy.maximum(i - 1, 0), numpy.minimum(i + 1, n - 1)
            sc = numpy.where((i == 0) | (i == n - 1), numpy.float32(1.0 / d[ax]),
                             numpy.float32(numpy.float32(1.0 / d[ax]) * numpy.float32(0.5))).astype(numpy.float32)
        shape = [1, 1, 1]
        shape[ax] = n
        dd = (numpy.take(r, hi, axis=ax) - numpy.take(r, lo, axis=ax)) * sc.reshape(shape)
        dd = dd.astype(numpy.float32).astype(numpy.float64)
        g2 = (dd * dd + g2).astype(numpy.float32).astype(numpy.float64)   # fma, then FP32 rounding
    return numpy.sqrt(g2.astype(numpy.float32)).astype(numpy.float64)


def features(div, gmag, periodic, delta):
    """Raw feature rows [npts, 64] of F-ordered (nx, ny, nz) fields, point order i + nx (j + ny k)."""
    div = numpy.asarray(div, dtype=numpy.float64)
    gmag = numpy.asarray(gmag, dtype=numpy.float64)
    nx, ny, nz = div.shape
    ii, jj, kk = numpy.meshgrid(numpy.arange(nx), numpy.arange(ny), numpy.arange(nz), indexing="ij")

    def idx(a, d, n, per):
        if n == 1:
            return numpy.zeros_like(a)
        b = a + d
        return b % n if per else numpy.clip(b, 0, n - 1)

    out = numpy.zeros((nx * ny * nz, NK))
    cols = []
    for s in range(27):
        di, dj, dk = s % 3 - 1, (s // 3) % 3 - 1, s // 9 - 1
        cols.append((idx(ii, di, nx, periodic[0]), idx(jj, dj, ny, periodic[1]), idx(kk, dk, nz, periodic[2])))
    d32 = numpy.float32(delta)
    for s, (a, b, c) in enumerate(cols):
        out[:, s] = (div[a, b, c].astype(numpy.float32) * d32).ravel(order="F")
        out[:, 27 + s] = (gmag[a, b, c].astype(numpy.float32) * d32).ravel(order="F")
    out[:, NIN - 1] = d32
    return out.astype(numpy.float32).astype(numpy.float64)
