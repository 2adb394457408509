"""Shared helpers of the test-suite: seeded fields, layout conversion, error norms."""
import numpy


def rng(seed=0):
    return numpy.random.default_rng(seed)


def smooth_field(shape, seed=0):
    """A seeded field with broadband content plus a smooth part, F-ordered."""
    r = rng(seed)
    nx, ny, nz = shape
    x = numpy.arange(nx)[:, None, None] / max(nx, 1)
    y = numpy.arange(ny)[None, :, None] / max(ny, 1)
    z = numpy.arange(nz)[None, None, :] / max(nz, 1)
    f = numpy.sin(2 * numpy.pi * x) * numpy.cos(4 * numpy.pi * y) + 0.5 * numpy.cos(2 * numpy.pi * z)
    f = f + 0.3 * r.standard_normal(shape)
    return numpy.asfortranarray(f)


def to_dev(a, torch):
    a = numpy.asfortranarray(numpy.asarray(a, dtype=numpy.float64))
    return torch.from_numpy(numpy.ascontiguousarray(a.transpose(2, 1, 0))).cuda().permute(2, 1, 0)


def to_host(t):
    return numpy.asfortranarray(t.permute(2, 1, 0).cpu().numpy().transpose(2, 1, 0))


def rel_l2(a, b):
    a = numpy.asarray(a, dtype=numpy.float64)
    b = numpy.asarray(b, dtype=numpy.float64)
    nb = numpy.linalg.norm(b.ravel())
    d = numpy.linalg.norm((a - b).ravel())
    return d / nb if nb > 0 else d
