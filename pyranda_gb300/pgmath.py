"""numpy-named functions over device fields, for the EOM/IC string language.

pyranda's translator rewrites ``sin(`` to ``numpy.sin(`` and scripts write
``numpy.minimum(...)`` directly (pyranda/pyranda.py:842-864,
examples/TaylorGreen.py:84-86).  The evaluation namespace binds the name
``numpy`` to this module, so those calls run on torch device tensors and on
plain Python numbers alike.
"""
import math

import numpy as _np
import torch

pi = math.pi
e = math.e
inf = math.inf
nan = math.nan
float64 = _np.float64


def _t(x):
    return isinstance(x, torch.Tensor)


def _unary(tfun, nfun):
    def f(x, *a, **k):
        if _t(x):
            return tfun(x, *a, **k)
        return nfun(x, *a, **k)
    f.__name__ = getattr(nfun, "__name__", "f")
    return f


sin = _unary(torch.sin, _np.sin)
cos = _unary(torch.cos, _np.cos)
tan = _unary(torch.tan, _np.tan)
arcsin = _unary(torch.asin, _np.arcsin)
arccos = _unary(torch.acos, _np.arccos)
arctan = _unary(torch.atan, _np.arctan)
sinh = _unary(torch.sinh, _np.sinh)
cosh = _unary(torch.cosh, _np.cosh)
tanh = _unary(torch.tanh, _np.tanh)
exp = _unary(torch.exp, _np.exp)
log = _unary(torch.log, _np.log)
log10 = _unary(torch.log10, _np.log10)
sqrt = _unary(torch.sqrt, _np.sqrt)
abs = _unary(torch.abs, _np.abs)
absolute = abs
sign = _unary(torch.sign, _np.sign)
floor = _unary(torch.floor, _np.floor)
ceil = _unary(torch.ceil, _np.ceil)
isnan = _unary(torch.isnan, _np.isnan)


def _pair(tfun, nfun):
    def f(a, b):
        if _t(a) or _t(b):
            dev = a.device if _t(a) else b.device
            a = a if _t(a) else torch.as_tensor(a, dtype=torch.float64, device=dev)
            b = b if _t(b) else torch.as_tensor(b, dtype=torch.float64, device=dev)
            return tfun(a, b)
        return nfun(a, b)
    return f


minimum = _pair(torch.minimum, _np.minimum)
maximum = _pair(torch.maximum, _np.maximum)
arctan2 = _pair(torch.atan2, _np.arctan2)
power = _pair(torch.pow, _np.power)
fmod = _pair(torch.fmod, _np.fmod)


def where(cond, a, b):
    if _t(cond) or _t(a) or _t(b):
        dev = next(x.device for x in (cond, a, b) if _t(x))
        a = a if _t(a) else torch.as_tensor(a, dtype=torch.float64, device=dev)
        b = b if _t(b) else torch.as_tensor(b, dtype=torch.float64, device=dev)
        cond = cond if _t(cond) else torch.as_tensor(cond, device=dev)
        return torch.where(cond, a, b)
    return _np.where(cond, a, b)


def dot(a, b):
    if _t(a) or _t(b):
        return (a * b).sum()
    return _np.dot(a, b)


def erf(x):
    return torch.special.erf(x) if _t(x) else math.erf(x)


def zeros_like(x):
    return torch.zeros_like(x) if _t(x) else _np.zeros_like(x)


def ones_like(x):
    return torch.ones_like(x) if _t(x) else _np.ones_like(x)


def max(x):
    return torch.amax(x) if _t(x) else _np.max(x)


def min(x):
    return torch.amin(x) if _t(x) else _np.min(x)


def sum(x):
    return torch.sum(x) if _t(x) else _np.sum(x)


class _Special:
    erf = staticmethod(erf)


class scipy:
    """``scipy.special.erf`` as produced by the translator (pyranda.py:856)."""
    special = _Special
