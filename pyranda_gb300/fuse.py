"""Fusion of the EOM's elementwise arithmetic into generated CUDA kernels.

pyranda evaluates every EOM line as numpy expressions, one temporary array
per operation (pyranda/pyrandaEq.py:16-48, pyranda.py:376-428).  Here each
maximal elementwise subtree of an equation's right-hand side (arithmetic,
constant powers and the numpy functions of the string language) becomes one
CUDA kernel that reads each field once and writes its result once; the
compact operators (ddx, fbar, ring, ...) and the reductions stay calls into
the library and become the kernels' inputs.

The kernels repeat torch's per-operation rounding: every product, quotient
and sum is rounded separately (no FMA contraction), x**2 is x*x, x**0.5 is
sqrt(x), x**-1 is 1/x (torch's pow special cases), and minimum/maximum
propagate NaN, so a fused step reproduces the unfused one bit for bit.  All
kernels of a simulation are generated into one source file, compiled once
with nvcc for sm_103a and cached under pyranda_gb300/_build/jit by the
source's hash.

That is the FP64 arithmetic (Fuser(..., arith="fp64")).  The fast paths may
instead evaluate the same expressions in FP32 (arith="fp32"): every FP64
load is narrowed by integer operations (round to nearest even; infinities
and NaN kept; magnitudes below 2**-126 flushed to zero), the arithmetic and
the math functions run at FP32 with FMA contraction, and the result is
widened back to the FP64 field.  GB300's FP64 rate is about 1/58 of its FP32
rate and its F2F conversions run on the FP64 pipe, which bounds the FP64
kernels; the RK state accumulation, the boundary-closure solves and the d8
LAD sweeps are not elementwise EOM arithmetic and keep FP64 either way.
A third form, arith="df64", evaluates them in double-float arithmetic
(FP32 hi + lo pairs, ~48 bits; PRELUDE_DF64).
"""
import ast
import copy
import ctypes
import hashlib
import os
import subprocess

import torch

from .build import ARCH, OUT, nvcc

JIT_DIR = os.path.join(OUT, "jit")


class _RkDone:
    """Returned for a PDE right-hand side whose kernel already applied the RK stage update."""

    def __repr__(self):
        return "RK_DONE"


RK_DONE = _RkDone()

_UNARY = {"sqrt": "PG_SQRT({0})", "abs": "PG_ABS({0})", "absolute": "PG_ABS({0})", "exp": "PG_EXP({0})",
          "log": "PG_LOG({0})", "sin": "PG_SIN({0})", "cos": "PG_COS({0})", "tan": "PG_TAN({0})",
          "tanh": "PG_TANH({0})", "sinh": "PG_SINH({0})", "cosh": "PG_COSH({0})", "arctan": "PG_ATAN({0})",
          "arcsin": "PG_ASIN({0})", "arccos": "PG_ACOS({0})", "log10": "PG_LOG10({0})",
          "floor": "PG_FLOOR({0})", "ceil": "PG_CEIL({0})", "sign": "pg_sign({0})"}
_BINARY = {"minimum": "pg_min({0}, {1})", "maximum": "pg_max({0}, {1})"}
_ARITH = {ast.Add: "PG_ADD({0}, {1})", ast.Sub: "PG_SUB({0}, {1})", ast.Mult: "PG_MUL({0}, {1})",
          ast.Div: "PG_DIV({0}, {1})"}

_COMMON = r"""#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>
__device__ __forceinline__ real pg_min(real a, real b) { return (a != a) ? a : ((b != b) ? b : (a < b ? a : b)); }
__device__ __forceinline__ real pg_max(real a, real b) { return (a != a) ? a : ((b != b) ? b : (a > b ? a : b)); }
__device__ __forceinline__ real pg_sign(real a) { return (a > (real)0) ? (real)1 : ((a < (real)0) ? (real)-1 : a); }
"""

# FP64 arithmetic: every operation rounded on its own, as torch's separate kernels do.
PRELUDE_FP64 = r"""typedef double real;
#define PG_CARG double
#define PG_LOADC(x) (x)
#define PG_LOAD(x) (x)
#define PG_STORE(x) (x)
#define PG_C(x) (x)
#define PG_ADD(a, b) __dadd_rn(a, b)
#define PG_SUB(a, b) __dsub_rn(a, b)
#define PG_MUL(a, b) __dmul_rn(a, b)
#define PG_DIV(a, b) __ddiv_rn(a, b)
#define PG_SQRT(x) sqrt(x)
#define PG_RSQRT(x) rsqrt(x)
#define PG_POW(a, b) pow(a, b)
#define PG_ABS(x) fabs(x)
#define PG_EXP(x) exp(x)
#define PG_LOG(x) log(x)
#define PG_SIN(x) sin(x)
#define PG_COS(x) cos(x)
#define PG_TAN(x) tan(x)
#define PG_TANH(x) tanh(x)
#define PG_SINH(x) sinh(x)
#define PG_COSH(x) cosh(x)
#define PG_ATAN(x) atan(x)
#define PG_ASIN(x) asin(x)
#define PG_ACOS(x) acos(x)
#define PG_LOG10(x) log10(x)
#define PG_FLOOR(x) floor(x)
#define PG_CEIL(x) ceil(x)
""" + _COMMON

# FP32 arithmetic on FP64 fields (the fast paths): values converted by integer
# operations (GB300 runs F2F on its FP64 pipe) keeping infinities and NaN,
# FP32 math, results widened back to FP64.
_CONV = r"""__device__ __forceinline__ float pg_d2f(double d) {
  const unsigned hi = (unsigned)__double2hiint(d), lo = (unsigned)__double2loint(d);
  const unsigned sign = hi & 0x80000000u, mag = hi & 0x7fffffffu;
  if (mag >= 0x7ff00000u) return __uint_as_float(sign | 0x7f800000u | ((((mag & 0xfffffu) | lo) != 0u) ? 0x400000u : 0u));
  if (mag >= (1151u << 20)) return __uint_as_float(sign | 0x7f800000u);
  if (mag < (897u << 20)) return __uint_as_float(sign);
  unsigned f = ((mag - (896u << 20)) << 3) | (lo >> 29);
  f += ((lo >> 28) & 1u) & (((lo & 0x0fffffffu) != 0u) | (f & 1u));
  return __uint_as_float(f | sign);
}
__device__ __forceinline__ double pg_f2d(float x) {
  const unsigned u = __float_as_uint(x);
  const unsigned sign = u & 0x80000000u, mag = u & 0x7fffffffu;
  if (mag >= 0x7f800000u) return __hiloint2double((int)(sign | 0x7ff00000u | ((mag & 0x7fffffu) ? 0x80000u : 0u)), 0);
  if (mag < 0x00800000u) return __hiloint2double((int)sign, 0);
  return __hiloint2double((int)(((mag >> 3) + (896u << 20)) | sign), (int)(mag << 29));
}
"""

PRELUDE_FP32 = r"""typedef float real;
""" + _CONV + r"""#define PG_CARG float
#define PG_LOADC(x) (x)
#define PG_LOAD(x) pg_d2f(x)
#define PG_STORE(x) pg_f2d(x)
#define PG_C(x) ((float)(x))
#define PG_ADD(a, b) ((a) + (b))
#define PG_SUB(a, b) ((a) - (b))
#define PG_MUL(a, b) ((a) * (b))
#define PG_DIV(a, b) ((a) / (b))
#define PG_SQRT(x) sqrtf(x)
#define PG_RSQRT(x) rsqrtf(x)
#define PG_POW(a, b) powf(a, b)
#define PG_ABS(x) fabsf(x)
#define PG_EXP(x) expf(x)
#define PG_LOG(x) logf(x)
#define PG_SIN(x) sinf(x)
#define PG_COS(x) cosf(x)
#define PG_TAN(x) tanf(x)
#define PG_TANH(x) tanhf(x)
#define PG_SINH(x) sinhf(x)
#define PG_COSH(x) coshf(x)
#define PG_ATAN(x) atanf(x)
#define PG_ASIN(x) asinf(x)
#define PG_ACOS(x) acosf(x)
#define PG_LOG10(x) log10f(x)
#define PG_FLOOR(x) floorf(x)
#define PG_CEIL(x) ceilf(x)
""" + _COMMON


# Double-float arithmetic on FP64 fields: every value is an unevaluated sum
# hi + lo of two FP32 numbers (about 48 significant bits), loaded from FP64
# by the integer narrowing above plus one FP64 subtraction for the residual,
# and stored as the FP64 sum hi + lo.  The operations are the classic
# error-free transformations on the FP32 pipes (Dekker 1971; Knuth's
# two-sum; the FMA form of the exact product): add / subtract ~2^-47,
# multiply ~2^-47, divide and square root with one correction step ~2^-46
# relative.  GB300 runs FP32 about 58x faster than FP64, so the EOM's long
# expressions (pressure, stresses, energy flux) leave the FP64 pipe.  Other
# functions (exp, log, pow with a non-integer exponent, ...) are evaluated
# in FP64 from the value's FP64 sum.  Non-finite values are not carried:
# an infinity becomes NaN (the simulation's NaN checks catch both).
PRELUDE_DF64 = r"""#include <cstdint>
#include <cmath>
#include <cuda_runtime.h>
struct pg_df { float hi, lo; };
typedef pg_df real;
""" + _CONV + r"""__device__ __forceinline__ pg_df pg_df_make(float h, float l) { pg_df r; r.hi = h; r.lo = l; return r; }
// FP64 -> hi + lo: hi the FP32 rounding, lo the FP32 rounding of the exact residual
__device__ __forceinline__ pg_df pg_df_load(double d) {
  const float h = pg_d2f(d);
  const float l = (__fsub_rn(h, h) == 0.0f) ? pg_d2f(__dsub_rn(d, pg_f2d(h))) : 0.0f;
  return pg_df_make(h, l);
}
__device__ __forceinline__ double pg_df_store(pg_df a) { return __dadd_rn(pg_f2d(a.hi), pg_f2d(a.lo)); }
// a literal: the conversions fold at compile time
__device__ __forceinline__ pg_df pg_df_c(double c) {
  const float h = (float)c;
  return pg_df_make(h, (float)(c - (double)h));
}
__device__ __forceinline__ pg_df pg_df_fast2sum(float s, float t) {  // |s| >= |t|
  const float h = __fadd_rn(s, t);
  return pg_df_make(h, __fsub_rn(t, __fsub_rn(h, s)));
}
__device__ __forceinline__ pg_df pg_df_add(pg_df a, pg_df b) {
  const float s = __fadd_rn(a.hi, b.hi);
  const float v = __fsub_rn(s, a.hi);
  const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, v)), __fsub_rn(b.hi, v));
  return pg_df_fast2sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ pg_df operator-(pg_df a) { return pg_df_make(-a.hi, -a.lo); }
__device__ __forceinline__ pg_df pg_df_sub(pg_df a, pg_df b) { return pg_df_add(a, -b); }
__device__ __forceinline__ pg_df pg_df_mul(pg_df a, pg_df b) {
  const float p = __fmul_rn(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.hi, -p);
  e = __fmaf_rn(a.hi, b.lo, e);
  e = __fmaf_rn(a.lo, b.hi, e);
  return pg_df_fast2sum(p, e);
}
__device__ __forceinline__ pg_df pg_df_div(pg_df a, pg_df b) {
  const float q1 = __fdiv_rn(a.hi, b.hi);
  const pg_df r = pg_df_sub(a, pg_df_mul(pg_df_make(q1, 0.0f), b));
  return pg_df_fast2sum(q1, __fdiv_rn(r.hi, b.hi));
}
__device__ __forceinline__ pg_df pg_df_sqrt(pg_df a) {
  if (!(a.hi > 0.0f)) return pg_df_make(__fsqrt_rn(a.hi), 0.0f);  // zero, negative or NaN
  const float s = __fsqrt_rn(a.hi);
  const pg_df e = pg_df_sub(a, pg_df_mul(pg_df_make(s, 0.0f), pg_df_make(s, 0.0f)));
  return pg_df_fast2sum(s, __fdiv_rn(e.hi, __fmul_rn(2.0f, s)));
}
__device__ __forceinline__ pg_df pg_df_abs(pg_df a) { return (a.hi < 0.0f) ? -a : a; }
__device__ __forceinline__ bool pg_df_lt(pg_df a, pg_df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ pg_df pg_min(pg_df a, pg_df b) {
  return (a.hi != a.hi) ? a : ((b.hi != b.hi) ? b : (pg_df_lt(a, b) ? a : b));
}
__device__ __forceinline__ pg_df pg_max(pg_df a, pg_df b) {
  return (a.hi != a.hi) ? a : ((b.hi != b.hi) ? b : (pg_df_lt(b, a) ? a : b));
}
__device__ __forceinline__ pg_df pg_sign(pg_df a) {
  return (a.hi > 0.0f) ? pg_df_make(1.0f, 0.0f) : ((a.hi < 0.0f) ? pg_df_make(-1.0f, 0.0f) : a);
}
#define PG_F64(f, x) pg_df_load(f(pg_df_store(x)))
#define PG_CARG double
#define PG_LOADC(x) pg_df_load(x)
#define PG_LOAD(x) pg_df_load(x)
#define PG_STORE(x) pg_df_store(x)
#define PG_C(x) pg_df_c(x)
#define PG_ADD(a, b) pg_df_add(a, b)
#define PG_SUB(a, b) pg_df_sub(a, b)
#define PG_MUL(a, b) pg_df_mul(a, b)
#define PG_DIV(a, b) pg_df_div(a, b)
#define PG_SQRT(x) pg_df_sqrt(x)
#define PG_RSQRT(x) pg_df_div(pg_df_make(1.0f, 0.0f), pg_df_sqrt(x))
#define PG_POW(a, b) pg_df_load(pow(pg_df_store(a), pg_df_store(b)))
#define PG_ABS(x) pg_df_abs(x)
#define PG_EXP(x) PG_F64(exp, x)
#define PG_LOG(x) PG_F64(log, x)
#define PG_SIN(x) PG_F64(sin, x)
#define PG_COS(x) PG_F64(cos, x)
#define PG_TAN(x) PG_F64(tan, x)
#define PG_TANH(x) PG_F64(tanh, x)
#define PG_SINH(x) PG_F64(sinh, x)
#define PG_COSH(x) PG_F64(cosh, x)
#define PG_ATAN(x) PG_F64(atan, x)
#define PG_ASIN(x) PG_F64(asin, x)
#define PG_ACOS(x) PG_F64(acos, x)
#define PG_LOG10(x) PG_F64(log10, x)
#define PG_FLOOR(x) PG_F64(floor, x)
#define PG_CEIL(x) PG_F64(ceil, x)
"""


def _const(node):
    if isinstance(node, ast.Constant) and isinstance(node.value, (int, float)) and not isinstance(node.value, bool):
        return float(node.value)
    if isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub):
        c = _const(node.operand)
        return None if c is None else -c
    return None


def _is_numpy(f):
    return isinstance(f, ast.Attribute) and isinstance(f.value, ast.Name) and f.value.id == "numpy"


def _elementwise(node):
    """True when the generator fuses this node (otherwise it is a leaf)."""
    if isinstance(node, ast.BinOp):
        return type(node.op) in _ARITH or (isinstance(node.op, ast.Pow))
    if isinstance(node, ast.UnaryOp):
        return isinstance(node.op, (ast.USub, ast.UAdd))
    if isinstance(node, ast.Call) and _is_numpy(node.func) and not node.keywords:
        return (node.func.attr in _UNARY and len(node.args) == 1) or (node.func.attr in _BINARY and len(node.args) == 2)
    return False


def _children(node):
    if isinstance(node, ast.BinOp):
        return [node.left, node.right]
    if isinstance(node, ast.UnaryOp):
        return [node.operand]
    return list(node.args)


def _ops(node):
    return (1 + sum(_ops(k) for k in _children(node))) if _elementwise(node) else 0


def _pow(x, c):
    # torch's pow(tensor, scalar) special cases
    if c == 2.0:
        return "PG_MUL(%s, %s)" % (x, x)
    if c == 3.0:
        return "PG_MUL(PG_MUL(%s, %s), %s)" % (x, x, x)
    if c == 0.5:
        return "PG_SQRT(%s)" % x
    if c == -0.5:
        return "PG_RSQRT(%s)" % x
    if c == -1.0:
        return "PG_DIV(PG_C(1.0), %s)" % x
    if c == -2.0:
        return "PG_DIV(PG_C(1.0), PG_MUL(%s, %s))" % (x, x)
    if c == 1.0:
        return x
    return "PG_POW(%s, PG_C(%r))" % (x, float(c))


class _Gen:
    """C expression and Python AST (leaves renamed L0..Ln) of one elementwise subtree."""

    def __init__(self):
        self.leaves = []

    def emit(self, node):
        c = _const(node)
        if c is not None and not isinstance(node, ast.UnaryOp):
            return "PG_C(%r)" % c, copy.copy(node)
        if isinstance(node, ast.Attribute) and _is_numpy(node) and node.attr == "pi":
            return "PG_C(%r)" % 3.141592653589793, copy.copy(node)
        if _elementwise(node):
            if isinstance(node, ast.UnaryOp):
                cx, px = self.emit(node.operand)
                return ("(-%s)" % cx if isinstance(node.op, ast.USub) else cx), ast.UnaryOp(op=node.op, operand=px)
            if isinstance(node, ast.BinOp):
                cl, pl = self.emit(node.left)
                if isinstance(node.op, ast.Pow) and _const(node.right) is not None:
                    return _pow(cl, _const(node.right)), ast.BinOp(left=pl, op=node.op, right=copy.copy(node.right))
                cr, pr = self.emit(node.right)
                fmt = _ARITH.get(type(node.op), "PG_POW({0}, {1})")
                return fmt.format(cl, cr), ast.BinOp(left=pl, op=node.op, right=pr)
            args = [self.emit(a) for a in node.args]
            fmt = _UNARY.get(node.func.attr) if len(args) == 1 else _BINARY[node.func.attr]
            return fmt.format(*[a[0] for a in args]), ast.Call(func=copy.copy(node.func), args=[a[1] for a in args],
                                                               keywords=[])
        self.leaves.append(node)
        name = "L%d" % (len(self.leaves) - 1)
        return name, ast.Name(id=name, ctx=ast.Load())


class Kernel:
    """One fused subtree: C expression, Python form, leaf kinds and compiled launcher."""

    def __init__(self, index, expr, pyform, nleaves, globals_):
        self.index, self.expr, self.nleaves = index, expr, nleaves
        lam = ast.Expression(body=ast.Lambda(
            args=ast.arguments(posonlyargs=[], args=[ast.arg(arg="L%d" % i) for i in range(nleaves)],
                               kwonlyargs=[], kw_defaults=[], defaults=[]), body=pyform))
        ast.fix_missing_locations(lam)
        self.eager = eval(compile(lam, "<fused %d>" % index, "eval"), globals_)
        self.sig = None      # leaf kinds of the recording call: f field, s device scalar, c number
        self.fn = None
        self.rk = None       # conserved variable whose RK stage update this kernel also performs
        self.rkfn = None

    def name(self):
        return "pg_fused_%d" % self.index

    def source(self):
        args, defs, call = [], [], []
        for i, k in enumerate(self.sig):
            if k in "fs":
                args.append("const double* __restrict__ p%d" % i)
                defs.append("const real L%d = PG_LOAD(p%d[%s]);" % (i, i, "i" if k == "f" else "0"))
                call.append("p%d" % i)
            else:
                args.append("PG_CARG c%d" % i)
                defs.append("const real L%d = PG_LOADC(c%d);" % (i, i))
                call.append("c%d" % i)
        params = ", ".join(["int64_t n", "double* __restrict__ out"] + args)
        return ('extern "C" __global__ void %(k)s(%(p)s) {\n'
                "  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;"
                " i += (int64_t)gridDim.x * blockDim.x) {\n    %(d)s\n    out[i] = PG_STORE(%(e)s);\n  }\n}\n"
                'extern "C" int %(k)s_launch(%(p)s, void* stream) {\n'
                "  if (n <= 0) return 0;\n"
                "  int64_t b = (n + 255) / 256;\n  if (b > 152 * 16) b = 152 * 16;\n"
                "  %(k)s<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(n, out%(c)s);\n"
                "  return (int)cudaGetLastError();\n}\n") % {
                    "k": self.name(), "p": params, "d": " ".join(defs), "e": self.expr,
                    "c": "".join(", " + c for c in call)} + (self._rk_source(args, defs, call) if self.rk else "")

    def _rk_source(self, args, defs, call):
        """The same expression as the right-hand side F of the PDE of self.rk, fused with its
        LSRK stage: PHI = A PHI + dt F, U = U + B PHI, in the arithmetic of the stage kernel
        (rk_stage_kernel), so the result equals the unfused stage bit for bit."""
        params = ", ".join(["int64_t n", "double* __restrict__ phi", "double* __restrict__ u", "double A", "double B",
                            "const double* __restrict__ dtp", "int dt_field"] + args)
        return ('extern "C" __global__ void %(k)s_rk(%(p)s) {\n'
                "  const double dt0 = dt_field ? 0.0 : dtp[0];\n"
                "  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;"
                " i += (int64_t)gridDim.x * blockDim.x) {\n    %(d)s\n"
                "    const double f = PG_STORE(%(e)s);\n"
                "    const double dt = dt_field ? dtp[i] : dt0;\n"
                "    const double p = __fma_rn(dt, f, __dmul_rn(A, phi[i]));\n"
                "    phi[i] = p;\n    u[i] = __fma_rn(B, p, u[i]);\n  }\n}\n"
                'extern "C" int %(k)s_rk_launch(%(p)s, void* stream) {\n'
                "  if (n <= 0) return 0;\n"
                "  int64_t b = (n + 255) / 256;\n  if (b > 152 * 16) b = 152 * 16;\n"
                "  %(k)s_rk<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(n, phi, u, A, B, dtp, dt_field%(c)s);\n"
                "  return (int)cudaGetLastError();\n}\n") % {
                    "k": self.name(), "p": params, "d": " ".join(defs), "e": self.expr,
                    "c": "".join(", " + c for c in call)}


def compile_source(src, fmad=False):
    """nvcc for sm_103a into a shared library cached under the source's hash; returns its path.

    FP64 arithmetic is compiled without FMA contraction (torch rounds every
    product on its own); FP32 arithmetic lets nvcc contract.
    """
    h = hashlib.sha1((src + ("fmad" if fmad else "")).encode()).hexdigest()[:16]
    os.makedirs(JIT_DIR, exist_ok=True)
    so = os.path.join(JIT_DIR, "fused_%s.so" % h)
    if not os.path.exists(so):
        cu = os.path.join(JIT_DIR, "fused_%s.cu" % h)
        with open(cu, "w") as f:
            f.write(src)
        tmp = so + ".%d.tmp" % os.getpid()
        cmd = [nvcc()] + ARCH + ["-O3", "-fmad=%s" % ("true" if fmad else "false"), "-shared",
                                 "-Xcompiler", "-fPIC", "-o", tmp, cu]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on the fused EOM kernels:\n" + r.stderr[-3000:])
        os.replace(tmp, so)
    return so


def _varname(node):
    """'x' for the translated variable reference self.variables["x"].data, else None."""
    if (isinstance(node, ast.Attribute) and node.attr == "data" and isinstance(node.value, ast.Subscript)
            and isinstance(node.value.value, ast.Attribute) and node.value.value.attr == "variables"
            and isinstance(node.value.value.value, ast.Name) and node.value.value.value.id == "self"):
        sl = node.value.slice
        if isinstance(sl, ast.Constant) and isinstance(sl.value, str):
            return sl.value
    return None


def _pure(node):
    """True when every leaf of an elementwise tree is a variable reference or a constant."""
    if _elementwise(node):
        return all(_pure(k) for k in _children(node))
    if _varname(node) is not None or _const(node) is not None:
        return True
    return isinstance(node, ast.Attribute) and _is_numpy(node) and node.attr == "pi"


class Group:
    """Consecutive algebraic equations with purely elementwise right-hand sides, fused into one kernel.

    The kernel loads every input variable once, keeps the values the group
    assigns in registers for the later equations, and writes each equation's
    result to its own output field.
    """

    def __init__(self, index, eqs):
        self.index, self.eqs = index, eqs
        self.inputs = []          # variable names read before the group assigns them
        self.exprs = []           # C expression of each equation
        self.refs = []            # variables each equation reads
        assigned = {}
        for k, eq in enumerate(eqs):
            node = ast.parse(eq.sRHS, mode="eval").body
            self.exprs.append(self._emit(node, assigned))
            self.refs.append({_varname(x) for x in ast.walk(node)} - {None})
            assigned[eq.LHS[0]] = "o%d" % k
        self.sig = None
        self.fn = None

    def _emit(self, node, assigned):
        name = _varname(node)
        if name is not None:
            if name in assigned:
                return assigned[name]
            if name not in self.inputs:
                self.inputs.append(name)
            return "L%d" % self.inputs.index(name)
        c = _const(node)
        if c is not None and not isinstance(node, ast.UnaryOp):
            return "PG_C(%r)" % c
        if isinstance(node, ast.Attribute):
            return "PG_C(%r)" % 3.141592653589793
        if isinstance(node, ast.UnaryOp):
            x = self._emit(node.operand, assigned)
            return "(-%s)" % x if isinstance(node.op, ast.USub) else x
        if isinstance(node, ast.BinOp):
            left = self._emit(node.left, assigned)
            if isinstance(node.op, ast.Pow) and _const(node.right) is not None:
                return _pow(left, _const(node.right))
            return _ARITH.get(type(node.op), "PG_POW({0}, {1})").format(left, self._emit(node.right, assigned))
        args = [self._emit(a, assigned) for a in node.args]
        fmt = _UNARY.get(node.func.attr) if len(args) == 1 else _BINARY[node.func.attr]
        return fmt.format(*args)

    def name(self):
        return "pg_fused_group_%d" % self.index

    def source(self):
        args, defs, call = [], [], []
        for i, k in enumerate(self.sig):
            if k in "fs":
                args.append("const double* __restrict__ p%d" % i)
                defs.append("const real L%d = PG_LOAD(p%d[%s]);" % (i, i, "i" if k == "f" else "0"))
                call.append("p%d" % i)
            else:
                args.append("PG_CARG c%d" % i)
                defs.append("const real L%d = PG_LOADC(c%d);" % (i, i))
                call.append("c%d" % i)
        outs = ["double* __restrict__ out%d" % k for k in range(len(self.eqs))]
        params = ", ".join(["int64_t n"] + outs + args)
        body = " ".join(defs) + " " + " ".join("const real o%d = %s;" % (k, e) for k, e in enumerate(self.exprs))
        stores = " ".join("out%d[i] = PG_STORE(o%d);" % (k, k) for k in range(len(self.eqs)))
        return ('extern "C" __global__ void %(k)s(%(p)s) {\n'
                "  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;"
                " i += (int64_t)gridDim.x * blockDim.x) {\n    %(b)s\n    %(s)s\n  }\n}\n"
                'extern "C" int %(k)s_launch(%(p)s, void* stream) {\n'
                "  if (n <= 0) return 0;\n"
                "  int64_t b = (n + 255) / 256;\n  if (b > 152 * 16) b = 152 * 16;\n"
                "  %(k)s<<<(unsigned)b, 256, 0, (cudaStream_t)stream>>>(n%(o)s%(c)s);\n"
                "  return (int)cudaGetLastError();\n}\n") % {
                    "k": self.name(), "p": params, "b": body, "s": stores,
                    "o": "".join(", out%d" % k for k in range(len(self.eqs))),
                    "c": "".join(", " + c for c in call)}

    def run(self, sim, fuser):
        """Evaluate the group; returns the outputs in equation order (or None: evaluate unfused)."""
        g = sim.grid
        kinds, args = [], []
        for name in self.inputs:
            v = sim.variables[name].data
            if isinstance(v, torch.Tensor) and v.dim() > 0:
                if not (v.dtype == torch.float64 and v.device == g.device and tuple(v.shape) == g.n
                        and g._fortran_ok(v)):
                    return None
                kinds.append("f")
                args.append(ctypes.c_void_p(v.data_ptr()))
            elif isinstance(v, torch.Tensor):
                if v.dtype != torch.float64 or v.device != g.device:
                    return None
                kinds.append("s")
                args.append(ctypes.c_void_p(v.data_ptr()))
            elif isinstance(v, (int, float)) and not isinstance(v, bool):
                kinds.append("c")
                args.append(fuser.scalar(v))
            else:
                return None
        sig = "".join(kinds)
        if not self._all_fields(sig):
            return None
        if self.sig is None:
            self.sig = sig
        if self.fn is None or self.sig != sig:
            return None
        outs = [g.empty() for _ in self.eqs]
        rc = self.fn(ctypes.c_int64(g.npts), *[ctypes.c_void_p(o.data_ptr()) for o in outs], *args,
                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc != 0:
            raise RuntimeError("fused kernel %s failed with CUDA error %d" % (self.name(), rc))
        fuser.fused_calls += 1
        return outs

    def _all_fields(self, sig):
        """Every equation's result is a field (reads a field input, directly or through an earlier output)."""
        field_vars = {n for n, k in zip(self.inputs, sig) if k == "f"}
        for eq, refs in zip(self.eqs, self.refs):
            if not (refs & field_vars):
                return False
            field_vars.add(eq.LHS[0])
        return True


class Fuser:
    """Rewrites a simulation's EOM right-hand sides to use fused kernels.

    ``install(globals_)`` rewrites every equation; the first evaluation of
    each fused subtree records its leaf kinds and runs unfused (torch);
    ``build()`` compiles all recorded kernels in one nvcc call, after which
    they run fused.  A call whose leaves do not match the recorded kinds, or
    whose fields are not in the grid's layout, runs unfused.
    """

    def __init__(self, sim, min_ops=2, arith="fp64"):
        if arith not in ("fp64", "fp32", "df64"):
            raise ValueError("arith must be 'fp64', 'fp32' or 'df64'")
        self.sim = sim
        self.arith = arith
        self.min_ops = min_ops
        self.scalar = (lambda v: ctypes.c_float(float(v))) if arith == "fp32" else (lambda v: ctypes.c_double(float(v)))
        self.kernels = []
        self.groups = []
        self.lib = None
        self.fused_calls = 0
        self.rk_ctx = None     # set by rk4 around the flux evaluation of a stage

    def rewrite(self, src, globals_):
        tree = ast.parse(src, mode="eval")
        fuser = self

        class T(ast.NodeTransformer):
            def visit(self, node):
                if _elementwise(node) and _ops(node) >= fuser.min_ops:
                    g = _Gen()
                    expr, pyform = g.emit(node)
                    leaves = [self.visit(lf) for lf in g.leaves]
                    k = Kernel(len(fuser.kernels), expr, pyform, len(leaves), globals_)
                    fuser.kernels.append(k)
                    call = ast.Call(func=ast.Attribute(value=ast.Attribute(value=ast.Name(id="self", ctx=ast.Load()),
                                                                           attr="_fuse", ctx=ast.Load()),
                                                       attr="run", ctx=ast.Load()),
                                    args=[ast.Constant(k.index)] + leaves, keywords=[])
                    return ast.copy_location(call, node)
                return self.generic_visit(node)

        body = T().visit(tree.body)
        lam = ast.Expression(body=ast.Lambda(args=ast.arguments(posonlyargs=[], args=[ast.arg(arg="self")],
                                                                kwonlyargs=[], kw_defaults=[], defaults=[]),
                                             body=body))
        ast.fix_missing_locations(lam)
        return eval(compile(lam, "<fused equation>", "eval"), globals_)

    def install(self, globals_):
        # runs of consecutive algebraic equations with purely elementwise
        # right-hand sides become multi-output group kernels
        self.groups = []
        eqs = self.sim.equations
        i = 0
        while i < len(eqs):
            j = i
            while j < len(eqs) and self._groupable(eqs[j]):
                j += 1
            if j - i >= 2:
                grp = Group(len(self.groups), eqs[i:j])
                self.groups.append(grp)
                eqs[i]._fused_group = grp
                for e in eqs[i + 1:j]:
                    e._fused_member = True
            i = max(j, i + 1)
        for eq in eqs:
            n0 = len(self.kernels)
            eq.RHS = self.rewrite(eq.sRHS, globals_)
            if eq.kind == "PDE" and len(self.kernels) > n0 and self._rk_fusable(eq):
                self.kernels[-1].rk = eq.LHS[0]

    def _rk_fusable(self, eq):
        """The PDE's right-hand side is one fused kernel (its root) and no later PDE reads the
        variable, so the kernel may update the variable's RK state in place."""
        root = ast.parse(eq.sRHS, mode="eval").body
        if not (_elementwise(root) and _ops(root) >= self.min_ops):
            return False
        eqs = self.sim.equations
        var = eq.LHS[0]
        for later in eqs[eqs.index(eq) + 1:]:
            if later.kind != "PDE":
                continue
            if "packages" in later.sRHS:
                return False
            tree = ast.parse(later.sRHS, mode="eval")
            if any(_varname(x) == var for x in ast.walk(tree)):
                return False
        return True

    @staticmethod
    def _groupable(eq):
        if eq.kind != "ALG" or not eq.LHS or eq.rank != 1 or not eq.active:
            return False
        node = ast.parse(eq.sRHS, mode="eval").body
        return _elementwise(node) and _pure(node)

    def run(self, index, *leaves):
        k = self.kernels[index]
        g = self.sim.grid
        kinds, args = [], []
        for v in leaves:
            if isinstance(v, torch.Tensor) and v.dim() > 0:
                if not (v.dtype == torch.float64 and v.device == g.device and tuple(v.shape) == g.n
                        and g._fortran_ok(v)):
                    return k.eager(*leaves)
                kinds.append("f")
                args.append(ctypes.c_void_p(v.data_ptr()))
            elif isinstance(v, torch.Tensor):
                if v.dtype != torch.float64 or v.device != g.device:
                    return k.eager(*leaves)
                kinds.append("s")
                args.append(ctypes.c_void_p(v.data_ptr()))
            elif isinstance(v, (int, float)) and not isinstance(v, bool):
                kinds.append("c")
                args.append(self.scalar(v))
            else:
                return k.eager(*leaves)
        sig = "".join(kinds)
        if "f" not in sig:
            return k.eager(*leaves)
        if k.sig is None:
            k.sig = sig
        if k.fn is None or k.sig != sig:
            return k.eager(*leaves)
        ctx = self.rk_ctx
        if k.rk is not None and k.rkfn is not None and ctx is not None and k.rk in ctx["phi"]:
            dt = ctx["dt"]
            if not (isinstance(dt, torch.Tensor) and dt.dtype == torch.float64 and dt.device == g.device
                    and (dt.dim() == 0 or dt.numel() == g.npts)):
                return k.eager(*leaves)
            u = self.sim._field_of(k.rk)
            rc = k.rkfn(ctypes.c_int64(g.npts), ctypes.c_void_p(ctx["phi"][k.rk].data_ptr()),
                        ctypes.c_void_p(u.data_ptr()), ctypes.c_double(ctx["A"]), ctypes.c_double(ctx["B"]),
                        ctypes.c_void_p(dt.data_ptr()), ctypes.c_int(1 if dt.dim() > 0 else 0), *args,
                        ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
            if rc != 0:
                raise RuntimeError("fused kernel %s_rk failed with CUDA error %d" % (k.name(), rc))
            self.fused_calls += 1
            return RK_DONE
        out = g.empty()
        rc = k.fn(ctypes.c_int64(g.npts), ctypes.c_void_p(out.data_ptr()), *args,
                  ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
        if rc != 0:
            raise RuntimeError("fused kernel %s failed with CUDA error %d" % (k.name(), rc))
        self.fused_calls += 1
        return out

    def source(self):
        ks = [k for k in self.kernels if k.sig is not None] + [g for g in self.groups if g.sig is not None]
        # loads every kernel now: a first launch inside a graph capture would load its module there
        pre = ('extern "C" int pg_fused_preload() {\n  cudaFuncAttributes a;\n  int rc = 0;\n%s  return rc;\n}\n'
               % "".join("  rc |= (int)cudaFuncGetAttributes(&a, %s);\n" % nm for k in ks
                         for nm in ([k.name()] + ([k.name() + "_rk"] if getattr(k, "rk", None) else []))))
        prelude = {"fp64": PRELUDE_FP64, "fp32": PRELUDE_FP32, "df64": PRELUDE_DF64}[self.arith]
        return prelude + "".join(k.source() for k in ks) + pre

    def build(self):
        """Compile every recorded kernel (once per distinct source) and bind them; returns the .so path."""
        so = compile_source(self.source(), fmad=self.arith != "fp64")
        self.lib = ctypes.CDLL(so)
        if self.lib.pg_fused_preload() != 0:
            raise RuntimeError("loading the fused EOM kernels failed")
        for k in list(self.kernels) + list(self.groups):
            if k.sig is not None:
                fn = getattr(self.lib, k.name() + "_launch")
                fn.restype = ctypes.c_int
                k.fn = fn
                if getattr(k, "rk", None) is not None:
                    k.rkfn = getattr(self.lib, k.name() + "_rk_launch")
                    k.rkfn.restype = ctypes.c_int
        return so
