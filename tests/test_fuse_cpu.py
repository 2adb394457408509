"""EOM fusion on the CPU: the rewrite of equations and the generated CUDA source.

The generated kernels must compile for sm_103a (nvcc runs here without a
GPU) and every elementwise subtree of the reference's example EOMs must be
found.  The bit-for-bit comparison with unfused steps is a GPU test.
"""
import ast
import shutil

import pytest

from pyranda_gb300 import fuse
from pyranda_gb300.problems import KH_EOM, SHOCK_EOM, TGV_EOM
from pyranda_gb300.pyranda import EVAL_GLOBALS, pyrandaEq, pyrandaSim


class _Sim:
    """Just enough of pyrandaSim to translate and rewrite equations."""

    def __init__(self, eom):
        self.sMap = {}
        pyrandaSim.get_sMap(self)
        self.sMap.update({"dt.courant(": "self.packages['Timestep'].courant(",
                          "dt.diff(": "self.packages['Timestep'].diff(",
                          "bc.extrap(": "self.packages['BC'].extrap(", "bc.const(": "self.packages['BC'].const("})
        self.equations = []
        for line in [el for el in eom.split("\n") if el.strip() and el.strip()[0] != "#"]:
            self.equations.append(pyrandaEq(line, self.sMap))


@pytest.mark.parametrize("arith", ["fp64", "fp32"])
@pytest.mark.parametrize("eom", [TGV_EOM, SHOCK_EOM, KH_EOM.replace("gamma", "1.4").replace("R0", "1.0")
                                 .replace("cv", "2.5")], ids=["tgv", "shock", "kh"])
def test_rewrite_and_generated_source_compiles(eom, arith, tmp_path):
    sim = _Sim(eom)
    f = fuse.Fuser(sim, arith=arith)
    f.install(EVAL_GLOBALS)
    assert len(f.kernels) >= 10
    for i, k in enumerate(f.kernels):   # as if every leaf were a field, some a device scalar or a number
        k.sig = "".join("fsc"[(i + q) % 3] if q else "f" for q in range(k.nleaves))
    for g in f.groups:
        g.sig = "f" * len(g.inputs)
    assert len(f.groups) >= 1
    src = f.source()
    ast_ok = all(k.expr.count("(") == k.expr.count(")") for k in f.kernels)
    assert ast_ok
    if shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    cu = tmp_path / "k.cu"
    cu.write_text(src)
    import subprocess
    from pyranda_gb300.build import ARCH, nvcc
    r = subprocess.run([nvcc()] + ARCH + ["-O3", "-fmad=%s" % ("true" if arith == "fp32" else "false"), "-c",
                        str(cu), "-o", str(tmp_path / "k.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]


def test_power_special_cases_follow_torch():
    g = fuse._Gen()
    c, _ = g.emit(ast.parse("a**2 + b**0.5 - c**-1", mode="eval").body)
    assert "PG_MUL(L0, L0)" in c and "PG_SQRT(L1)" in c and "PG_DIV(PG_C(1.0), L2)" in c
    assert "#define PG_MUL(a, b) __dmul_rn(a, b)" in fuse.PRELUDE_FP64
    assert "#define PG_SQRT(x) sqrt(x)" in fuse.PRELUDE_FP64


def test_unknown_arithmetic_is_refused():
    with pytest.raises(ValueError):
        fuse.Fuser(_Sim(TGV_EOM), arith="fp16")


def test_pde_kernels_own_their_stage_update():
    """Every PDE of the TGV EOM ends in one fused kernel and no later PDE reads its variable, so each
    kernel also applies its variable's LSRK stage; a later PDE reading the variable blocks it."""
    sim = _Sim(TGV_EOM)
    f = fuse.Fuser(sim)
    f.install(EVAL_GLOBALS)
    assert [k.rk for k in f.kernels if k.rk] == ["rho", "rhou", "rhov", "rhow", "Et"]
    eom = "ddt(:a:) = -ddx(:a:*:b:) - ddy(:a:)\nddt(:b:) = -ddx(:b:*:a:) - ddy(:b:)\n"
    f = fuse.Fuser(_Sim(eom))
    f.install(EVAL_GLOBALS)
    assert [k.rk for k in f.kernels if k.rk] == ["b"]
