"""The solve tables on the host: the Crout band factors with the
Schur-complement wrap (periodic lines) and the split-line tables (segment
blocks, spikes, the reduced system's inverse), applied to random right-hand
sides the way the sweeps apply them, solve the assembled LHS to FP64
rounding, for every implicit operator, periodic and non-periodic lines,
every boundary code and both symmetry variants, and line lengths from 8 to
2000 (single-segment, ragged last segment, many segments).  No GPU: the
harness (tests/solve_tables_harness.cpp) is compiled with pg_setup.cpp."""
import ctypes
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
OPK_D1, OPK_D8, OPK_SF, OPK_GF, OPK_D2, OPK_D4 = range(6)


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ is not available")
    out = str(tmp_path_factory.mktemp("solve") / "harness.so")
    cmd = [cxx, "-std=c++17", "-O2", "-shared", "-fPIC", "-o", out,
           os.path.join(ROOT, "tests", "solve_tables_harness.cpp"),
           os.path.join(ROOT, "pyranda_gb300", "csrc", "pg_setup.cpp")]
    for inc in ("/usr/local/cuda/include",):
        if os.path.isdir(inc):
            cmd[1:1] = ["-I", inc]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    lib.pg_test_solve_residual.restype = ctypes.c_int
    lib.pg_test_solve_residual.argtypes = [ctypes.c_int] * 7 + [ctypes.POINTER(ctypes.c_double)] * 2
    return lib


@pytest.mark.parametrize("kind", [OPK_D1, OPK_D8, OPK_SF, OPK_D2])
@pytest.mark.parametrize("n", [8, 31, 64, 100, 257, 2000])
@pytest.mark.parametrize("ends", ["PERI", "NONE", "SYMM+", "SYMM-", "XTND", "SYMM/NONE"])
def test_tables_solve_the_lhs(harness, kind, n, ends):
    per = ends == "PERI"
    bl, bh, sym = {"PERI": (0, 0, 1), "NONE": (0, 0, 1), "SYMM+": (1, 1, 1), "SYMM-": (1, 1, -1),
                   "XTND": (2, 2, 1), "SYMM/NONE": (1, 0, 1)}[ends]
    rb, rs = ctypes.c_double(), ctypes.c_double()
    rc = harness.pg_test_solve_residual(kind, n, int(per), bl, bh, sym, 7, ctypes.byref(rb), ctypes.byref(rs))
    assert rc == 0, rc
    assert rb.value <= 1e-13, ("banded", rb.value)
    assert rs.value <= 1e-12, ("split", rs.value)
