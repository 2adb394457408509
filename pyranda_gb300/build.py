"""Build the CUDA library ``libpyranda_gpu.so`` in-tree for sm_103a.

The translation units are compiled in parallel with nvcc and linked into
``pyranda_gb300/_build/libpyranda_gpu.so``; nothing is installed elsewhere.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpyranda_gpu.so")
SOURCES = ["pg_setup.cpp", "pg_sweep_f64.cu", "pg_sweep_f32.cu", "pg_sweep_f32_r4.cu", "pg_elem.cu", "pg_capi.cu", "pg_noalloc.cu", "pg_dense.cu", "pg_lad.cu", "pg_split.cu", "pg_seg_r3.cu", "pg_seg_r4.cu", "pg_metric.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpyranda_gpu.so")


def _needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(SRC, s) for s in SOURCES] + [os.path.join(SRC, "pg_internal.h"), os.path.join(SRC, "pg_sweep.cuh"),
                                                      os.path.join(SRC, "pg_split.cuh"), os.path.join(SRC, "pg_tc.cuh"),
                                                      os.path.join(HERE, "..", "include", "pyranda_gpu.h")]
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, verbose):
    obj = os.path.join(OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
           "-I", os.path.join(HERE, "..", "include"), "-c", os.path.join(SRC, src), "-o", obj]
    if src == "pg_metric.cu":  # the metric forms round operation by operation, as the reference's loops
        cmd.insert(1, "-fmad=false")
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose=False):
    """Compile and link the library; returns its path."""
    if not force and not _needs_build():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            sys.stderr.write(err)
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
