"""Build the in-tree shared library falcon_gb300/_lib/libfalcon_gb300.so.

nvcc compiles every CUDA translation unit for sm_103a only; the FP64 kernels get
-fmad=false so no multiply-add is contracted (bit-comparable with the CPU
oracle). Host C++ is compiled with -ffp-contract=off for the same reason: the
block geometry and the ghost map must match the reference bit for bit, and gcc
on aarch64 contracts by default. Translation units build in parallel.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(OUT_DIR, "obj")
LIB = os.path.join(OUT_DIR, "libfalcon_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
HOST_FLAGS = "-fPIC,-fopenmp,-ffp-contract=off,-fno-fast-math"

# (source, extra nvcc flags)
UNITS = [
    ("mhd_fp64.cu", ["-fmad=false"]),
    ("mhd_mixed.cu", []),
    ("synth.cu", []),
    ("capi.cu", []),
    ("state_range.cu", []),
    ("output.cu", ["-fmad=false"]),
    ("host_setup.cpp", []),
    ("solver.cu", ["-fmad=false"]),
    ("solver_host.cpp", []),
    ("lcc.cu", []),
]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _deps():
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [
        os.path.join(HERE, "..", "include", "falcon_gb300.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(unit):
    src, extra = unit
    obj = os.path.join(OBJ_DIR, os.path.splitext(src)[0] + ".o")
    if src.endswith(".cpp"):
        cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               "-c", os.path.join(CSRC, src), "-o", obj]
    else:
        cmd = [nvcc(), "-std=c++17", *ARCH, "-lineinfo", "-O3", *extra, "-Xcompiler", HOST_FLAGS,
               "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj


def build(force=False, verbose=False):
    """Compile (if stale) and return the path of the shared library."""
    deps = _deps()
    if not force and not _stale(LIB, deps):
        return LIB
    os.makedirs(OBJ_DIR, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(_compile, UNITS))
    cmd = [nvcc(), *ARCH, "-shared", "-o", LIB + ".tmp", *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
