"""Build the in-tree shared library lib/libdg_gb300.so for sm_103a.

Each translation unit in csrc/ is compiled in parallel (nvcc for .cu, g++ for
.cpp) and linked with nvcc.  The OP2 drop-in kernels (op2_kernels.cu) are
compiled with --fmad=false so that they keep the reference's rounding; the
native kernels use FMA contraction freely.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libdg_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

GENCODE = "-gencode=arch=compute_103a,code=sm_103a"
# Host code must give the same results on x86 and Arm: no FMA contraction on the host side.
NVCC_FLAGS = ["-O3", "-std=c++17", GENCODE, "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", CSRC, "-I", INCLUDE]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I", CSRC, "-I", INCLUDE]
# TUs that must not contract a*b+c into fma: they restate the reference's rounding.
NO_FMAD = {"op2_kernels.cu"}


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_include():
    return os.path.join(os.path.dirname(os.path.dirname(_nvcc())), "include")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src):
    path = os.path.join(CSRC, src)
    obj = os.path.join(OBJ, src + ".o")
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps + [path]):
        return obj, ""
    if src.endswith(".cu"):
        cmd = [_nvcc()] + NVCC_FLAGS + (["--fmad=false"] if src in NO_FMAD else []) + ["-c", path, "-o", obj]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-I", _cuda_include(), "-c", path, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(_compile, srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, log in results:
            if log.strip():
                print(o, log)
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [_nvcc(), "-shared", GENCODE, "-o", LIB] + objs  # cudart linked statically
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
