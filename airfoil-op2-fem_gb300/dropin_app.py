"""Build and run the C++ application of the OP2 drop-in (apps/dropin_airfoil.cpp): the
reference's airfoil main loop (src/airfoil.cpp:135-334) compiled against include/op2_gb300.h
and linked with libdg_gb300.so, as a user of the drop-in builds it.

    exe = compile_app(out_dir)
    q, dts, timing = run_app(exe, mesh_tables, operators, freestream, iters, work_dir)
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "apps", "dropin_airfoil.cpp")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
PHYS_KEYS = ("gam", "bc_mach", "bc_alpha", "bc_p", "bc_r", "bc_u", "bc_v", "bc_e")


def compile_app(out_dir, lib_path):
    """g++ the application against the headers and the built library; returns the executable."""
    if not shutil.which("g++"):
        raise RuntimeError("g++ not available")
    lib_dir = os.path.dirname(lib_path)
    exe = os.path.join(str(out_dir), "dropin_airfoil")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-I", INCLUDE, SRC, "-L", lib_dir, "-ldg_gb300",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    return exe


def write_input(path, m, ops, phys, iters):
    """The application's input file: counts, mesh tables, freestream constants, operators."""
    N = int(ops["N"])
    with open(path, "wb") as f:
        np.array([len(m["coords"]), len(m["cell2nodes"]), len(m["edge2cells"]), len(m["bedge2cell"]), N, iters],
                 dtype=np.int32).tofile(f)
        np.asarray(m["coords"], dtype=np.float64).tofile(f)
        for k in ("cell2nodes", "edge2cells", "edgeNum", "bedge2cell", "bedgeNum", "bedge_type"):
            np.asarray(m[k], dtype=np.int32).tofile(f)
        np.array([phys[k] for k in PHYS_KEYS], dtype=np.float64).tofile(f)
        for k in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT"):
            np.asarray(ops[k], dtype=np.float64).ravel().tofile(f)
        np.asarray(ops["FMASK"], dtype=np.int32).tofile(f)


def run_app(exe, m, ops, phys, iters, work_dir):
    """Run the application; returns (q, dt sequence, timing dict, stdout)."""
    inp, out = os.path.join(str(work_dir), "in.bin"), os.path.join(str(work_dir), "out.bin")
    write_input(inp, m, ops, phys, iters)
    r = subprocess.run([exe, inp, out], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("dropin_airfoil failed (%d): %s" % (r.returncode, r.stderr))
    N = int(ops["N"])
    K, Np = len(m["cell2nodes"]), (N + 1) * (N + 2) // 2
    data = np.fromfile(out, dtype=np.float64)
    timing = {}
    mt = re.search(r"dropin_timing total_s=([0-9.eE+-]+) steps_s=([0-9.eE+-]+)", r.stdout)
    if mt:
        timing = {"total_s": float(mt.group(1)), "steps_s": float(mt.group(2))}
    return data[:K * Np * 4], data[K * Np * 4:], timing, r.stdout
