"""The OP2 drop-in from C++ (tests/cpp/dropin_airfoil.cpp): a compiled application passes op_arg
by value to the op_par_loop_<kernel> functions, as the reference's translated driver does.
CPU: the driver compiles and links against include/op2_gb300.h and the library.  GPU: its q and
dt sequence after 10 steps equal the oracle's bit for bit."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "dropin_airfoil.cpp")


def compile_driver(pkg, out_dir):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    lib_dir = os.path.dirname(pkg.LIB_PATH)
    exe = os.path.join(str(out_dir), "dropin_airfoil")
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), SRC, "-L", lib_dir,
                    "-ldg_gb300", "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    return exe


def test_driver_compiles_and_links(pkg, tmp_path):
    assert os.path.exists(compile_driver(pkg, tmp_path))


def write_input(path, m, ops, phys, iters):
    N = int(ops["N"])
    with open(path, "wb") as f:
        np.array([len(m["coords"]), len(m["cell2nodes"]), len(m["edge2cells"]), len(m["bedge2cell"]), N, iters],
                 dtype=np.int32).tofile(f)
        np.asarray(m["coords"], dtype=np.float64).tofile(f)
        for k in ("cell2nodes", "edge2cells", "edgeNum", "bedge2cell", "bedgeNum", "bedge_type"):
            np.asarray(m[k], dtype=np.int32).tofile(f)
        np.array([phys[k] for k in ("gam", "bc_mach", "bc_alpha", "bc_p", "bc_r", "bc_u", "bc_v", "bc_e")]).tofile(f)
        for k in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT"):
            np.asarray(ops[k], dtype=np.float64).ravel().tofile(f)
        np.asarray(ops["FMASK"], dtype=np.int32).tofile(f)


@pytest.mark.gpu
@pytest.mark.parametrize("N", [3, 4])
def test_cpp_driver_bitwise_equals_oracle(pkg, orc, oops, omesh, tmp_path, N):
    exe = compile_driver(pkg, tmp_path)
    m = omesh.naca_ogrid(48, 12, farfield="reference")
    ops, phys = oops.operators(N), orc.freestream(0.45, -1.0)
    iters = 10
    write_input(tmp_path / "in.bin", m, ops, phys, iters)
    r = subprocess.run([exe, str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    K, Np = len(m["cell2nodes"]), (N + 1) * (N + 2) // 2
    out = np.fromfile(tmp_path / "out.bin", dtype=np.float64)
    q, dts = out[:K * Np * 4], out[K * Np * 4:]
    o = orc.Oracle(m, ops, phys, kind="port")
    o.init(1.0)
    dto = o.run(iters, nthreads=1)
    assert np.array_equal(dts, dto)
    assert np.array_equal(q, o.get("q"))
    assert "euler_rhs" in r.stdout  # op_timing_output lists the loops
