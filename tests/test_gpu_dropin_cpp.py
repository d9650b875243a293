"""The OP2 drop-in from C++ (airfoil-op2-fem_gb300/apps/dropin_airfoil.cpp): a compiled
application passes op_arg by value to the op_par_loop_<kernel> functions, as the reference's
translated driver does.  CPU: the application compiles and links against include/op2_gb300.h
and the library.  GPU: its q and dt sequence after 10 steps equal the oracle's bit for bit."""
import importlib
import shutil

import numpy as np
import pytest


@pytest.fixture(scope="module")
def app(pkg):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    return importlib.import_module(pkg.__name__ + ".dropin_app")


def test_driver_compiles_and_links(pkg, app, tmp_path):
    import os
    assert os.path.exists(app.compile_app(tmp_path, pkg.LIB_PATH))


@pytest.mark.gpu
@pytest.mark.parametrize("N", [3, 4])
def test_cpp_driver_bitwise_equals_oracle(pkg, app, orc, oops, omesh, tmp_path, N):
    exe = app.compile_app(tmp_path, pkg.LIB_PATH)
    m = omesh.naca_ogrid(48, 12, farfield="reference")
    ops, phys = oops.operators(N), orc.freestream(0.45, -1.0)
    iters = 10
    q, dts, timing, stdout = app.run_app(exe, m, ops, phys, iters, tmp_path)
    o = orc.Oracle(m, ops, phys, kind="port")
    o.init(1.0)
    dto = o.run(iters, nthreads=1)
    assert np.array_equal(dts, dto)
    assert np.array_equal(q, o.get("q"))
    assert "euler_rhs" in stdout  # op_timing_output lists the loops
    assert timing["total_s"] > timing["steps_s"] > 0.0
