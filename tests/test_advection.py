"""The scalar advection app (advec/src/advec.cpp): the oracle against the reference's own
advection kernels and the golden fixture (CPU), and the device path (include/dg_gb300.h,
dg_advec_*) against both (GPU).

Tolerances (relative L2):
  * oracle port vs the reference build with the reference's tables: bit-identical;
  * oracle port with generated tables vs the golden fixture: 1e-12 (table rounding);
  * device vs the oracle with the device's affine geometry pushed in: 1e-13 for one RHS,
    1e-12 after 200 steps (FMA contraction, flux once per face node, metric order);
  * device vs the golden fixture on the reference's mesh: 1e-11."""
import os

import numpy as np
import pytest

from conftest import REFERENCE_TREE, reference_tables


def perturbed(q, seed, amp):
    return q * (1.0 + amp * np.random.default_rng(seed).standard_normal(q.size))


def push_geometry(o, geo):
    """The device's per-cell affine metrics and face normals into the oracle's per-node dats."""
    geo = geo.reshape(-1, 16)
    Np, Nfp = o.Np, o.Nfp
    for j, name in enumerate(("rx", "ry", "sx", "sy")):
        o.set(name, np.repeat(geo[:, j], Np))
    for j, name in enumerate(("nx", "ny", "fscale")):
        o.set(name, np.repeat(geo[:, [4 + j, 7 + j, 10 + j]], Nfp, axis=1).ravel())


def test_oracle_matches_golden(orc, oops, golden_advec):
    g, m = golden_advec
    a = orc.Advection(m, oops.operators(4))
    a.init(float(g["dt"]))
    q0 = a.get("q")
    a.set("workingQ", perturbed(q0, int(g["perturb_seed"]), float(g["perturb_amp"])))
    assert orc.rel_l2(a.rhs(0), g["rhs_perturbed"]) < 1e-12
    a.set("workingQ", q0)
    a.run(100)
    assert orc.rel_l2(a.get("q"), g["q100"]) < 1e-12
    assert a.t == g["t100"]
    assert g["q100_dropped"] < 1e-15 and g["rhs_perturbed_dropped"] < 1e-15


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree absent")
def test_oracle_bit_exact_vs_reference_build(orc, oops, omesh):
    orc.build(ref=True)
    coords, cells = omesh.read_vtk(os.path.join(REFERENCE_TREE, "advec", "grid.vtk"))
    m = omesh.build_tables(coords, cells)
    ops = dict(oops.operators(4))
    ops.update(reference_tables())
    for vel in ((1.0, 1.0), (0.7, -0.3)):
        a = orc.Advection(m, ops, *vel, kind="port")
        b = orc.Advection(m, ops, *vel, kind="reference")
        a.init(2e-3)
        b.init(2e-3)
        for s in range(4):
            assert np.array_equal(a.rhs(s), b.rhs(s))
        a.run(20, nthreads=4)
        b.run(20, nthreads=1)
        assert np.array_equal(a.get("q"), b.get("q"))


def test_oracle_order_independent(orc, oops, omesh):
    """Single-writer face slots: the thread count changes nothing."""
    m = omesh.vortex_square(24, 0.0, 2.0)
    out = []
    for nt in (1, 3):
        a = orc.Advection(m, oops.operators(3), 1.0, 0.5)
        a.init(1e-3)
        a.run(10, nthreads=nt)
        out.append(a.get("q"))
    assert np.array_equal(out[0], out[1])


def test_create_rejects_bad_arguments(pkg, omesh):
    mesh = pkg.Mesh.from_tables(omesh.naca_ogrid(16, 4))
    for kw in (dict(N=0), dict(N=7), dict(dt=0.0), dict(dt=-1.0), dict(vel_x=float("nan"))):
        with pytest.raises(pkg.DGError):
            pkg.Advection(mesh, **kw)


# ---------------------------------------------------------------- GPU
def device_and_oracle(pkg, orc, oops, m, N, vel=(1.0, 1.0), dt=1e-3):
    a = pkg.Advection(pkg.Mesh.from_tables(m), N=N, vel_x=vel[0], vel_y=vel[1], dt=dt).init()
    o = orc.Advection(m, oops.operators(N), *vel)
    o.init(dt)
    push_geometry(o, a.get("geo"))
    return a, o


@pytest.mark.gpu
@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_device_rhs_matches_oracle(pkg, orc, oops, omesh, N):
    m = omesh.vortex_square(16, 0.0, 1.0)
    a, o = device_and_oracle(pkg, orc, oops, m, N, vel=(0.8, -0.45))
    q = o.get("q")
    assert orc.rel_l2(a.get("q"), q) < 1e-14
    W = perturbed(q, N, 0.5)
    o.set("workingQ", W)
    assert orc.rel_l2(a.rhs(W), o.rhs(0)) < 1e-13


@pytest.mark.gpu
@pytest.mark.parametrize("N", [2, 4])
def test_device_steps_match_oracle(pkg, orc, oops, omesh, N):
    m = omesh.vortex_square(20, 0.0, 1.5)
    a, o = device_and_oracle(pkg, orc, oops, m, N, vel=(1.0, 0.6), dt=5e-4)
    a.run(200)
    a.sync()
    o.run(200)
    assert orc.rel_l2(a.get("q"), o.get("q")) < 1e-12
    t, k = a.time()
    assert k == 200 and t == o.t


@pytest.mark.gpu
def test_device_golden(pkg, orc, golden_advec):
    g, m = golden_advec
    a = pkg.Advection(pkg.Mesh.from_tables(m), N=4, vel_x=1.0, vel_y=1.0, dt=float(g["dt"])).init()
    q0 = a.get("q")
    r = a.rhs(perturbed(q0, int(g["perturb_seed"]), float(g["perturb_amp"])))
    assert orc.rel_l2(r, g["rhs_perturbed"]) < 1e-11
    a.set("workingQ", q0)
    a.run(100)
    a.sync()
    assert orc.rel_l2(a.get("q"), g["q100"]) < 1e-11
    assert a.time()[0] == g["t100"]


@pytest.mark.gpu
def test_device_graph_equals_separate_launches(pkg, omesh):
    m = omesh.vortex_square(24, 0.0, 1.0)
    a = pkg.Advection(pkg.Mesh.from_tables(m), N=3).init()
    b = pkg.Advection(pkg.Mesh.from_tables(m), N=3).init()
    a.run(30)
    for _ in range(30):
        assert len(b.step_timed()) == 8
    a.sync()
    assert np.array_equal(a.get("q"), b.get("q"))


@pytest.mark.gpu
def test_device_vertex_values_and_vtk(pkg, orc, omesh, tmp_path):
    """advec/src/save_solution.cpp:13-52: q at each vertex from the last cell containing it."""
    m = omesh.vortex_square(16, 0.0, 1.0)
    mesh = pkg.Mesh.from_tables(m)
    a = pkg.Advection(mesh, N=3).init()
    a.run(10)
    a.sync()
    q = a.get("q").reshape(len(m["cell2nodes"]), -1)
    want = np.zeros(len(m["coords"]))
    for c, tri in enumerate(m["cell2nodes"]):
        want[tri] = q[c, [0, 3, q.shape[1] - 1]]
    assert np.array_equal(a.vertex_values(), want)
    a.write_vtk(tmp_path / "advec.vtk")
    assert np.array_equal(orc.read_vtk_point_data(tmp_path / "advec.vtk")["q"], want)


@pytest.mark.gpu
@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_device_even_odd_equals_dense(pkg, orc, omesh, N):
    """The element-kernel forms: dense FP64 (0), even/odd FP64 (1) and the default (3: the
    even/odd contraction on the tensor cores at N = 3, form 1 at the other orders) give the same
    RHS and steps."""
    m = omesh.vortex_square(12, 0.0, 1.0)
    out = []
    prev = pkg.lib().dg_elem_variant()
    for variant in (0, 1, 3):
        pkg.lib().dg_set_elem_variant(variant)
        try:
            a = pkg.Advection(pkg.Mesh.from_tables(m), N=N, vel_x=0.9, vel_y=-0.4).init()
            q = a.get("q")
            r = a.rhs(perturbed(q, N, 0.5))
            a.set("workingQ", q)
            a.run(15)
            a.sync()
            out.append((r, a.get("q")))
        finally:
            pkg.lib().dg_set_elem_variant(prev)
    for k in (1, 2):
        assert orc.rel_l2(out[k][0], out[0][0]) < 1e-13
        assert orc.rel_l2(out[k][1], out[0][1]) < 1e-13
    if N == 3:
        assert not np.array_equal(out[2][0], out[1][0])  # the tensor-core kernel ran
    else:
        assert np.array_equal(out[2][0], out[1][0])
