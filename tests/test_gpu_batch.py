"""The batched persistent-kernel path (dg_batch_*): every instance must compute exactly what its
own plain solver computes (same device functions, same operation order, one writer per face
slot, order-independent dt maximum) — bitwise, before and after autotuning, for mixed orders
and mixed airfoil / vortex instances."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def instances(pkg):
    specs = [
        (pkg.Mesh.naca_ogrid(48, 12), pkg.config(N=3, cfl=0.5, mach=0.45, alpha_deg=2.0)),
        (pkg.Mesh.naca_ogrid(64, 16, farfield="reference"), pkg.config(N=4, cfl=0.5, mach=0.35, alpha_deg=-3.0)),
        (pkg.Mesh.vortex_square(12), pkg.config(N=3, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.5,
                                                vortex_x0=0.0)),
        (pkg.Mesh.naca_ogrid(32, 8), pkg.config(N=2, cfl=0.5)),
        (pkg.Mesh.naca_ogrid(40, 10), pkg.config(N=4, cfl=0.4, mach=0.55)),
    ]
    return [m for m, _ in specs], [c for _, c in specs]


def plain(pkg, meshes, cfgs, steps):
    out = []
    for m, c in zip(meshes, cfgs):
        s = pkg.Solver(m, c).init()
        s.run(steps)
        s.sync()
        out.append((s.get("q"), s.time()))
    return out


def test_batch_equals_plain_solvers(pkg):
    meshes, cfgs = instances(pkg)
    ref = plain(pkg, meshes, cfgs, 25)
    b = pkg.Batch(meshes, cfgs).init()
    b.run(25)
    b.sync()
    assert b.shape()["graph"]  # the step runs as one graph launch
    for k in range(len(cfgs)):
        assert np.array_equal(b.get(k, "q"), ref[k][0]), k
        assert b.time(k) == ref[k][1], k


def test_batch_autotuned_equals_plain(pkg):
    meshes, cfgs = instances(pkg)
    ref = plain(pkg, meshes, cfgs, 12)
    b = pkg.Batch(meshes, cfgs).init()
    ms = b.autotune(steps=2)
    assert ms > 0
    sh = b.shape()
    assert sh["block"] >= 32 * 15 and sh["grid"] > 0
    b.run(12)
    b.sync()
    for k in range(len(cfgs)):
        assert np.array_equal(b.get(k, "q"), ref[k][0]), k


@pytest.mark.parametrize("shape", [(0, 512), (2, 2048), (99, 64), (99, 256)])
def test_batch_every_shape_equals_plain(pkg, shape):
    """Persistent-kernel variants and the grouped launches: bitwise the plain solvers' results."""
    meshes, cfgs = instances(pkg)
    ref = plain(pkg, meshes, cfgs, 10)
    b = pkg.Batch(meshes, cfgs).init()
    b.use_shape(*shape)
    b.run(10)
    b.sync()
    sh = b.shape()
    assert sh["variant"] == shape[0] and sh["graph"]
    for k in range(len(cfgs)):
        assert np.array_equal(b.get(k, "q"), ref[k][0]), k


@pytest.mark.parametrize("shape", [(0, 512), (99, 64)])
def test_batch_tied_dt_estimates_equal_plain(pkg, shape):
    """Freestream on uniform square meshes with inflow boundaries (dt recomputed every step): the
    calc_dt estimates of every cell tie, so the batched finalize evaluates a large share of each
    instance's node-warps in FP64 over several blocks per instance.  Bitwise the plain solvers'
    q, time and dt."""
    meshes, cfgs = [], []
    for n, N in ((24, 3), (16, 4), (32, 3)):
        m = pkg.Mesh.vortex_square(n)
        m.set_bedge_type(np.zeros(m.size("bedges"), dtype=np.int32))
        meshes.append(m)
        cfgs.append(pkg.config(N=N, cfl=0.5, mach=0.4))
    ref = plain(pkg, meshes, cfgs, 6)
    b = pkg.Batch(meshes, cfgs).init()
    b.use_shape(*shape)
    b.run(6)
    b.sync()
    for k in range(len(cfgs)):
        assert np.array_equal(b.get(k, "q"), ref[k][0]), k
        assert b.time(k) == ref[k][1], k


def test_batch_reports_nonphysical(pkg):
    meshes, cfgs = instances(pkg)
    b = pkg.Batch(meshes[:2], cfgs[:2]).init()
    b.run(1)
    b.sync()
    bad = pkg.Batch([pkg.Mesh.naca_ogrid(32, 8)], [pkg.config(N=3, cfl=50.0)]).init()
    bad.run(40)
    with pytest.raises(pkg.DGError):
        bad.sync()


def test_batch_reports_barrier_timeout(pkg):
    """Host-side injection of a timed-out grid barrier (no kernel is made to wait): sync reports
    DG_ERR_TIMEOUT once, then the batch runs on."""
    meshes, cfgs = instances(pkg)
    b = pkg.Batch(meshes[:2], cfgs[:2]).init()
    b.run(2)
    b.sync()
    pkg.lib().dg_batch_inject_barrier_timeout(b.h)
    with pytest.raises(pkg.DGError) as e:
        b.sync()
    assert e.value.code == pkg.ERR_TIMEOUT
    b.init()
    b.run(2)
    b.sync()


def test_batch_barrier_wait_runs_out_on_device(pkg):
    """The grid barrier's bounded wait, on the device: with a limit of 20,000 SM clocks (~10 us)
    and block 0 held back 4,000,000 clocks (~2 ms, a bounded delay) the other blocks' waits run
    out, they record the timeout and return, block 0 then completes the barrier alone, and sync
    reports DG_ERR_TIMEOUT.  Without the hold the same launch completes normally, and the batch
    steps on afterwards with the default limit."""
    meshes, cfgs = instances(pkg)
    b = pkg.Batch(meshes[:2], cfgs[:2]).init()
    lib = pkg.lib()
    assert lib.dg_batch_barrier_check(b.h, 0) == 0
    b.sync()  # no hold: completes
    assert lib.dg_batch_set_barrier_limit(b.h, 20000) == 0
    assert lib.dg_batch_barrier_check(b.h, 4000000) == 0
    with pytest.raises(pkg.DGError) as e:
        b.sync()
    assert e.value.code == pkg.ERR_TIMEOUT
    assert lib.dg_batch_barrier_check(b.h, 1 << 41) != 0  # beyond the longest hold: refused
    assert lib.dg_batch_set_barrier_limit(b.h, 0) == 0
    b.init()
    b.run(2)
    b.sync()
