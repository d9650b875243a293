"""GPU parity of the native fused solver (include/dg_gb300.h) against the CPU oracle and the
golden fixtures from the reference's own kernels.

Tolerances (relative L2 over all of q or of the RHS):
  * vs the oracle with the solver's affine geometry pushed into it: rounding only
    (FMA contraction, rcp/rsqrt, Shu-Osher stage form, Roe once per face) -> 1e-13 for one
    RHS, 1e-12 after up to 1000 steps;
  * vs the reference build's golden q after 1000 steps on its own mesh: 1e-11, the parity
    target of the port (the reference computes its metrics as Dr*x per node, the solver
    analytically per cell; the difference is inside the target).
"""
import numpy as np
import pytest

from conftest import push_affine_geometry

pytestmark = pytest.mark.gpu


def solver_and_oracle(pkg, orc, oops, m, N, cfl, app=0, phys=None, dt_mode=0, **cfgkw):
    phys = phys or orc.freestream(cfgkw.get("mach", 0.4), cfgkw.get("alpha_deg", 0.0))
    cfg = pkg.config(N=N, app=app, dt_mode=dt_mode, cfl=cfl, vortex_x0=phys["vortex_x0"],
                     vortex_y0=phys["vortex_y0"], vortex_beta=phys["vortex_beta"], **cfgkw)
    s = pkg.Solver(pkg.Mesh.from_tables(m), cfg).init()
    o = orc.Oracle(m, oops.operators(N), phys, app=app, kind="port")
    o.init(cfl)
    push_affine_geometry(o, s.get("geo").reshape(-1, 16))
    return s, o


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_rhs_matches_oracle(pkg, orc, oops, omesh, N):
    m = omesh.naca_ogrid(32, 8, farfield="characteristic")
    s, o = solver_and_oracle(pkg, orc, oops, m, N, 0.5)
    rng = np.random.default_rng(N)
    q = o.get("q")
    W = q * (1.0 + 0.05 * rng.standard_normal(q.size))
    o.set("workingQ", W)
    assert orc.rel_l2(s.rhs(W), o.rhs(0)) < 1e-13


def test_golden_rhs(pkg, orc, golden_naca):
    """One RHS of the reference's perturbed state on its own mesh (reference-computed)."""
    g, m = golden_naca
    s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=4, cfl=1.0)).init()
    rng = np.random.default_rng(int(g["perturb_seed"]))
    q0 = s.get("q")
    W = q0 * (1.0 + 0.05 * rng.standard_normal(q0.size))
    assert orc.rel_l2(s.rhs(W), g["rhs_perturbed"]) < 1e-10


def test_golden_1000_steps(pkg, orc, golden_naca):
    """The headline gate: q after 1000 SSPRK3 steps on the reference's mesh and state,
    against the reference's own kernels, relative L2 <= 1e-11; dt sequence likewise."""
    g, m = golden_naca
    s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=4, cfl=1.0)).init()
    _, dt0, _ = s.time()
    assert abs(dt0 / g["dt0"] - 1) < 1e-10
    s.record_dt(1000)
    s.run(1000)
    s.sync()
    err = orc.rel_l2(s.get("q"), g["q1000"])
    assert err < 1e-11, err
    assert np.abs(s.dt_history(1000) / g["dt1000"] - 1).max() < 1e-9
    t, _, step = s.time()
    assert step == 1000 and abs(t / g["t1000"] - 1) < 1e-10


def test_golden_vortex(pkg, orc, golden_vortex):
    g, m = golden_vortex
    cfg = pkg.config(N=4, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.1, vortex_x0=5.0)
    s = pkg.Solver(pkg.Mesh.from_tables(m), cfg).init()
    assert abs(s.time()[1] / g["dt"] - 1) < 1e-10
    s.run(100)
    s.sync()
    assert orc.rel_l2(s.get("q"), g["q100"]) < 1e-11
    assert np.abs(s.l2_error() / g["l2_100"] - 1).max() < 1e-7


@pytest.mark.parametrize("farfield", ["reference", "characteristic"])
def test_ogrid_steps_match_oracle(pkg, orc, oops, omesh, farfield):
    m = omesh.naca_ogrid(64, 16, farfield=farfield, radius=3.0)
    s, o = solver_and_oracle(pkg, orc, oops, m, 3, 0.5, mach=0.5, alpha_deg=2.0)
    s.record_dt(300)
    s.run(300)
    s.sync()
    dts = o.run(300, nthreads=0)
    assert orc.rel_l2(s.get("q"), o.get("q")) < 1e-12
    assert np.abs(s.dt_history(300) / dts - 1).max() < 1e-12


@pytest.mark.parametrize("N", [1, 2, 4, 5, 6])
def test_steps_every_order_match_oracle(pkg, orc, oops, omesh, N):
    """100 SSPRK3 steps with dt recomputed every step, every order."""
    m = omesh.naca_ogrid(32, 8, farfield="characteristic")
    s, o = solver_and_oracle(pkg, orc, oops, m, N, 0.5, mach=0.45, alpha_deg=1.0)
    s.record_dt(100)
    s.run(100)
    s.sync()
    dts = o.run(100, nthreads=0)
    assert orc.rel_l2(s.get("q"), o.get("q")) < 1e-12
    assert np.abs(s.dt_history(100) / dts - 1).max() < 1e-12


@pytest.mark.parametrize("n", [32, 128])
def test_dt_with_tied_estimates_matches_oracle(pkg, orc, oops, omesh, n):
    """Freestream on a uniform square mesh with inflow boundaries: the calc_dt estimates of the
    nodes on the largest-fscale faces of every cell tie, so the step's finalize evaluates a large
    share of all node-warps in FP64 (n = 128: 32768 cells, the step graph over cell ranges).  The
    dt sequence must equal the oracle's."""
    m = omesh.vortex_square(n)
    s, o = solver_and_oracle(pkg, orc, oops, m, 3, 0.5)
    s.record_dt(5)
    s.run(5)
    s.sync()
    dts = o.run(5, nthreads=0)
    assert np.abs(s.dt_history(5) / dts - 1).max() < 1e-13
    assert orc.rel_l2(s.get("q"), o.get("q")) < 1e-13


def test_vortex_config_matches_oracle(pkg, orc, oops, omesh):
    """The vortex case: [-5,5]^2, 2048 cells, N=3, beta=5, dt = 0.5/dt1 frozen."""
    m = omesh.vortex_square(32)
    phys = orc.freestream(0.4, 0.0)
    phys.update(vortex_x0=0.0, vortex_y0=0.0, vortex_beta=5.0)
    s, o = solver_and_oracle(pkg, orc, oops, m, 3, 0.5, app=1, phys=phys, dt_mode=1)
    s.run(1000)
    s.sync()
    o.run(1000, dt_mode=orc.DT_FROZEN, nthreads=0)
    assert orc.rel_l2(s.get("q"), o.get("q")) < 1e-12
    assert np.abs(s.l2_error() / o.l2_error() - 1).max() < 1e-9


def test_bench_workload_against_oracle(pkg, orc, oops, omesh):
    """The benchmark case itself (K=32768, N=3, characteristic farfield, CFL 0.5)."""
    m = omesh.naca_ogrid(256, 64, farfield="characteristic")
    s, o = solver_and_oracle(pkg, orc, oops, m, 3, 0.5)
    s.run(60)
    s.sync()
    o.run(60, nthreads=0)
    assert orc.rel_l2(s.get("q"), o.get("q")) < 1e-12


def test_freestream_preserved_full_size(pkg):
    """Size-independent property at the largest size: with inflow-only boundaries the
    freestream is a fixed point of the discrete step (to rounding)."""
    mesh = pkg.Mesh.vortex_square(512)
    mesh.set_bedge_type(np.zeros(mesh.size("bedges"), dtype=np.int32))
    s = pkg.Solver(mesh, pkg.config(N=3, cfl=0.5)).init()
    q0 = s.get("q")
    s.run(20)
    s.sync()
    assert np.abs(s.get("q") - q0).max() < 1e-11 * np.abs(q0).max()


def test_deterministic_and_graph_equals_direct(pkg, omesh):
    m = omesh.naca_ogrid(64, 16)
    a = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    b = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    a.run(50)
    for _ in range(50):
        b.step_timed()  # the same step as separate launches
    a.sync()
    b.sync()
    assert np.array_equal(a.get("q"), b.get("q"))


def test_step_host_equals_run(pkg, omesh):
    m = omesh.naca_ogrid(64, 16)
    a = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    b = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    q = a.get("q")
    out = np.empty_like(q)
    a.step_host(q, 5, out)
    b.run(5)
    b.sync()
    assert np.array_equal(out, b.get("q"))


@pytest.mark.parametrize("nsteps", [1, 3])
def test_step_host_pinned_buffers_equal_run(pkg, omesh, nsteps):
    """Pinned host buffers in and out, one and several steps per call."""
    m = omesh.naca_ogrid(64, 16)
    a = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    b = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    q = a.get("q")
    h_in, h_out = pkg.PinnedArray(q.size), pkg.PinnedArray(q.size)
    h_in.array[:] = q
    h_out.array[:] = np.nan
    a.step_host(h_in.array, nsteps, h_out.array)
    b.run(nsteps)
    b.sync()
    assert np.array_equal(h_out.array, b.get("q"))
    assert np.array_equal(a.get("q"), b.get("q")) and a.time() == b.time()


@pytest.mark.parametrize("variant", [0, 1, 2, 3])
@pytest.mark.parametrize("case", ["ogrid_n2", "ogrid_n3", "ogrid_n4", "tiny_n3", "vortex_n3"])
def test_step_host_ranges_equal_run(pkg, omesh, variant, case):
    """The host-buffer call's last step runs its final element kernel as four ranges of cells
    on separate streams, each copied back as soon as it is final: bitwise the graph step, for
    every element-kernel form, with fewer tiles than ranges and with the time-dependent vortex
    boundary."""
    if case == "vortex_n3":
        m = omesh.vortex_square(16)
        cfg = pkg.config(N=3, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.5, vortex_x0=0.0,
                         vortex_y0=0.0, vortex_beta=5.0)
    else:
        m = omesh.naca_ogrid(8, 4) if case == "tiny_n3" else omesh.naca_ogrid(64, 16)
        cfg = pkg.config(N={"ogrid_n4": 4, "ogrid_n2": 2}.get(case, 3), cfl=0.5)
    prev = pkg.lib().dg_elem_variant()
    pkg.lib().dg_set_elem_variant(variant)
    try:
        a = pkg.Solver(pkg.Mesh.from_tables(m), cfg).init()
        b = pkg.Solver(pkg.Mesh.from_tables(m), cfg).init()
        q = a.get("q")
        h_in, h_out = pkg.PinnedArray(q.size), pkg.PinnedArray(q.size)
        h_in.array[:] = q
        h_out.array[:] = np.nan
        for _ in range(3):
            a.step_host(h_in.array, 2, h_out.array)
            h_in.array[:] = h_out.array
        b.run(6)
        b.sync()
        assert np.array_equal(h_out.array, b.get("q"))
        assert np.array_equal(a.get("q"), b.get("q")) and a.time() == b.time()
    finally:
        pkg.lib().dg_set_elem_variant(prev)


def test_nonphysical_state_is_reported(pkg, omesh):
    """Host-side fault injection: a negative density makes the kernel's guard flag fire and
    the host call return DG_ERR_NONPHYSICAL; the context stays usable."""
    m = omesh.naca_ogrid(32, 8)
    s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    q = s.get("q")
    q[0::4][:40] = -1.0
    s.set("q", q)
    s.set("workingQ", q)
    s.run(1)
    with pytest.raises(pkg.DGError) as e:
        s.sync()
    assert e.value.code == pkg.ERR_NONPHYSICAL
    t = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=3, cfl=0.5)).init()
    t.run(2)
    t.sync()


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_even_odd_form_equals_dense_form(pkg, orc, omesh, N):
    """The element-kernel forms compute the same RHS and steps: dense FP64 rows (0), the even/odd
    split in FP64 (1), the even/odd split with the tensor-core contraction (2; used at N = 3, 4,
    5, FP64 at the other orders) and form 3 (the default: the dense rows on the tensor cores at
    N = 1, 2, form 2 at the other orders)."""
    m = omesh.naca_ogrid(32, 8, farfield="characteristic")
    out = []
    prev = pkg.lib().dg_elem_variant()
    assert prev == 3
    for variant in (0, 1, 2, 3):
        pkg.lib().dg_set_elem_variant(variant)
        try:
            s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=N, cfl=0.5)).init()
            q = s.get("q")
            W = q * (1.0 + 0.05 * np.random.default_rng(N).standard_normal(q.size))
            r = s.rhs(W)
            s.run(20)
            s.sync()
            out.append((r, s.get("q")))
        finally:
            pkg.lib().dg_set_elem_variant(prev)
    for k in (1, 2, 3):
        assert orc.rel_l2(out[k][0], out[0][0]) < 1e-13
        assert orc.rel_l2(out[k][1], out[0][1]) < 1e-13
    if N not in (3, 4, 5):
        assert np.array_equal(out[2][0], out[1][0])  # form 2 is form 1 at the other orders
    if N >= 3:
        assert np.array_equal(out[3][0], out[2][0])  # form 3 is form 2 from N = 3 on
        assert np.array_equal(out[3][1], out[2][1])
    else:
        assert not np.array_equal(out[3][0], out[1][0])  # the dense tensor-core rows ran


def _rhs_forms(pkg, m, W, N=3, tc_variant=2):
    out = []
    prev = pkg.lib().dg_elem_variant()
    for variant in (1, tc_variant):
        pkg.lib().dg_set_elem_variant(variant)
        try:
            s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=N, cfl=0.5)).init()
            out.append(s.rhs(W))
        finally:
            pkg.lib().dg_set_elem_variant(prev)
    return out


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_tensor_core_contraction_wide_range(pkg, omesh, N):
    """Cells whose states differ by up to 1e6 in scale (each cell's state scaled as a whole, so
    it stays physical): the tensor-core contraction scales every column by its own largest
    exponent, and agrees with the FP64 contraction to rounding."""
    m = omesh.naca_ogrid(32, 8, farfield="characteristic")
    s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=N, cfl=0.5)).init()
    q = s.get("q").reshape(m["cell2nodes"].shape[0], -1)
    lam = 10.0 ** np.random.default_rng(7).uniform(-3, 3, q.shape[0])
    W = (q * lam[:, None]).ravel()
    r1, r2 = _rhs_forms(pkg, m, W, N, tc_variant=3 if N <= 2 else 2)
    assert np.all(np.isfinite(r2))
    assert np.linalg.norm(r2 - r1) <= 1e-13 * np.linalg.norm(r1)
    # entrywise: near the wall the staged fluxes are ~1e3-1e4 and cancel to an O(1) RHS, so
    # both contractions carry ~1e-12 absolute rounding there
    assert np.abs(r2 - r1).max() <= 1e-11 * np.abs(r1).max()


@pytest.mark.parametrize("N", [2, 3, 4, 5])
def test_tensor_core_contraction_nonfinite(pkg, omesh, N):
    """A non-finite value in a cell's staged column gives NaN there, as the FP64 contraction
    does, and leaves the cells it does not reach finite (the dense rows at N = 2, the even/odd
    blocks with their integer-prepared operands at N = 3, 4, 5)."""
    m = omesh.naca_ogrid(32, 8, farfield="characteristic")
    s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=N, cfl=0.5)).init()
    q = s.get("q")
    nc = 2 * (N + 1) * (N + 2)  # doubles per cell
    W = q * (1.0 + 0.05 * np.random.default_rng(3).standard_normal(q.size))
    W[nc * 17 + 5] = np.nan
    r1, r2 = _rhs_forms(pkg, m, W, N, tc_variant=3 if N <= 2 else 2)
    assert np.isnan(r2).any()
    assert np.array_equal(np.isnan(r1.reshape(-1, nc)).any(1), np.isnan(r2.reshape(-1, nc)).any(1))
    ok = ~np.isnan(r1)
    assert np.linalg.norm(r2[ok] - r1[ok]) <= 1e-13 * np.linalg.norm(r1[ok])
    assert np.abs(r2[ok] - r1[ok]).max() <= 1e-11 * np.abs(r1[ok]).max()


@pytest.mark.parametrize("N", [3, 4])
def test_programmatic_launch_equals_stream_order(pkg, omesh, N):
    """Face and element kernels launched with programmatic dependent launch (default) compute
    exactly what plain stream-ordered launches compute, in graphs and direct launches."""
    m = omesh.naca_ogrid(64, 16, farfield="characteristic")
    res = []
    for pdl in (0, 1):
        pkg.lib().dg_set_pdl(pdl)
        try:
            s = pkg.Solver(pkg.Mesh.from_tables(m), pkg.config(N=N, cfl=0.5)).init()
            q = s.get("q")
            r = s.rhs(q * (1.0 + 0.05 * np.random.default_rng(N).standard_normal(q.size)))
            s.run(40)
            for _ in range(5):
                s.step_timed()
            s.sync()
            res.append((r, s.get("q"), s.time()))
        finally:
            pkg.lib().dg_set_pdl(1)
    assert np.array_equal(res[0][0], res[1][0])
    assert np.array_equal(res[0][1], res[1][1])
    assert res[0][2] == res[1][2]


@pytest.mark.parametrize("cells", [[[0, 1, 2]], [[0, 1, 2], [0, 2, 3]]])
def test_tiny_meshes_match_oracle(pkg, orc, oops, omesh, cells):
    """One and two cells (every face, or all but one, on the boundary; grids of one block)."""
    coords = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])[: max(max(c) for c in cells) + 1]
    m = omesh.build_tables(coords, np.array(cells, dtype=np.int32))
    m["bedge_type"] = np.array([2, 0, 1, 2][: len(m["bedge2cell"])], dtype=np.int32)
    s, o = solver_and_oracle(pkg, orc, oops, m, 3, 0.3, mach=0.3, alpha_deg=5.0)
    s.record_dt(10)
    s.run(10)
    s.sync()
    dts = o.run(10, nthreads=1)
    assert orc.rel_l2(s.get("q"), o.get("q")) < 1e-12
    assert np.abs(s.dt_history(10) / dts - 1).max() < 1e-12
