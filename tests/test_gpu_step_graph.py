"""The step graph over cell ranges (dg_set_step_parts): the face and element launches of P
ranges of cells, each depending only on the launches that share its cells, so that ranges of
different stages overlap.  Every launch computes what the single-range step computes for its
faces and tiles, so q, the dt sequence and the time must be bitwise the same for every P,
including on a mesh whose cell numbering has no locality (every range then depends on every
other one) and for the vortex app (its boundary state reads the stage time)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def run_parts(pkg, mesh, cfg, parts, steps):
    pkg.set_step_parts(parts)
    try:
        s = pkg.Solver(mesh, cfg).init()
        s.record_dt(steps)
        s.run(steps)
        s.sync()
        return s.get("q"), s.dt_history(steps), s.time(), s.kernels_per_step()
    finally:
        pkg.set_step_parts(0)


def shuffled(m, seed):
    """The same mesh with its cells renumbered at random (every table mapped through the
    permutation; edge order and boundary types kept)."""
    rng = np.random.default_rng(seed)
    K = m["cell2nodes"].shape[0]
    new_of_old = rng.permutation(K).astype(np.int32)
    out = dict(m)
    c2n = np.empty_like(m["cell2nodes"])
    c2n[new_of_old] = m["cell2nodes"]
    out["cell2nodes"] = c2n
    out["edge2cells"] = new_of_old[m["edge2cells"]]
    out["bedge2cell"] = new_of_old[m["bedge2cell"]]
    return out


@pytest.mark.parametrize("flags", [0, 1, 2, 3, 5])
def test_graph_flags_bitwise_equal(pkg, flags):
    """With and without programmatic dependent launch between the ranges' kernels, with and
    without per-range priorities: the same bits."""
    mesh = pkg.Mesh.naca_ogrid(96, 24, farfield="characteristic")
    cfg = pkg.config(N=3, cfl=0.5, mach=0.5, alpha_deg=2.0)
    q1, dt1, _, _ = run_parts(pkg, mesh, cfg, 1, 20)
    prev = pkg.lib().dg_step_graph_flags()
    pkg.lib().dg_set_step_graph_flags(flags)
    try:
        q, dt, _, _ = run_parts(pkg, mesh, cfg, 4, 20)
    finally:
        pkg.lib().dg_set_step_graph_flags(prev)
    assert np.array_equal(q, q1) and np.array_equal(dt, dt1)


@pytest.mark.parametrize("N", [3, 4])
def test_parts_bitwise_equal_airfoil(pkg, omesh, N):
    mesh = pkg.Mesh.naca_ogrid(128, 32, farfield="characteristic")
    cfg = pkg.config(N=N, cfl=0.5, mach=0.5, alpha_deg=2.0)
    q1, dt1, t1, k1 = run_parts(pkg, mesh, cfg, 1, 40)
    assert k1 == 7
    for P in (2, 3, 8):
        q, dt, t, k = run_parts(pkg, mesh, cfg, P, 40)
        assert k == 6 * P + 1
        assert np.array_equal(q, q1) and np.array_equal(dt, dt1) and t == t1, P


def test_parts_bitwise_equal_unordered_cells(pkg, omesh):
    m = omesh.naca_ogrid(96, 24, farfield="characteristic")
    mesh = pkg.Mesh.from_tables(shuffled(m, 3))
    cfg = pkg.config(N=3, cfl=0.5, mach=0.45, alpha_deg=-1.0)
    q1, dt1, t1, _ = run_parts(pkg, mesh, cfg, 1, 30)
    for P in (4, 9):
        q, dt, t, _ = run_parts(pkg, mesh, cfg, P, 30)
        assert np.array_equal(q, q1) and np.array_equal(dt, dt1) and t == t1, P


def test_parts_bitwise_equal_vortex(pkg):
    mesh = pkg.Mesh.vortex_square(64)
    cfg = pkg.config(N=3, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.5, vortex_x0=0.0, vortex_y0=0.0,
                     vortex_beta=5.0)
    q1, _, t1, _ = run_parts(pkg, mesh, cfg, 1, 50)
    for P in (2, 5):
        q, _, t, _ = run_parts(pkg, mesh, cfg, P, 50)
        assert np.array_equal(q, q1) and t == t1, P


def test_parts_setting(pkg):
    """0 (automatic) by default; out-of-range values fall back to it; the automatic choice
    takes ranges of at least 128 tiles, at most 4."""
    lib = pkg.lib()
    assert pkg.step_parts() == 0
    for v in (-1, 33, 1000):
        pkg.set_step_parts(v)
        assert pkg.step_parts() == 0
    pkg.set_step_parts(0)
    small = pkg.Solver(pkg.Mesh.naca_ogrid(32, 8), pkg.config(N=3)).init()
    assert small.kernels_per_step() == 7
    big = pkg.Solver(pkg.Mesh.naca_ogrid(256, 64), pkg.config(N=3)).init()
    assert big.kernels_per_step() == 6 * 4 + 1
    assert lib.dg_step_parts() == 0


@pytest.mark.parametrize("nsteps", [1, 3])
@pytest.mark.parametrize("pinned", [True, False])
def test_step_host_over_ranges_equals_run(pkg, nsteps, pinned):
    """The host-buffer call over cell ranges (each range uploaded before its first face launch,
    downloaded after its last element launch, in one captured graph; pageable buffers take the
    single-range path): bitwise the same as run(), on two calls with the same buffers (the second
    reuses the graph) and one with new buffers (a new graph)."""
    mesh = pkg.Mesh.naca_ogrid(96, 24, farfield="characteristic")
    cfg = pkg.config(N=3, cfl=0.5, mach=0.45, alpha_deg=1.0)
    pkg.set_step_parts(4)
    try:
        a = pkg.Solver(mesh, cfg).init()
        b = pkg.Solver(mesh, cfg).init()
    finally:
        pkg.set_step_parts(0)
    q = a.get("q")
    if pinned:
        bufs = [(pkg.PinnedArray(q.size), pkg.PinnedArray(q.size)) for _ in range(2)]
        views = [(x.array, y.array) for x, y in bufs]
    else:
        views = [(np.empty_like(q), np.empty_like(q)) for _ in range(2)]
    for call, (h_in, h_out) in enumerate((views[0], views[0], views[1])):
        h_in[:] = b.get("q")
        h_out[:] = np.nan
        a.step_host(h_in, nsteps, h_out)
        b.run(nsteps)
        b.sync()
        assert np.array_equal(h_out, b.get("q")), call
        assert np.array_equal(a.get("q"), b.get("q")) and a.time() == b.time(), call


def test_face_kernel_register_bound_bitwise(pkg):
    """The face kernel compiled for at most 64 registers: the same bits, chain and ranges."""
    lib = pkg.lib()
    mesh = pkg.Mesh.naca_ogrid(96, 24, farfield="characteristic")
    cfg = pkg.config(N=3, cfl=0.5, mach=0.5, alpha_deg=2.0)
    q1, dt1, _, _ = run_parts(pkg, mesh, cfg, 1, 20)
    lib.dg_set_face_regs64(1)
    try:
        for P in (1, 4):
            q, dt, _, _ = run_parts(pkg, mesh, cfg, P, 20)
            assert np.array_equal(q, q1) and np.array_equal(dt, dt1), P
    finally:
        lib.dg_set_face_regs64(0)


@pytest.mark.parametrize("G", [1, 2, 3])
@pytest.mark.parametrize("app", ["airfoil", "vortex"])
def test_steps_per_graph_bitwise(pkg, G, app):
    """Several steps in one graph launch (the next step's face launches overlapping the previous
    step's element launches), with a step count that leaves a remainder of one-step graphs: the
    same q, dt sequence and time as one chain of launches per step."""
    lib = pkg.lib()
    if app == "vortex":
        mesh = pkg.Mesh.vortex_square(64)
        cfg = pkg.config(N=3, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.5, vortex_x0=0.0, vortex_y0=0.0,
                         vortex_beta=5.0)
    else:
        mesh = pkg.Mesh.naca_ogrid(96, 24, farfield="characteristic")
        cfg = pkg.config(N=3, cfl=0.5, mach=0.5, alpha_deg=2.0)
    q1, dt1, t1, _ = run_parts(pkg, mesh, cfg, 1, 7)
    prev = lib.dg_steps_per_graph()
    lib.dg_set_steps_per_graph(G)
    try:
        q, dt, t, _ = run_parts(pkg, mesh, cfg, 4, 7)
    finally:
        lib.dg_set_steps_per_graph(prev)
    assert np.array_equal(q, q1) and np.array_equal(dt, dt1) and t == t1
