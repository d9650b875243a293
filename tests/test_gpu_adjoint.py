"""The discrete adjoint of the lift objective (dg_adjoint_*).

* one right-hand side: <v, dL/dW u> by central differences of L against <(dL/dW)^T v, u> from
  the reverse kernels, and the same for d/dalpha (dot-product test of every reverse kernel);
* whole trajectories: dJ/dalpha and dJ/dq0 . delta against central finite differences with
  h = 1e-6 and the frozen dt sequence, to 1e-7;
* checkpoint intervals change nothing (recomputation is bit-exact).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def setup(pkg, N=3, ntheta=32, nr=8, nsteps=60, navg=20, C=7, alpha=2.0, mach=0.5, farfield="reference"):
    mesh = pkg.Mesh.naca_ogrid(ntheta, nr, radius=4.0, farfield=farfield)
    cfg = pkg.config(N=N, cfl=0.5, mach=mach, alpha_deg=alpha)
    return mesh, cfg, pkg.LiftObjective(mesh, cfg, nsteps, navg, C)


@pytest.mark.parametrize("N,farfield", [(1, "reference"), (2, "reference"), (3, "reference"), (4, "reference"),
                                        (5, "reference"), (6, "reference"), (2, "characteristic"),
                                        (3, "characteristic"), (5, "characteristic")])
def test_rhs_vjp_dot_product(pkg, N, farfield):
    mesh, cfg, obj = setup(pkg, N=N, farfield=farfield)
    s = pkg.Solver(mesh, cfg).init()
    rng = np.random.default_rng(N)
    q = s.get("q")
    W = q * (1.0 + 0.05 * rng.standard_normal(q.size))
    u = q * rng.standard_normal(q.size)
    v = rng.standard_normal(q.size)
    h = 1e-6
    jvp = (s.rhs(W + h * u) - s.rhs(W - h * u)) / (2 * h)
    vjp, _ = obj.rhs_vjp(W, v)
    lhs, rhs = np.dot(v, jvp), np.dot(vjp, u)
    assert abs(lhs - rhs) <= 1e-7 * max(abs(lhs), abs(rhs))
    # alpha: through the inflow/outflow (or characteristic farfield) ghost states
    def rhs_at(alpha):
        c2 = pkg.config(N=N, cfl=0.5, mach=cfg.mach, alpha_deg=alpha)
        return pkg.Solver(mesh, c2).init().rhs(W)
    ha = 1e-5
    da = np.dot(v, (rhs_at(cfg.alpha_deg + ha) - rhs_at(cfg.alpha_deg - ha)) / (2 * ha))
    _, ap = obj.rhs_vjp(W, v)
    assert abs(da - ap) <= 1e-6 * max(abs(da), 1e-30)


@pytest.mark.parametrize("farfield", ["reference", "characteristic"])
def test_gradient_matches_finite_differences(pkg, farfield):
    mesh, cfg, obj = setup(pkg, farfield=farfield)
    J = obj.forward()
    ga, gq = obj.backward()
    assert obj.evaluate(cfg.alpha_deg) == J  # frozen-dt re-evaluation is the same function
    h = 1e-6
    fd = (obj.evaluate(cfg.alpha_deg + h) - obj.evaluate(cfg.alpha_deg - h)) / (2 * h)
    assert abs(ga - fd) <= 1e-7 * max(abs(fd), 1e-30), (ga, fd)
    s = pkg.Solver(mesh, cfg).init()
    q0 = s.get("q")
    delta = q0 * np.random.default_rng(5).standard_normal(q0.size) * 1e-2
    fdq = (obj.evaluate(cfg.alpha_deg, q0 + h * delta) - obj.evaluate(cfg.alpha_deg, q0 - h * delta)) / (2 * h)
    adq = float(np.dot(gq, delta))
    assert abs(adq - fdq) <= 1e-7 * max(abs(fdq), 1e-30), (adq, fdq)


def test_checkpoint_interval_invariance(pkg):
    res = []
    for C in (1, 7, 60):
        _, _, obj = setup(pkg, C=C)
        J = obj.forward()
        ga, gq = obj.backward()
        res.append((J, ga, gq))
    for J, ga, gq in res[1:]:
        assert J == res[0][0] and ga == res[0][1] and np.array_equal(gq, res[0][2])


def test_backward_scales_with_grad_output(pkg):
    _, _, obj = setup(pkg, nsteps=20, navg=5, C=5)
    obj.forward()
    ga1, gq1 = obj.backward(1.0)
    ga2, gq2 = obj.backward(-2.5)
    assert ga2 == -2.5 * ga1 and np.allclose(gq2, -2.5 * gq1, rtol=0, atol=0)


def test_farfield_branches_dot_product(pkg):
    """The reverse sweep of the characteristic farfield in each of its branches: at M 1.3 the
    circular farfield of the O-grid has supersonic inflow and outflow faces as well as subsonic
    ones (where |v_n| < c); with every boundary edge of type 3 all four branches are taken."""
    mesh = pkg.Mesh.naca_ogrid(32, 8, radius=4.0, farfield="characteristic")
    mesh.set_bedge_type(np.full(mesh.size("bedges"), 3, dtype=np.int32))
    for mach in (0.5, 1.3):
        cfg = pkg.config(N=3, cfl=0.5, mach=mach, alpha_deg=10.0)
        obj = pkg.LiftObjective(mesh, cfg, 10, 5, 5)
        s = pkg.Solver(mesh, cfg).init()
        rng = np.random.default_rng(31)
        q = s.get("q")
        W = q * (1.0 + 0.05 * rng.standard_normal(q.size))
        u = q * rng.standard_normal(q.size)
        v = rng.standard_normal(q.size)
        h = 1e-6
        jvp = (s.rhs(W + h * u) - s.rhs(W - h * u)) / (2 * h)
        vjp, ap = obj.rhs_vjp(W, v)
        lhs, rhs = np.dot(v, jvp), np.dot(vjp, u)
        assert abs(lhs - rhs) <= 1e-7 * max(abs(lhs), abs(rhs)), mach

        def rhs_at(alpha):
            return pkg.Solver(mesh, pkg.config(N=3, cfl=0.5, mach=mach, alpha_deg=alpha)).init().rhs(W)
        ha = 1e-5
        da = np.dot(v, (rhs_at(10.0 + ha) - rhs_at(10.0 - ha)) / (2 * ha))
        assert abs(da - ap) <= 1e-6 * max(abs(da), 1e-30), mach


# ---------------------------------------------------------------- isentropic vortex: d/d beta
def vortex_setup(pkg, N=2, n=16, nsteps=40, C=7, beta=5.0):
    mesh = pkg.Mesh.vortex_square(n)
    cfg = pkg.config(N=N, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.5, vortex_x0=0.0,
                     vortex_y0=0.0, vortex_beta=beta)
    return mesh, cfg, pkg.LiftObjective(mesh, cfg, nsteps, 1, C)


@pytest.mark.parametrize("N", [1, 2, 3])
def test_vortex_rhs_vjp_dot_product(pkg, N):
    mesh, cfg, obj = vortex_setup(pkg, N=N)
    s = pkg.Solver(mesh, cfg).init()
    rng = np.random.default_rng(10 + N)
    q = s.get("q")
    W = q * (1.0 + 0.05 * rng.standard_normal(q.size))
    u = q * rng.standard_normal(q.size)
    v = rng.standard_normal(q.size)
    h = 1e-6
    jvp = (s.rhs(W + h * u) - s.rhs(W - h * u)) / (2 * h)
    vjp, _ = obj.rhs_vjp(W, v)
    lhs, rhs = np.dot(v, jvp), np.dot(vjp, u)
    assert abs(lhs - rhs) <= 1e-7 * max(abs(lhs), abs(rhs))


def test_vortex_beta_gradient_matches_finite_differences(pkg):
    mesh, cfg, obj = vortex_setup(pkg)
    J = obj.forward()
    gb, gq = obj.backward()
    assert obj.evaluate(cfg.vortex_beta) == J
    h = 1e-6
    fd = (obj.evaluate(cfg.vortex_beta + h) - obj.evaluate(cfg.vortex_beta - h)) / (2 * h)
    assert abs(gb - fd) <= 1e-7 * max(abs(fd), 1e-30), (gb, fd)
    q0 = pkg.Solver(mesh, cfg).init().get("q")
    # Perturbation h * delta of 1e-6 relative to q: J is O(10), so a step 100x smaller puts the
    # central difference at its rounding-noise floor (measured 3e-7 relative there, 4e-10 here).
    delta = q0 * np.random.default_rng(6).standard_normal(q0.size)
    fdq = (obj.evaluate(cfg.vortex_beta, q0 + h * delta) - obj.evaluate(cfg.vortex_beta, q0 - h * delta)) / (2 * h)
    assert abs(np.dot(gq, delta) - fdq) <= 1e-7 * max(abs(fdq), 1e-30)


def test_vortex_checkpoint_interval_invariance(pkg):
    res = []
    for C in (1, 6, 40):
        _, _, obj = vortex_setup(pkg, C=C)
        J = obj.forward()
        res.append((J,) + obj.backward())
    for J, gb, gq in res[1:]:
        assert J == res[0][0] and gb == res[0][1] and np.array_equal(gq, res[0][2])


def test_vortex_batched_gradient_equals_individual(pkg):
    """Instances with different beta, forward and backward in one batched call each."""
    betas = (3.0, 4.0, 5.0)   # stronger vortices are under-resolved on this small mesh
    objs = [vortex_setup(pkg, beta=b)[2] for b in betas]
    J = pkg.adjoint_batch_forward(objs)
    g, gq = pkg.adjoint_batch_backward(objs, want_q0=True)
    for k, b in enumerate(betas):
        ref = vortex_setup(pkg, beta=b)[2]
        assert ref.forward() == J[k]
        gb, gqk = ref.backward()
        assert gb == g[k] and np.array_equal(gqk, gq[k])


# ---------------------------------------------------------------- tangent-linear FP64 run
@pytest.mark.parametrize("farfield", ["reference", "characteristic"])
def test_tangent_linear_matches_adjoint(pkg, farfield):
    """Forward-mode derivative (dual numbers through the forward formulas, hand-written ghost
    state and stage tangents) against the reverse-mode gradient: the same discrete derivative
    by two independent routes."""
    mesh, cfg, obj = setup(pkg, farfield=farfield)
    obj.forward()
    ga, gq = obj.backward()
    ta = obj.tangent(1.0)
    assert abs(ta - ga) <= 1e-10 * abs(ga), (ta, ga)
    q0 = pkg.Solver(mesh, cfg).init().get("q")
    delta = q0 * np.random.default_rng(8).standard_normal(q0.size) * 1e-2
    tq = obj.tangent(0.0, delta)
    assert abs(tq - np.dot(gq, delta)) <= 1e-10 * abs(tq), (tq, np.dot(gq, delta))
    both = obj.tangent(0.5, delta)
    assert abs(both - (0.5 * ta + tq)) <= 1e-12 * abs(both)


def test_vortex_tangent_linear_matches_adjoint(pkg):
    mesh, cfg, obj = vortex_setup(pkg)
    obj.forward()
    gb, gq = obj.backward()
    tb = obj.tangent(1.0)
    assert abs(tb - gb) <= 1e-10 * abs(gb), (tb, gb)
    q0 = pkg.Solver(mesh, cfg).init().get("q")
    delta = q0 * np.random.default_rng(9).standard_normal(q0.size) * 1e-2
    tq = obj.tangent(0.0, delta)
    assert abs(tq - np.dot(gq, delta)) <= 1e-10 * abs(tq)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_even_odd_adjoint_equals_dense(pkg, N):
    """The transposed even/odd element adjoint (default) and the dense one: same vector-Jacobian
    product to rounding, and the same whole-trajectory gradient."""
    mesh, cfg, _ = setup(pkg, N=N)
    rng = np.random.default_rng(40 + N)
    out = []
    prev = pkg.lib().dg_elem_variant()
    for variant in (0, 1):
        pkg.lib().dg_set_elem_variant(variant)
        try:
            obj = pkg.LiftObjective(mesh, cfg, 12, 4, 5)
            q = pkg.Solver(mesh, cfg).init().get("q")
            W = q * (1.0 + 0.05 * np.random.default_rng(N).standard_normal(q.size))
            v = np.random.default_rng(N + 1).standard_normal(q.size)
            vjp, ap = obj.rhs_vjp(W, v)
            obj.forward()
            out.append((vjp, ap) + obj.backward())
        finally:
            pkg.lib().dg_set_elem_variant(prev)
    a, b = out
    assert np.linalg.norm(a[0] - b[0]) <= 1e-13 * np.linalg.norm(a[0])
    assert abs(a[1] - b[1]) <= 1e-12 * abs(a[1])
    assert abs(a[2] - b[2]) <= 1e-12 * abs(a[2])
    assert np.linalg.norm(a[3] - b[3]) <= 1e-12 * np.linalg.norm(a[3])


def test_torch_autograd_function(pkg):
    """The objective as a torch.autograd.Function: autograd's gradient is the adjoint's."""
    torch = pytest.importorskip("torch")
    mesh, cfg, obj = setup(pkg, nsteps=30, navg=10, C=7)
    f = pkg.torch_objective(obj)
    p = torch.tensor(cfg.alpha_deg, dtype=torch.float64, requires_grad=True)
    J = f(p)
    (3.0 * J).backward()
    ref = pkg.LiftObjective(mesh, cfg, 30, 10, 7)
    assert float(J.detach()) == ref.forward()
    ga, _ = ref.backward(3.0, want_q0=False)
    assert float(p.grad) == ga
