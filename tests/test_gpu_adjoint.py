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


def setup(pkg, N=3, ntheta=32, nr=8, nsteps=60, navg=20, C=7, alpha=2.0, mach=0.5):
    mesh = pkg.Mesh.naca_ogrid(ntheta, nr, radius=4.0, farfield="reference")
    cfg = pkg.config(N=N, cfl=0.5, mach=mach, alpha_deg=alpha)
    return mesh, cfg, pkg.LiftObjective(mesh, cfg, nsteps, navg, C)


@pytest.mark.parametrize("N", [2, 3, 4])
def test_rhs_vjp_dot_product(pkg, N):
    mesh, cfg, obj = setup(pkg, N=N)
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
    # alpha: through the inflow/outflow ghost states
    def rhs_at(alpha):
        c2 = pkg.config(N=N, cfl=0.5, mach=cfg.mach, alpha_deg=alpha)
        return pkg.Solver(mesh, c2).init().rhs(W)
    ha = 1e-5
    da = np.dot(v, (rhs_at(cfg.alpha_deg + ha) - rhs_at(cfg.alpha_deg - ha)) / (2 * ha))
    _, ap = obj.rhs_vjp(W, v)
    assert abs(da - ap) <= 1e-6 * max(abs(da), 1e-30)


def test_gradient_matches_finite_differences(pkg):
    mesh, cfg, obj = setup(pkg)
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


def test_rejects_characteristic_farfield(pkg):
    mesh = pkg.Mesh.naca_ogrid(32, 8, farfield="characteristic")
    with pytest.raises(pkg.DGError):
        pkg.LiftObjective(mesh, pkg.config(N=3), 10, 5)
