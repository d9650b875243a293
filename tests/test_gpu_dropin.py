"""GPU parity of the OP2 drop-in (include/op2_gb300.h).

The driver below is the reference's main loop (src/airfoil.cpp:135-331) written against the
OP2 mirror.  The drop-in kernels keep the reference's operation order without FMA
contraction, so with equal constant tables they must equal the oracle's restated kernels
bit for bit (and those equal the reference build bit for bit, tests/test_oracle.py).
Against the reference build's golden run (its literal tables vs the generated ones here) the
parity target is relative L2 <= 1e-11 after 1000 steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def op2(pkg):
    import importlib
    return importlib.import_module(pkg.__name__ + ".op2")


class Airfoil:
    """src/airfoil.cpp:135-237 on the drop-in."""

    def __init__(self, op2, m, ops, phys, cfl=1.0):
        self.op2, self.cfl = op2, cfl
        N = int(ops["N"])
        Np, Nfp = (N + 1) * (N + 2) // 2, N + 1
        self.Np, self.Nfp = Np, Nfp
        o = op2
        o.op_init(0)
        K = m["cell2nodes"].shape[0]
        self.K = K
        nodes = o.op_decl_set(m["coords"].shape[0], "nodes")
        self.cells = cells = o.op_decl_set(K, "cells")
        self.edges = edges = o.op_decl_set(m["edge2cells"].shape[0], "edges")
        self.bedges = bedges = o.op_decl_set(m["bedge2cell"].shape[0], "bedges")
        cell2nodes = o.op_decl_map(cells, nodes, 3, m["cell2nodes"], "cell2nodes")
        self.edge2cells = o.op_decl_map(edges, cells, 2, m["edge2cells"], "edge2cells")
        self.bedge2cells = o.op_decl_map(bedges, cells, 1, m["bedge2cell"], "bedge2cells")
        node_coords = o.op_decl_dat(nodes, 2, "double", m["coords"], "node_coords")
        d = {}
        for name, dim in (("nodeX", 3), ("nodeY", 3), ("x", Np), ("y", Np), ("xr", Np), ("yr", Np),
                          ("xs", Np), ("ys", Np), ("rx", Np), ("ry", Np), ("sx", Np), ("sy", Np),
                          ("nx", 3 * Nfp), ("ny", 3 * Nfp), ("fscale", 3 * Nfp), ("q", 4 * Np),
                          ("workingQ", 4 * Np), ("rk1", 4 * Np), ("rk2", 4 * Np), ("rk3", 4 * Np),
                          ("exteriorQ", 12 * Nfp)):
            d[name] = (o.op_decl_dat(cells, dim, "double", np.zeros(K * dim), name), dim)
        self.d = d
        self.bedge_type = o.op_decl_dat(bedges, 1, "int", m["bedge_type"], "bedge_type")
        self.edgeNum = o.op_decl_dat(edges, 2, "int", m["edgeNum"], "edgeNum")
        self.bedgeNum = o.op_decl_dat(bedges, 1, "int", m["bedgeNum"], "bedgeNum")
        for k in ("gam", "bc_mach", "bc_alpha", "bc_p", "bc_r", "bc_u", "bc_v", "bc_e"):
            o.op_decl_const2(k, 1, "double", phys[k])
        o.op_decl_const2("ones", Np, "double", np.ones(Np))
        for k in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT"):
            o.op_decl_const2(k, np.asarray(ops[k]).size, "double", np.asarray(ops[k]).ravel())
        o.op_decl_const2("FMASK", 3 * Nfp, "int", np.asarray(ops["FMASK"], dtype=np.int32))
        A = self.A
        o.op_par_loop_init_grid("init_grid", cells,
                                o.op_arg_dat(node_coords, 0, cell2nodes, 2, "double", o.OP_READ),
                                o.op_arg_dat(node_coords, 1, cell2nodes, 2, "double", o.OP_READ),
                                o.op_arg_dat(node_coords, 2, cell2nodes, 2, "double", o.OP_READ),
                                *[A(n, o.OP_WRITE) for n in ("nodeX", "nodeY", "x", "y", "xr", "yr", "xs", "ys",
                                                             "rx", "ry", "sx", "sy", "nx", "ny", "fscale")])
        o.op_par_loop_set_ic("set_ic", cells, A("q", o.OP_WRITE), A("workingQ", o.OP_WRITE))
        o.op_par_loop_neighbour_zero("neighbour_zero", cells, A("exteriorQ", o.OP_WRITE))
        self.dt = (1.0 / self.calc_dt()) * cfl

    def A(self, name, acc, idx=-1, mp=None):
        dat, dim = self.d[name]
        return self.op2.op_arg_dat(dat, idx, mp, dim, "double", acc)

    def calc_dt(self):
        o = self.op2
        dt1 = np.zeros(1)
        o.op_par_loop_calc_dt("calc_dt", self.cells, self.A("q", o.OP_READ), self.A("fscale", o.OP_READ),
                              o.op_arg_gbl(dt1, 1, "double", o.OP_MAX))
        return float(dt1[0])

    def run(self, iters):
        """src/airfoil.cpp:252-334"""
        o, A, e2c, b2c = self.op2, self.A, self.edge2cells, self.bedge2cells
        dts = []
        for _ in range(iters):
            dts.append(self.dt)
            dt = np.array([self.dt])
            for j in range(3):
                o.op_par_loop_get_neighbour_q(
                    "get_neighbour_q", self.edges, o.op_arg_dat(self.edgeNum, -1, None, 2, "int", o.OP_READ),
                    A("nodeX", o.OP_READ, 0, e2c), A("nodeY", o.OP_READ, 0, e2c),
                    A("nodeX", o.OP_READ, 1, e2c), A("nodeY", o.OP_READ, 1, e2c),
                    A("workingQ", o.OP_READ, 0, e2c), A("workingQ", o.OP_READ, 1, e2c),
                    A("exteriorQ", o.OP_INC, 0, e2c), A("exteriorQ", o.OP_INC, 1, e2c))
                o.op_par_loop_get_bedge_q(
                    "get_bedge_q", self.bedges, o.op_arg_dat(self.bedge_type, -1, None, 1, "int", o.OP_READ),
                    o.op_arg_dat(self.bedgeNum, -1, None, 1, "int", o.OP_READ),
                    A("nx", o.OP_READ, 0, b2c), A("ny", o.OP_READ, 0, b2c), A("workingQ", o.OP_READ, 0, b2c),
                    A("exteriorQ", o.OP_INC, 0, b2c))
                o.op_par_loop_euler_rhs(
                    "euler_rhs", self.cells, A("workingQ", o.OP_READ), A("exteriorQ", o.OP_RW),
                    A("rx", o.OP_READ), A("ry", o.OP_READ), A("sx", o.OP_READ), A("sy", o.OP_READ),
                    A("fscale", o.OP_READ), A("nx", o.OP_READ), A("ny", o.OP_READ), A("rk%d" % (j + 1), o.OP_WRITE))
                if j != 2:
                    o.op_par_loop_set_workingQ(
                        "set_workingQ", self.cells, o.op_arg_gbl(dt, 1, "double", o.OP_READ),
                        o.op_arg_gbl(np.array([j], dtype=np.int32), 1, "int", o.OP_READ),
                        A("q", o.OP_READ), A("rk1", o.OP_READ), A("rk2", o.OP_READ), A("workingQ", o.OP_WRITE))
            o.op_par_loop_update_Q("update_Q", self.cells, o.op_arg_gbl(dt, 1, "double", o.OP_READ),
                                   A("q", o.OP_RW), A("rk1", o.OP_READ), A("rk2", o.OP_READ), A("rk3", o.OP_READ),
                                   A("workingQ", o.OP_WRITE))
            self.dt = (1.0 / self.calc_dt()) * self.cfl
        return np.array(dts)

    def fetch(self, name):
        dat, dim = self.d[name]
        out = np.empty(self.K * dim)
        self.op2.op_fetch_data(dat, out)
        return out


@pytest.mark.parametrize("N", [3, 4])
def test_dropin_bitwise_equals_oracle(op2, orc, oops, omesh, N):
    m = omesh.naca_ogrid(48, 12, farfield="reference")
    ops, phys = oops.operators(N), orc.freestream(0.4, 1.5)
    a = Airfoil(op2, m, ops, phys)
    o = orc.Oracle(m, ops, phys, kind="port")
    o.init(1.0)
    for name in ("x", "y", "rx", "sy", "nx", "ny", "fscale", "q"):
        assert np.array_equal(a.fetch(name), o.get(name)), name
    assert a.dt == o.dt
    dts = a.run(10)
    dto = o.run(10, nthreads=1)
    assert np.array_equal(dts, dto)
    assert np.array_equal(a.fetch("q"), o.get("q"))
    assert np.array_equal(a.fetch("rk3"), o.get("rk3"))


def test_dropin_golden_1000_steps(op2, orc, oops, golden_naca):
    """Reference parity through the drop-in: the reference's mesh and state, 1000 steps."""
    g, m = golden_naca
    a = Airfoil(op2, m, oops.operators(4), orc.freestream(0.4, 0.0))
    assert abs(a.dt / g["dt0"] - 1) < 1e-10
    dts = a.run(1000)
    assert orc.rel_l2(a.fetch("q"), g["q1000"]) < 1e-11
    assert np.abs(dts / g["dt1000"] - 1).max() < 1e-9


def test_dropin_rejects_bad_arguments(op2, oops, orc, omesh):
    m = omesh.naca_ogrid(16, 4)
    a = Airfoil(op2, m, oops.operators(3), orc.freestream(0.4, 0.0))
    o = op2
    with pytest.raises(o.Op2Error):  # rk dat of the wrong dimension
        bad = o.op_decl_dat(a.cells, 7, "double", np.zeros(a.K * 7), "bad")
        o.op_par_loop_euler_rhs("euler_rhs", a.cells, a.A("workingQ", o.OP_READ), a.A("exteriorQ", o.OP_RW),
                                a.A("rx", o.OP_READ), a.A("ry", o.OP_READ), a.A("sx", o.OP_READ), a.A("sy", o.OP_READ),
                                a.A("fscale", o.OP_READ), a.A("nx", o.OP_READ), a.A("ny", o.OP_READ),
                                o.op_arg_dat(bad, -1, None, 7, "double", o.OP_WRITE))
    with pytest.raises(o.Op2Error):  # direct access on the wrong set
        o.op_par_loop_neighbour_zero("neighbour_zero", a.edges, a.A("exteriorQ", o.OP_WRITE))
    with pytest.raises(o.Op2Error):  # map entry out of range
        o.op_decl_map(a.edges, a.cells, 2, np.full(2 * op2.op_get_size(a.edges), 10 ** 6), "bad")
    with pytest.raises(o.Op2Error):
        o.op_par_loop_calc_dt("calc_dt", a.cells, a.A("q", o.OP_READ), a.A("fscale", o.OP_READ),
                              o.op_arg_gbl(np.zeros(1), 1, "double", o.OP_READ))
    # the runtime is still usable
    assert a.calc_dt() > 0.0


class Vortex(Airfoil):
    """vortex/src/vortex.cpp:112-318 on the drop-in: the vortex app's loops (set_ic, get_neighbour_q,
    get_bedge_q with their vortex argument lists, exteriorQ zeroed every stage and read by
    euler_rhs, dt = 0.1/dt1 frozen, l2_error at the end)."""

    def __init__(self, op2, m, ops, phys, cfl=0.1):
        self.op2, self.cfl = op2, cfl
        N = int(ops["N"])
        Np, Nfp = (N + 1) * (N + 2) // 2, N + 1
        self.Np, self.Nfp = Np, Nfp
        o = op2
        o.op_init(0)
        K = m["cell2nodes"].shape[0]
        self.K = K
        nodes = o.op_decl_set(m["coords"].shape[0], "nodes")
        self.cells = cells = o.op_decl_set(K, "cells")
        self.edges = edges = o.op_decl_set(m["edge2cells"].shape[0], "edges")
        self.bedges = bedges = o.op_decl_set(m["bedge2cell"].shape[0], "bedges")
        cell2nodes = o.op_decl_map(cells, nodes, 3, m["cell2nodes"], "cell2nodes")
        self.edge2nodes = o.op_decl_map(edges, nodes, 2, m["edge2nodes"], "edge2nodes")
        self.edge2cells = o.op_decl_map(edges, cells, 2, m["edge2cells"], "edge2cells")
        self.bedge2nodes = o.op_decl_map(bedges, nodes, 2, m["bedge2nodes"], "bedge2nodes")
        self.bedge2cells = o.op_decl_map(bedges, cells, 1, m["bedge2cell"], "bedge2cells")
        self.node_coords = node_coords = o.op_decl_dat(nodes, 2, "double", m["coords"], "node_coords")
        d = {}
        for name, dim in (("nodeX", 3), ("nodeY", 3), ("x", Np), ("y", Np), ("xr", Np), ("yr", Np),
                          ("xs", Np), ("ys", Np), ("rx", Np), ("ry", Np), ("sx", Np), ("sy", Np),
                          ("nx", 3 * Nfp), ("ny", 3 * Nfp), ("fscale", 3 * Nfp), ("q", 4 * Np),
                          ("workingQ", 4 * Np), ("rk1", 4 * Np), ("rk2", 4 * Np), ("rk3", 4 * Np),
                          ("exteriorQ", 12 * Nfp), ("error", 4 * Np)):
            d[name] = (o.op_decl_dat(cells, dim, "double", np.zeros(K * dim), name), dim)
        self.d = d
        self.edgeNum = o.op_decl_dat(edges, 2, "int", m["edgeNum"], "edgeNum")
        self.bedgeNum = o.op_decl_dat(bedges, 1, "int", m["bedgeNum"], "bedgeNum")
        for k in ("gam", "vortex_x0", "vortex_y0", "vortex_beta"):
            o.op_decl_const2(k, 1, "double", phys[k])
        o.op_decl_const2("ones", Np, "double", np.ones(Np))
        for k in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT"):
            o.op_decl_const2(k, np.asarray(ops[k]).size, "double", np.asarray(ops[k]).ravel())
        o.op_decl_const2("FMASK", 3 * Nfp, "int", np.asarray(ops["FMASK"], dtype=np.int32))
        A = self.A
        o.op_par_loop_init_grid("init_grid", cells,
                                o.op_arg_dat(node_coords, 0, cell2nodes, 2, "double", o.OP_READ),
                                o.op_arg_dat(node_coords, 1, cell2nodes, 2, "double", o.OP_READ),
                                o.op_arg_dat(node_coords, 2, cell2nodes, 2, "double", o.OP_READ),
                                *[A(n, o.OP_WRITE) for n in ("nodeX", "nodeY", "x", "y", "xr", "yr", "xs", "ys",
                                                             "rx", "ry", "sx", "sy", "nx", "ny", "fscale")])
        o.op_par_loop_set_ic("set_ic", cells, o.op_arg_gbl(np.zeros(1), 1, "double", o.OP_READ),
                             A("x", o.OP_READ), A("y", o.OP_READ), A("q", o.OP_WRITE), A("workingQ", o.OP_WRITE))
        self.dt = (1.0 / self.calc_dt()) * cfl
        self.t = 0.0

    def run(self, iters):
        """vortex/src/vortex.cpp:226-305"""
        o, A, e2c, b2c = self.op2, self.A, self.edge2cells, self.bedge2cells
        nc = self.node_coords
        rk_t_frac = (0.0, 1.0, 0.5)
        for _ in range(iters):
            dt = np.array([self.dt])
            for j in range(3):
                o.op_par_loop_neighbour_zero("neighbour_zero", self.cells, A("exteriorQ", o.OP_WRITE))
                o.op_par_loop_get_neighbour_q(
                    "get_neighbour_q", self.edges, o.op_arg_dat(self.edgeNum, -1, None, 2, "int", o.OP_READ),
                    o.op_arg_dat(nc, 0, self.edge2nodes, 2, "double", o.OP_READ),
                    o.op_arg_dat(nc, 1, self.edge2nodes, 2, "double", o.OP_READ),
                    A("nodeX", o.OP_READ, 0, e2c), A("nodeY", o.OP_READ, 0, e2c),
                    A("nodeX", o.OP_READ, 1, e2c), A("nodeY", o.OP_READ, 1, e2c),
                    A("workingQ", o.OP_READ, 0, e2c), A("workingQ", o.OP_READ, 1, e2c),
                    A("exteriorQ", o.OP_INC, 0, e2c), A("exteriorQ", o.OP_INC, 1, e2c))
                t1 = np.array([self.t + rk_t_frac[j] * self.dt])
                o.op_par_loop_get_bedge_q(
                    "get_bedge_q", self.bedges, o.op_arg_dat(self.bedgeNum, -1, None, 1, "int", o.OP_READ),
                    o.op_arg_dat(nc, 0, self.bedge2nodes, 2, "double", o.OP_READ),
                    o.op_arg_dat(nc, 1, self.bedge2nodes, 2, "double", o.OP_READ),
                    A("nodeX", o.OP_READ, 0, b2c), A("nodeY", o.OP_READ, 0, b2c),
                    A("x", o.OP_READ, 0, b2c), A("y", o.OP_READ, 0, b2c),
                    o.op_arg_gbl(t1, 1, "double", o.OP_READ), A("exteriorQ", o.OP_INC, 0, b2c))
                o.op_par_loop_euler_rhs(
                    "euler_rhs", self.cells, A("workingQ", o.OP_READ), A("exteriorQ", o.OP_READ),
                    A("rx", o.OP_READ), A("ry", o.OP_READ), A("sx", o.OP_READ), A("sy", o.OP_READ),
                    A("fscale", o.OP_READ), A("nx", o.OP_READ), A("ny", o.OP_READ), A("rk%d" % (j + 1), o.OP_WRITE))
                if j != 2:
                    o.op_par_loop_set_workingQ(
                        "set_workingQ", self.cells, o.op_arg_gbl(dt, 1, "double", o.OP_READ),
                        o.op_arg_gbl(np.array([j], dtype=np.int32), 1, "int", o.OP_READ),
                        A("q", o.OP_READ), A("rk1", o.OP_READ), A("rk2", o.OP_READ), A("workingQ", o.OP_WRITE))
            o.op_par_loop_update_Q("update_Q", self.cells, o.op_arg_gbl(dt, 1, "double", o.OP_READ),
                                   A("q", o.OP_RW), A("rk1", o.OP_READ), A("rk2", o.OP_READ), A("rk3", o.OP_READ),
                                   A("workingQ", o.OP_WRITE))
            self.t += self.dt

    def l2_error(self):
        o = self.op2
        e = [np.zeros(1) for _ in range(4)]
        o.op_par_loop_l2_error("l2_error", self.cells, self.A("x", o.OP_READ), self.A("y", o.OP_READ),
                               self.A("q", o.OP_READ), o.op_arg_gbl(np.array([self.t]), 1, "double", o.OP_READ),
                               *[o.op_arg_gbl(x, 1, "double", o.OP_INC) for x in e], self.A("error", o.OP_WRITE))
        return np.array([float(x[0]) for x in e])


@pytest.mark.parametrize("N", [3, 4])
def test_dropin_vortex_matches_oracle(op2, orc, oops, omesh, N):
    """The vortex app's loop sequence: geometry and dt bit-exact; q after 20 steps and the L2
    error sums to rounding (exp/pow of the analytic state differ in the last bits between the
    device and host maths libraries)."""
    m = omesh.vortex_square(16)
    phys = orc.freestream(0.4, 0.0)
    phys.update(vortex_x0=0.0, vortex_y0=0.0, vortex_beta=5.0)
    ops = oops.operators(N)
    v = Vortex(op2, m, ops, phys)
    o = orc.Oracle(m, ops, phys, app=orc.APP_VORTEX, kind="port")
    o.init(0.1)
    for name in ("x", "y", "rx", "sy", "nx", "fscale"):
        assert np.array_equal(v.fetch(name), o.get(name)), name
    assert orc.rel_l2(v.fetch("q"), o.get("q")) < 1e-15
    assert abs(v.dt / o.dt - 1) < 1e-15
    v.run(20)
    o.run(20, dt_mode=orc.DT_FROZEN, nthreads=1)
    assert orc.rel_l2(v.fetch("q"), o.get("q")) < 1e-13
    assert np.abs(v.l2_error() / o.l2_error() - 1).max() < 1e-9
    sums = v.l2_error()
    err = v.fetch("error").reshape(-1, 4)  # the per-node squared errors the loop also writes
    assert np.allclose(err.sum(0), sums, rtol=1e-12, atol=0)


def test_dropin_vortex_golden(op2, orc, oops, golden_vortex):
    """The reference's vortex mesh and state (x0=5, beta=5, dt=0.1/dt1), 100 steps."""
    g, m = golden_vortex
    phys = orc.freestream(0.4, 0.0)
    phys.update(vortex_x0=5.0, vortex_y0=0.0, vortex_beta=5.0)
    v = Vortex(op2, m, oops.operators(4), phys)
    assert abs(v.dt / g["dt"] - 1) < 1e-10
    v.run(100)
    assert orc.rel_l2(v.fetch("q"), g["q100"]) < 1e-11
    assert np.abs(v.l2_error() / g["l2_100"] - 1).max() < 1e-7


def test_dropin_vortex_rejects_missing_constants(op2, omesh, oops):
    """A vortex loop without the vortex constants is an error, as OP2's would be."""
    op2.op_init(0)
    m = omesh.vortex_square(4)
    cells = op2.op_decl_set(m["cell2nodes"].shape[0], "cells")
    x = op2.op_decl_dat(cells, 10, "double", np.zeros(10 * len(m["cell2nodes"])), "x")
    q = op2.op_decl_dat(cells, 40, "double", np.zeros(40 * len(m["cell2nodes"])), "q")
    with pytest.raises(op2.Op2Error):
        op2.op_par_loop_set_ic("set_ic", cells, op2.op_arg_gbl(np.zeros(1), 1, "double", op2.OP_READ),
                               op2.op_arg_dat(x, -1, None, 10, "double", op2.OP_READ),
                               op2.op_arg_dat(x, -1, None, 10, "double", op2.OP_READ),
                               op2.op_arg_dat(q, -1, None, 40, "double", op2.OP_WRITE),
                               op2.op_arg_dat(q, -1, None, 40, "double", op2.OP_WRITE))


class Advec:
    """advec/src/advec.cpp:107-262 on the drop-in: one value per node, classical RK4, dt fixed."""

    def __init__(self, op2, m, ops, vel, dt, q0=None):
        o = self.op2 = op2
        N = int(ops["N"])
        Np, Nfp = (N + 1) * (N + 2) // 2, N + 1
        self.Np, self.Nfp, self.dt, self.t = Np, Nfp, dt, 0.0
        o.op_init(0)
        K = self.K = m["cell2nodes"].shape[0]
        nodes = o.op_decl_set(m["coords"].shape[0], "nodes")
        self.cells = cells = o.op_decl_set(K, "cells")
        self.edges = o.op_decl_set(m["edge2cells"].shape[0], "edges")
        self.bedges = o.op_decl_set(m["bedge2cell"].shape[0], "bedges")
        cell2nodes = o.op_decl_map(cells, nodes, 3, m["cell2nodes"], "cell2nodes")
        self.edge2nodes = o.op_decl_map(self.edges, nodes, 2, m["edge2nodes"], "edge2nodes")
        self.edge2cells = o.op_decl_map(self.edges, cells, 2, m["edge2cells"], "edge2cells")
        self.bedge2nodes = o.op_decl_map(self.bedges, nodes, 2, m["bedge2nodes"], "bedge2nodes")
        self.bedge2cells = o.op_decl_map(self.bedges, cells, 1, m["bedge2cell"], "bedge2cells")
        self.nc = nc = o.op_decl_dat(nodes, 2, "double", m["coords"], "node_coords")
        d = {}
        for name, dim in (("nodeX", 3), ("nodeY", 3), ("x", Np), ("y", Np), ("xr", Np), ("yr", Np),
                          ("xs", Np), ("ys", Np), ("rx", Np), ("ry", Np), ("sx", Np), ("sy", Np),
                          ("nx", 3 * Nfp), ("ny", 3 * Nfp), ("fscale", 3 * Nfp), ("rk1", Np), ("rk2", Np),
                          ("rk3", Np), ("rk4", Np), ("exteriorQ", 3 * Nfp)):
            d[name] = (o.op_decl_dat(cells, dim, "double", np.zeros(K * dim), name), dim)
        init = np.zeros(K * Np) if q0 is None else q0
        d["q"] = (o.op_decl_dat(cells, Np, "double", init, "q"), Np)
        d["workingQ"] = (o.op_decl_dat(cells, Np, "double", init, "workingQ"), Np)
        self.d = d
        self.edgeNum = o.op_decl_dat(self.edges, 2, "int", m["edgeNum"], "edgeNum")
        self.bedgeNum = o.op_decl_dat(self.bedges, 1, "int", m["bedgeNum"], "bedgeNum")
        o.op_decl_const2("velX", 1, "double", vel[0])
        o.op_decl_const2("velY", 1, "double", vel[1])
        o.op_decl_const2("ones", Np, "double", np.ones(Np))
        for k in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT"):
            o.op_decl_const2(k, np.asarray(ops[k]).size, "double", np.asarray(ops[k]).ravel())
        o.op_decl_const2("FMASK", 3 * Nfp, "int", np.asarray(ops["FMASK"], dtype=np.int32))
        A = self.A
        o.op_par_loop_init_grid("init_grid", cells, *[o.op_arg_dat(nc, k, cell2nodes, 2, "double", o.OP_READ)
                                                      for k in range(3)],
                                *[A(n, o.OP_WRITE) for n in ("nodeX", "nodeY", "x", "y", "xr", "yr", "xs", "ys",
                                                             "rx", "ry", "sx", "sy", "nx", "ny", "fscale")])
        if q0 is None:
            o.op_par_loop_set_ic("set_ic", cells, A("x", o.OP_READ), A("y", o.OP_READ), A("q", o.OP_WRITE),
                                 A("workingQ", o.OP_WRITE))

    def A(self, name, acc, idx=-1, mp=None):
        dat, dim = self.d[name]
        return self.op2.op_arg_dat(dat, idx, mp, dim, "double", acc)

    def fetch(self, name):
        dat, dim = self.d[name]
        out = np.empty(self.K * dim)
        self.op2.op_fetch_data(dat, out)
        return out

    def run(self, iters):
        o, A, e2c, b2c, nc = self.op2, self.A, self.edge2cells, self.bedge2cells, self.nc
        dt = np.array([self.dt])
        rk_frac = (0.5, 0.5, 1.0)
        for _ in range(iters):
            for j in range(4):
                o.op_par_loop_neighbour_zero("neighbour_zero", self.cells, A("exteriorQ", o.OP_WRITE))
                o.op_par_loop_get_neighbour_q(
                    "get_neighbour_q", self.edges, o.op_arg_dat(self.edgeNum, -1, None, 2, "int", o.OP_READ),
                    o.op_arg_dat(nc, 0, self.edge2nodes, 2, "double", o.OP_READ),
                    o.op_arg_dat(nc, 1, self.edge2nodes, 2, "double", o.OP_READ),
                    A("nodeX", o.OP_READ, 0, e2c), A("nodeY", o.OP_READ, 0, e2c),
                    A("nodeX", o.OP_READ, 1, e2c), A("nodeY", o.OP_READ, 1, e2c),
                    A("workingQ", o.OP_READ, 0, e2c), A("workingQ", o.OP_READ, 1, e2c),
                    A("exteriorQ", o.OP_INC, 0, e2c), A("exteriorQ", o.OP_INC, 1, e2c))
                o.op_par_loop_get_bedge_q(
                    "get_bedge_q", self.bedges, o.op_arg_dat(self.bedgeNum, -1, None, 1, "int", o.OP_READ),
                    o.op_arg_dat(nc, 0, self.bedge2nodes, 2, "double", o.OP_READ),
                    o.op_arg_dat(nc, 1, self.bedge2nodes, 2, "double", o.OP_READ),
                    A("nodeX", o.OP_READ, 0, b2c), A("nodeY", o.OP_READ, 0, b2c),
                    A("x", o.OP_READ, 0, b2c), A("y", o.OP_READ, 0, b2c), A("exteriorQ", o.OP_INC, 0, b2c))
                o.op_par_loop_advec_rhs(
                    "advec_rhs", self.cells, A("workingQ", o.OP_READ), A("exteriorQ", o.OP_READ),
                    A("rx", o.OP_READ), A("ry", o.OP_READ), A("sx", o.OP_READ), A("sy", o.OP_READ),
                    A("fscale", o.OP_READ), A("nx", o.OP_READ), A("ny", o.OP_READ), A("rk%d" % (j + 1), o.OP_WRITE))
                if j != 3:
                    o.op_par_loop_set_workingQ(
                        "set_workingQ", self.cells, o.op_arg_gbl(dt, 1, "double", o.OP_READ), A("q", o.OP_READ),
                        A("rk%d" % (j + 1), o.OP_READ), o.op_arg_gbl(np.array([rk_frac[j]]), 1, "double", o.OP_READ),
                        A("workingQ", o.OP_WRITE))
            o.op_par_loop_update_Q("update_Q", self.cells, o.op_arg_gbl(dt, 1, "double", o.OP_READ),
                                   A("q", o.OP_RW), A("rk1", o.OP_READ), A("rk2", o.OP_READ), A("rk3", o.OP_READ),
                                   A("rk4", o.OP_READ), A("workingQ", o.OP_WRITE))
            self.t += self.dt


@pytest.mark.parametrize("N", [2, 4])
def test_dropin_advec_bitwise_equals_oracle(op2, orc, oops, omesh, N):
    """The advection app's loops: geometry bit-exact, set_ic to the last bits of exp, and, from
    the same initial state, q and all four stage right-hand sides bit for bit after 8 RK4 steps."""
    m = omesh.vortex_square(12, 0.0, 1.0)
    ops, vel, dt = oops.operators(N), (0.8, -0.35), 1e-3
    o = orc.Advection(m, ops, *vel)
    o.init(dt)
    a = Advec(op2, m, ops, vel, dt)
    for name in ("x", "y", "rx", "sy", "nx", "fscale"):
        assert np.array_equal(a.fetch(name), o.get(name)), name
    assert orc.rel_l2(a.fetch("q"), o.get("q")) < 1e-15
    b = Advec(op2, m, ops, vel, dt, q0=o.get("q"))
    b.run(8)
    o.run(8, nthreads=1)
    assert np.array_equal(b.fetch("q"), o.get("q"))
    for k in range(1, 5):
        assert np.array_equal(b.fetch("rk%d" % k), o.get("rk%d" % k)), k


def test_dropin_advec_golden(op2, orc, oops, golden_advec):
    """The reference's advection mesh and run (advec/grid.vtk, 100 RK4 steps) through the drop-in."""
    g, m = golden_advec
    a = Advec(op2, m, oops.operators(4), (1.0, 1.0), float(g["dt"]))
    a.run(100)
    assert orc.rel_l2(a.fetch("q"), g["q100"]) < 1e-11
