"""The warp-specialised persistent element kernel (dg_set_elem_ws): one block per SM walks a
range of 32-cell tiles, node warps staging and combining while contraction warps run the tensor-
core product, double-buffered.  Same device functions and operation order as the one-block-per-
tile kernel, so q, the dt sequence and one right-hand side must be bitwise equal to it: at order
3 (the order it serves), with a partial last tile, with fewer tiles than SMs (one tile per block), with many tiles
per block, over cell ranges, for the vortex app and for one RHS."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def with_ws(pkg, mode, fn):
    lib = pkg.lib()
    prev = lib.dg_elem_ws()
    lib.dg_set_elem_ws(mode)
    try:
        return fn()
    finally:
        lib.dg_set_elem_ws(prev)


def steps(pkg, mesh, cfg, n, parts=1):
    def go():
        pkg.set_step_parts(parts)
        try:
            s = pkg.Solver(mesh, cfg).init()
        finally:
            pkg.set_step_parts(0)
        s.record_dt(n)
        s.run(n)
        s.sync()
        return s.get("q"), s.dt_history(n), s.time()
    return go


@pytest.mark.parametrize("N", [3])
@pytest.mark.parametrize("grid", ["small", "large"])
def test_ws_bitwise_equals_tile_kernel(pkg, N, grid):
    # small: 50 tiles, fewer than the SMs (one tile per block, the last one partial: K = 1584);
    # large: 1536 tiles, ~10 per block
    mesh = pkg.Mesh.naca_ogrid(66, 12) if grid == "small" else pkg.Mesh.naca_ogrid(384, 64)
    cfg = pkg.config(N=N, cfl=0.5, mach=0.5, alpha_deg=2.0)
    ref = with_ws(pkg, 0, steps(pkg, mesh, cfg, 12))
    got = with_ws(pkg, 1, steps(pkg, mesh, cfg, 12))
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1]) and got[2] == ref[2]


@pytest.mark.parametrize("mode", [1, 2])
def test_ws_over_ranges_bitwise(pkg, mode):
    mesh = pkg.Mesh.naca_ogrid(256, 64)
    cfg = pkg.config(N=3, cfl=0.5, mach=0.4)
    ref = with_ws(pkg, 0, steps(pkg, mesh, cfg, 8, parts=1))
    got = with_ws(pkg, mode, steps(pkg, mesh, cfg, 8, parts=4))
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])


def test_ws_vortex_and_rhs_bitwise(pkg):
    mesh = pkg.Mesh.vortex_square(40)
    cfg = pkg.config(N=3, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=0.5, vortex_x0=0.0, vortex_y0=0.0,
                     vortex_beta=5.0)
    ref = with_ws(pkg, 0, steps(pkg, mesh, cfg, 20))
    got = with_ws(pkg, 1, steps(pkg, mesh, cfg, 20))
    assert np.array_equal(got[0], ref[0]) and got[2] == ref[2]
    m2 = pkg.Mesh.naca_ogrid(64, 16)
    c2 = pkg.config(N=3, cfl=0.5)

    def rhs():
        s = pkg.Solver(m2, c2).init()
        q = s.get("q")
        W = q * (1.0 + 0.05 * np.random.default_rng(3).standard_normal(q.size))
        return s.rhs(W)
    assert np.array_equal(with_ws(pkg, 1, rhs), with_ws(pkg, 0, rhs))


def test_ws_setting(pkg):
    lib = pkg.lib()
    assert lib.dg_elem_ws() == 0
    for v in (-1, 3, 9):
        lib.dg_set_elem_ws(v)
        assert lib.dg_elem_ws() == 0
    lib.dg_set_elem_ws(0)


def test_two_blocks_per_sm_variant_bitwise(pkg):
    """The order-3 tile kernel compiled for two resident blocks per SM instead of three (more
    registers): the same bits, chain and cell ranges."""
    lib = pkg.lib()
    mesh = pkg.Mesh.naca_ogrid(128, 32)
    cfg = pkg.config(N=3, cfl=0.5, mach=0.45, alpha_deg=1.0)
    ref = steps(pkg, mesh, cfg, 10)()
    prev = lib.dg_elem_blocks_per_sm()
    lib.dg_set_elem_blocks_per_sm(2)
    try:
        assert lib.dg_elem_blocks_per_sm() == 2
        got = steps(pkg, mesh, cfg, 10)()
        got4 = steps(pkg, mesh, cfg, 10, parts=4)()
    finally:
        lib.dg_set_elem_blocks_per_sm(prev)
    assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
    assert np.array_equal(got4[0], ref[0]) and np.array_equal(got4[1], ref[1])
