"""Solution output (src/save_solution.cpp:13-98): per-vertex rho, u, v, p sampled from each
cell's vertex nodes, the last cell in cell order winning, written out as a file.

The reference writes CGNS (an external library); the framework writes legacy VTK.  CPU tests
check the oracle's restatement against a plain loop over cells in the reference's order and the
writer's round trip; the GPU test checks the device sampling bit for bit against the oracle."""
import numpy as np
import pytest


def loop_restatement(cells, q, N, gam, n_nodes):
    """src/save_solution.cpp:23-46 as a loop (small cases only)."""
    Np = (N + 1) * (N + 2) // 2
    out = np.zeros((4, n_nodes))
    q = q.reshape(-1, Np, 4)
    for c, tri in enumerate(cells.reshape(-1, 3)):
        for node, loc in zip(tri, (0, N, Np - 1)):
            r = q[c, loc, 0]
            u = q[c, loc, 1] / r
            v = q[c, loc, 2] / r
            out[:, node] = r, u, v, (gam - 1) * (q[c, loc, 3] - 0.5 * (q[c, loc, 1] * u + q[c, loc, 2] * v))
    return out


def random_state(K, N, seed):
    Np = (N + 1) * (N + 2) // 2
    rng = np.random.default_rng(seed)
    q = rng.uniform(0.5, 2.0, (K, Np, 4))
    q[..., 3] += 3.0
    return q.reshape(-1)


@pytest.mark.parametrize("N", [1, 3, 4])
def test_oracle_matches_loop(orc, omesh, N):
    m = omesh.naca_ogrid(16, 4)
    q = random_state(len(m["cell2nodes"]), N, N)
    n = len(m["coords"])
    a = orc.vertex_fields(m["cell2nodes"], q, N, 1.4, n)
    b = loop_restatement(np.asarray(m["cell2nodes"]), q, N, 1.4, n)
    assert np.array_equal(a, b)


def test_vtk_writer_round_trip(pkg, orc, omesh, tmp_path):
    m = omesh.naca_ogrid(16, 4)
    mesh = pkg.Mesh.from_tables(m)
    n = mesh.size("nodes")
    f = np.random.default_rng(1).standard_normal((4, n))
    path = tmp_path / "sol.vtk"
    mesh.write_vtk(path, *f)
    d = orc.read_vtk_point_data(path)
    assert np.array_equal(d["rho"], f[0]) and np.array_equal(d["p"], f[3])
    assert np.array_equal(d["velocity"][:, 0], f[1]) and np.array_equal(d["velocity"][:, 1], f[2])
    assert not d["velocity"][:, 2].any()
    # the grid part reads back as the mesh (read_vtk swaps vertices 1 and 2 of each triangle,
    # as the reference's Gmsh converter does, so undo that here)
    coords, cells = omesh.read_vtk(str(path))
    assert np.array_equal(coords, m["coords"])
    assert np.array_equal(np.asarray(cells).reshape(-1, 3)[:, [0, 2, 1]].reshape(-1),
                          np.asarray(m["cell2nodes"]).reshape(-1))


def test_writer_rejects_bad_input(pkg, omesh, tmp_path):
    mesh = pkg.Mesh.from_tables(omesh.naca_ogrid(16, 4))
    n = mesh.size("nodes")
    with pytest.raises(ValueError):
        mesh.write_vtk(tmp_path / "x.vtk", *np.zeros((4, n - 1)))
    with pytest.raises(pkg.DGError):
        mesh.write_vtk(tmp_path / "no_such_dir" / "x.vtk", *np.zeros((4, n)))


@pytest.mark.gpu
@pytest.mark.parametrize("N", [2, 3, 4])
def test_device_vertex_fields_bit_exact(pkg, orc, omesh, N, tmp_path):
    m = omesh.naca_ogrid(64, 16)
    mesh = pkg.Mesh.from_tables(m)
    s = pkg.Solver(mesh, pkg.config(N=N, cfl=0.5, mach=0.5, alpha_deg=3.0)).init()
    s.run(30)
    s.sync()
    got = np.array(s.vertex_fields())
    want = orc.vertex_fields(m["cell2nodes"], s.get("q"), N, 1.4, mesh.size("nodes"))
    assert np.array_equal(got, want)
    s.write_vtk(tmp_path / "sol.vtk")
    d = orc.read_vtk_point_data(tmp_path / "sol.vtk")
    assert np.array_equal(d["rho"], want[0]) and np.array_equal(d["p"], want[3])
