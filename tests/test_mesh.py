"""Mesh tables: the product's C++ builder against the oracle's restatement of
tools/vtk2CGNS.cpp:112-199 and src/load_mesh.cpp:147-171, the golden mesh tables, and
input validation."""
import os

import numpy as np
import pytest

from conftest import REFERENCE_TREE


def same(a, b):
    return set(a) == set(b) and all(np.array_equal(a[k], b[k]) for k in b)


def test_mt19937_64_known_value(omesh):
    g = omesh.MT19937_64(5489)
    for _ in range(9999):
        g()
    assert g() == 9981545732273789042  # the C++ standard's required 10000th value


@pytest.mark.parametrize("farfield", ["reference", "characteristic"])
def test_ogrid_matches_oracle(pkg, omesh, farfield):
    a = pkg.Mesh.naca_ogrid(64, 16, farfield=farfield).arrays()
    b = omesh.naca_ogrid(64, 16, farfield=farfield)
    assert same(a, b)


def test_bench_ogrid_size(pkg):
    m = pkg.Mesh.naca_ogrid(256, 64)
    assert m.size("cells") == 32768
    t = m.arrays()["bedge_type"]
    assert (t == 2).sum() == 256 and (t == 3).sum() == 256


def test_vortex_square_matches_oracle(pkg, omesh):
    a = pkg.Mesh.vortex_square(32).arrays()
    assert a["cell2nodes"].shape == (2048, 3)
    assert same(a, omesh.vortex_square(32))


def test_golden_mesh_rebuilds(pkg, golden_naca):
    _, m = golden_naca
    a = pkg.Mesh.from_cells(m["coords"], m["cell2nodes"]).arrays()
    for k in ("cell2nodes", "edge2nodes", "edge2cells", "edgeNum", "bedge2nodes", "bedge2cell", "bedgeNum"):
        assert np.array_equal(a[k], m[k]), k


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree not present")
def test_vtk_reader_matches_oracle(pkg, omesh):
    path = os.path.join(REFERENCE_TREE, "naca0012.vtk")
    a = pkg.Mesh.read_vtk(path).arrays()
    c, cells = omesh.read_vtk(path)
    b = omesh.build_tables(c, cells)
    b["bedge_type"] = omesh.classify_box(b)
    assert same(a, b)
    assert a["cell2nodes"].shape[0] == 2450 and a["edge2cells"].shape[0] == 3505 and a["bedge2cell"].shape[0] == 340


def test_clockwise_cells_are_fixed(pkg):
    coords = np.array([[0, 0], [1, 0], [0, 1], [1, 1]], dtype=float)
    cells = np.array([[0, 2, 1], [1, 2, 3]])  # first clockwise
    a = pkg.Mesh.from_cells(coords, cells).arrays()
    assert a["cell2nodes"][0].tolist() == [1, 2, 0]
    assert a["edge2cells"].shape == (1, 2) and a["bedge2cell"].shape == (4,)


def test_rejects_bad_tables(pkg, golden_naca):
    _, m = golden_naca
    bad = dict(m)
    bad["edgeNum"] = m["edgeNum"].copy()
    bad["edgeNum"][0, 0] = 3
    with pytest.raises(pkg.DGError):
        pkg.Mesh.from_tables(bad)
    bad = dict(m)
    bad["bedge2cell"] = m["bedge2cell"][:-1]
    bad["bedgeNum"] = m["bedgeNum"][:-1]
    bad["bedge_type"] = m["bedge_type"][:-1]
    with pytest.raises(pkg.DGError, match="covered"):
        pkg.Mesh.from_tables(bad)
    with pytest.raises(pkg.DGError):
        pkg.Mesh.from_cells(m["coords"], np.array([[0, 1, 1 << 20]]))


# ---------------------------------------------------------------- edge tables built on the GPU
def _scrambled(coords, cells, seed):
    """The same triangles with some orientations flipped and the cells shuffled: exercises the
    orientation fix and the side-0 rule (first cell in cell order)."""
    rng = np.random.default_rng(seed)
    c = np.array(cells, dtype=np.int32).reshape(-1, 3)[rng.permutation(len(cells))]
    flip = rng.random(len(c)) < 0.5
    c[flip] = c[flip][:, [0, 2, 1]]
    return np.asarray(coords, dtype=np.float64), c


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["golden", "ogrid", "square", "large"])
def test_device_edge_tables_equal_host(pkg, omesh, golden_naca, case):
    if case == "golden":
        coords, cells = golden_naca[1]["coords"], golden_naca[1]["cell2nodes"]
    elif case == "ogrid":
        m = omesh.naca_ogrid(64, 16)
        coords, cells = m["coords"], m["cell2nodes"]
    else:
        n = 24 if case == "square" else 512     # 524288 cells for "large"
        m = pkg.Mesh.vortex_square(n).arrays()
        coords, cells = m["coords"], m["cell2nodes"]
    coords, cells = _scrambled(coords, cells, 3)
    host = pkg.Mesh.from_cells(coords, cells).arrays()
    dev_mesh = pkg.Mesh.from_cells(coords, cells, device=True)
    dev = dev_mesh.arrays()
    for k in host:
        assert np.array_equal(host[k], dev[k]), k
    assert dev_mesh.build_ms > 0.0


@pytest.mark.gpu
def test_device_edge_tables_reject_bad_cells(pkg, golden_naca):
    coords, cells = golden_naca[1]["coords"], np.array(golden_naca[1]["cell2nodes"])
    bad = cells.copy()
    bad[5, 1] = len(coords)                      # vertex out of range
    with pytest.raises(pkg.DGError):
        pkg.Mesh.from_cells(coords, bad, device=True)
    tri = np.concatenate([cells, cells[:1]])     # an edge shared by three cells
    with pytest.raises(pkg.DGError):
        pkg.Mesh.from_cells(coords, tri, device=True)
    ok = pkg.Mesh.from_cells(coords, cells, device=True)   # the context is still usable
    assert ok.size("cells") == len(cells)
