"""Operator tables: the product's C++ generator, the oracle's numpy restatement and the
reference's literal N=4 tables (src/constants/constant_*.h, FMASK at constant_util.h:15)."""
import os

import numpy as np
import pytest

from conftest import REFERENCE_TREE, reference_tables

NAMES = ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT")


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_cpp_matches_numpy(pkg, oops, N):
    a, b = pkg.operators(N), oops.operators(N)
    tol = {1: 1e-15, 2: 1e-14, 3: 1e-13, 4: 1e-13, 5: 1e-12, 6: 1e-12}[N]
    for k in NAMES:
        assert np.abs(a[k].ravel() - b[k].ravel()).max() < tol, k
    assert np.array_equal(a["FMASK"], b["FMASK"])


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_derivatives_exact_on_polynomials(pkg, N):
    o = pkg.operators(N)
    r, s = o["r"], o["s"]
    for i in range(N + 1):
        for j in range(N + 1 - i):
            f = r ** i * s ** j
            dfr = i * r ** max(i - 1, 0) * s ** j
            dfs = j * r ** i * s ** max(j - 1, 0)
            assert np.abs(o["Dr"] @ f - dfr).max() < 1e-11
            assert np.abs(o["Ds"] @ f - dfs).max() < 1e-11


def test_fmask_n4_is_reference():
    import __graft_entry__ as g
    pkg = g.load_package()
    assert pkg.operators(4)["FMASK"].tolist() == [0, 1, 2, 3, 4, 4, 8, 11, 13, 14, 14, 12, 9, 5, 0]


@pytest.mark.skipif(not os.path.isdir(REFERENCE_TREE), reason="reference tree not present")
def test_n4_matches_reference_tables(pkg):
    ref = reference_tables()
    o = pkg.operators(4)
    for k in NAMES:
        assert np.abs(o[k].ravel() - ref[k]).max() < 3e-14, k
