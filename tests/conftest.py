"""Shared fixtures.  Tests marked gpu need a CUDA device (GB300); the rest run on CPU."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, os.path.join(ROOT, "oracle"))
from oracle import REFERENCE_TREE  # noqa: E402  (one setting: DG_REFERENCE_TREE)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def pkg():
    import __graft_entry__ as g
    mod = g.load_package()
    if not os.path.exists(mod.LIB_PATH):
        mod.build()
    mod.lib()
    return mod


@pytest.fixture(scope="session")
def orc():
    import __graft_entry__ as g
    orc_, om, oo = g.load_oracle()
    if not os.path.exists(orc_.PORT_LIB):
        orc_.build(ref=False)
    return orc_


@pytest.fixture(scope="session")
def omesh():
    import __graft_entry__ as g
    return g.load_oracle()[1]


@pytest.fixture(scope="session")
def oops():
    import __graft_entry__ as g
    return g.load_oracle()[2]


def load_golden(name):
    d = dict(np.load(os.path.join(GOLDEN, name)))
    mesh = {k[5:]: v for k, v in d.items() if k.startswith("mesh_")}
    return d, mesh


@pytest.fixture(scope="session")
def golden_naca():
    return load_golden("naca0012_n4.npz")


@pytest.fixture(scope="session")
def golden_vortex():
    return load_golden("vortex_n4.npz")


@pytest.fixture(scope="session")
def golden_advec():
    d, mesh = load_golden("advec_n4.npz")
    for k in ("rhs_perturbed", "q100"):       # stored sparse: rebuild the dense vector
        a = np.zeros(int(d[k + "_n"]))
        a[d[k + "_idx"]] = d[k + "_val"]
        d[k] = a
    return d, mesh


def reference_tables():
    """The reference's literal N=4 tables, read from its constants headers (only where the
    reference tree exists)."""
    out = {}
    for name in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT"):
        with open(os.path.join(REFERENCE_TREE, "src", "constants", "constant_%s.h" % name)) as f:
            body = f.read().split("{", 1)[1].split("}")[0]
        out[name] = np.array([float(x) for x in body.replace("\n", " ").split(",") if x.strip()])
    return out


def push_affine_geometry(o, geo):
    import __graft_entry__ as g
    g._push_affine_geometry(o, geo)
