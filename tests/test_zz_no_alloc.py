"""The allocation-free right-hand side (dg_rhs_noalloc, include/dg_gb300.h).

It serves callers that cannot allocate device memory themselves or through us (their memory
belongs to another runtime's pool, or the call may happen during someone else's graph capture):
the face-flux scratch is a fixed device array inside the library.  Its output must equal the
solver's own RHS entry point (dg_solver_rhs, solver-allocated scratch) within the RHS
tolerance of the other tests, on two calls in a row (the second reuses the scratch the
first left behind).  Device buffers for the inputs and output come from torch, as they would
from a caller's own allocator.  This file is collected last on purpose."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RHS_TOL = 1e-13


def kernel_tables(m):
    """edges {cL, cR, fL | fR << 2 | reverse << 4, 0} and bedges {cell, face, type, 0}; reverse as
    src/get_neighbour_q.h:10-34 decides it (vertex fL of L against vertex fR of R)."""
    c2n, xy = m["cell2nodes"], m["coords"]
    cL, cR = m["edge2cells"][:, 0], m["edge2cells"][:, 1]
    fL, fR = m["edgeNum"][:, 0], m["edgeNum"][:, 1]
    vL, vR = c2n[cL, fL], c2n[cR, fR]
    rev = ~np.all(xy[vL] == xy[vR], axis=1)
    edges = np.stack([cL, cR, fL | (fR << 2) | (rev.astype(np.int32) << 4), np.zeros_like(cL)], 1)
    bedges = np.stack([m["bedge2cell"], m["bedgeNum"], m["bedge_type"], np.zeros_like(m["bedgeNum"])], 1)
    return np.ascontiguousarray(edges, dtype=np.int32), np.ascontiguousarray(bedges, dtype=np.int32)


def noalloc_fn(pkg):
    f = pkg.lib().dg_rhs_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(pkg.Config), C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 6
    e = pkg.lib().dg_rhs_noalloc_error
    e.restype = C.c_char_p
    return f, e


def run_twice(pkg, orc, m, cfg, seed):
    """Two allocation-free calls in a row on perturbed states, each against dg_solver_rhs."""
    torch = pytest.importorskip("torch")
    s = pkg.Solver(pkg.Mesh.from_tables(m), cfg).init()
    edges, bedges = kernel_tables(m)
    dev = torch.device("cuda", 0)
    geo_d = torch.from_numpy(s.get("geo")).to(dev)
    edges_d = torch.from_numpy(edges).to(dev)
    bedges_d = torch.from_numpy(bedges).to(dev)
    fn, err = noalloc_fn(pkg)
    rng = np.random.default_rng(seed)
    q = s.get("q")
    stream = torch.cuda.current_stream(dev).cuda_stream
    for _ in range(2):
        W = q * (1.0 + 0.05 * rng.standard_normal(q.size))
        expect = s.rhs(W)
        W_d = torch.from_numpy(W).to(dev)
        out_d = torch.full_like(W_d, float("nan"))
        torch.cuda.synchronize(dev)
        rc = fn(C.byref(cfg), s.K, edges.shape[0], bedges.shape[0], W_d.data_ptr(), geo_d.data_ptr(),
                edges_d.data_ptr(), bedges_d.data_ptr(), out_d.data_ptr(), stream)
        assert rc == 0, err().decode()
        torch.cuda.synchronize(dev)
        got = out_d.cpu().numpy()
        assert np.isfinite(got).all()
        assert orc.rel_l2(got, expect) < RHS_TOL


def test_noalloc_rhs_matches_solver_rhs_twice(pkg, orc, omesh):
    m = omesh.naca_ogrid(64, 16, farfield="characteristic")
    run_twice(pkg, orc, m, pkg.config(N=3, cfl=0.5, mach=0.5, alpha_deg=1.25), 11)


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5, 6])
def test_noalloc_every_order(pkg, orc, omesh, N):
    """Each order takes its own element-kernel form (dense rows on the tensor cores at N = 1, 2,
    the even/odd blocks on the tensor cores at N = 3-5, FP64 at N = 6) and its own tables: every
    one must be set up by the first call on the device, whatever that call's order was."""
    m = omesh.naca_ogrid(16, 8, farfield="characteristic")
    run_twice(pkg, orc, m, pkg.config(N=N, cfl=0.5, mach=0.45, alpha_deg=-1.5), 100 + N)
    lib = pkg.lib()
    assert lib.dg_rhs_noalloc_ready(0) == 1
    assert [lib.dg_order_tables_loaded(0, n) for n in range(1, 7)] == [1] * 6


def test_noalloc_rejects_bad_sizes(pkg):
    """A mesh whose face fluxes exceed the 32 MiB scratch, or whose edge counts cannot cover its
    cell faces exactly once, is refused before any device work."""
    fn, err = noalloc_fn(pkg)
    cfg = pkg.config(N=4)
    fake = 256  # never dereferenced: the size checks come first
    K = 1 << 20
    rc = fn(C.byref(cfg), K, (3 * K - 2) // 2, 2, fake, fake, fake, fake, fake, None)
    assert rc == -1 and b"too large" in err()
    rc = fn(C.byref(cfg), 16, 20, 9, fake, fake, fake, fake, fake, None)
    assert rc == -1 and b"inconsistent" in err()
    rc = fn(C.byref(cfg), 1 << 30, 1 << 30, 1 << 30, fake, fake, fake, fake, fake, None)
    assert rc == -1 and b"too large" in err()
    rc = fn(C.byref(pkg.config(N=3, app=1)), 16, 23, 2, fake, fake, fake, fake, fake, None)
    assert rc == -1 and b"app 0" in err()
