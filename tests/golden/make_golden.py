"""Generate the golden fixtures from the reference's own kernels.

Runs only where the reference tree is present: it builds oracle/_ref/libref.so
(the reference's src/*.h user kernels and src/constants/*.h N=4 tables, compiled
unmodified with the CBLAS shim) and drives it through the shared oracle driver
on the reference's own meshes:

  naca0012_n4.npz  naca0012.vtk (K=2450, N=4), boundary types of
                   src/load_mesh.cpp:147-171, freestream M=0.4, alpha=0, dt=1/dt1
                   (src/airfoil.cpp:79-99,237,331):
                     dt0, rhs of a seeded perturbed state, q and dt after 10 and
                     1000 SSPRK3 steps.
  vortex_n4.npz    vortex/grid.vtk (K=618, N=4), isentropic vortex x0=5, beta=5,
                   dt = 0.1/dt1 frozen (vortex/src/vortex.cpp:209-306): q and the
                   L2 error sums after 100 steps.
  advec_n4.npz     advec/grid.vtk (K=23252, N=4), scalar advection with velocity
                   (1, 1) and dt = 0.001 (advec/src/advec.cpp:197): the RHS of a
                   seeded perturbed state and q after 100 RK4 steps (the app's
                   default -iter).  Both are stored sparse (entries of magnitude at least
                   1e-16 of the largest, with the relative L2 of the rest, below 4e-16):
                   the boundary ghost value seeds a tail of tiny values that would not
                   compress.
Each file also holds the mesh tables (coordinates, cells, edge and boundary-edge
tables built with the conventions of tools/vtk2CGNS.cpp), so that tests can run
where the reference tree is absent.

    python tests/golden/make_golden.py [naca] [vortex] [advec]   (default: all)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import mesh as om  # noqa: E402
import operators as oo  # noqa: E402
import oracle as orc  # noqa: E402

REF = orc.REFERENCE_TREE  # DG_REFERENCE_TREE, see oracle/oracle.py
PERTURB_SEED = 7


def perturbed(q, seed=PERTURB_SEED, amp=0.05):
    rng = np.random.default_rng(seed)
    return q * (1.0 + amp * rng.standard_normal(q.size))


def mesh_arrays(m):
    return {"mesh_" + k: v for k, v in m.items()}


def make_naca(ops):
    coords, cells = om.read_vtk(os.path.join(REF, "naca0012.vtk"))
    m = om.build_tables(coords, cells)
    m["bedge_type"] = om.classify_box(m)
    phys = orc.freestream(0.4, 0.0)
    o = orc.Oracle(m, ops, phys, app=orc.APP_AIRFOIL, kind="reference")
    o.init(1.0)
    dt0 = o.dt
    q0 = o.get("q")
    W = perturbed(q0)
    o.set("workingQ", W)
    rhs_p = o.rhs(0)
    o.set("workingQ", q0)
    o2 = orc.Oracle(m, ops, phys, app=orc.APP_AIRFOIL, kind="reference")
    o2.init(1.0)
    dt10 = o2.run(10, nthreads=1)
    q10 = o2.get("q")
    dt1000 = np.concatenate([dt10, o2.run(990, nthreads=8)])
    q1000 = o2.get("q")
    np.savez_compressed(os.path.join(HERE, "naca0012_n4.npz"), dt0=dt0, rhs_perturbed=rhs_p,
                        perturb_seed=PERTURB_SEED, q10=q10, dt10=dt10, q1000=q1000, dt1000=dt1000,
                        t1000=o2.t, **mesh_arrays(m))
    print("naca0012: K=%d dt0=%.17g t1000=%.17g" % (o.K, dt0, o2.t))


def make_vortex(ops):
    coords, cells = om.read_vtk(os.path.join(REF, "vortex", "grid.vtk"))
    mv = om.build_tables(coords, cells)
    mv["bedge_type"] = np.zeros(mv["bedge2cell"].shape[0], dtype=np.int32)
    physv = orc.freestream(0.4, 0.0)
    physv.update(vortex_x0=5.0, vortex_y0=0.0, vortex_beta=5.0)
    v = orc.Oracle(mv, ops, physv, app=orc.APP_VORTEX, kind="reference")
    v.init(0.1)
    dtv = v.dt
    v.run(100, dt_mode=orc.DT_FROZEN, nthreads=1)
    np.savez_compressed(os.path.join(HERE, "vortex_n4.npz"), dt=dtv, q100=v.get("q"), t100=v.t,
                        l2_100=v.l2_error(), **mesh_arrays(mv))
    print("vortex: K=%d dt=%.17g l2=%s" % (v.K, dtv, v.l2_error()))


def sparse(name, a, rel=1e-16):
    """{name_idx, name_val, name_n, name_dropped}: the entries with |a| >= rel * max|a|."""
    keep = np.abs(a) >= rel * np.abs(a).max()
    dropped = np.linalg.norm(a[~keep]) / np.linalg.norm(a)
    return {name + "_idx": np.flatnonzero(keep).astype(np.int32), name + "_val": a[keep],
            name + "_n": a.size, name + "_dropped": dropped}


def make_advec(ops):
    coords, cells = om.read_vtk(os.path.join(REF, "advec", "grid.vtk"))
    m = om.build_tables(coords, cells)
    a = orc.Advection(m, ops, 1.0, 1.0, kind="reference")
    a.init(1e-3)
    q0 = a.get("q")
    a.set("workingQ", perturbed(q0, amp=0.5))
    rhs_p = a.rhs(0)
    a.set("workingQ", q0)
    a.run(100, nthreads=8)
    np.savez_compressed(os.path.join(HERE, "advec_n4.npz"), dt=1e-3, vel=np.array([1.0, 1.0]),
                        perturb_seed=PERTURB_SEED, perturb_amp=0.5, t100=a.t,
                        **sparse("rhs_perturbed", rhs_p), **sparse("q100", a.get("q")),
                        **mesh_arrays(m))
    print("advec: K=%d t100=%.17g" % (a.K, a.t))


def main(which):
    if not os.path.isdir(REF):
        raise SystemExit("reference tree not present")
    orc.build(ref=True)
    ops = oo.operators(4)  # ignored by the reference build except for N
    makers = {"naca": make_naca, "vortex": make_vortex, "advec": make_advec}
    for name in which or list(makers):
        makers[name](ops)


if __name__ == "__main__":
    main(sys.argv[1:])
