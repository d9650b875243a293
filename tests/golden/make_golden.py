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
Each file also holds the mesh tables (coordinates, cells, edge and boundary-edge
tables built with the conventions of tools/vtk2CGNS.cpp), so that tests can run
where the reference tree is absent.

    python tests/golden/make_golden.py
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

REF = "/root/reference"
PERTURB_SEED = 7


def perturbed(q, seed=PERTURB_SEED, amp=0.05):
    rng = np.random.default_rng(seed)
    return q * (1.0 + amp * rng.standard_normal(q.size))


def mesh_arrays(m):
    return {"mesh_" + k: v for k, v in m.items()}


def main():
    if not os.path.isdir(REF):
        raise SystemExit("reference tree not present")
    orc.build(ref=True)
    ops = oo.operators(4)  # ignored by the reference build except for N

    # --- airfoil
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

    # --- vortex
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


if __name__ == "__main__":
    main()
