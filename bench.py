"""Benchmark: DOF-stage updates/s of the FP64 DG Euler RHS + SSPRK3 step on one GB300.

Workload (the plain-method airfoil case): NACA 0012 O-grid, 256 x 64 cells
layers (K = 2*256*64 = 32768 triangles), polynomial order N = 3 (Np = 10),
Mach 0.4, alpha 0, slip wall + characteristic farfield, SSPRK3 at CFL 0.5 with
dt recomputed after every step.  One bench step = one SSPRK3 time step (three
RHS evaluations) over the whole mesh; DOF = one conserved variable at one node,
so a step is 3 * 4 * K * Np DOF-stage updates.  Synthetic mesh and freestream
initial state (the reference publishes no benchmark data set).

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl gb300|reference]

value   device-resident: CUDA events around each step's graph launch on the
        solver stream, L2 flushed (512 MB write) between steps outside the events.
e2e     the C-ABI call dg_solver_step_host with pinned host buffers: H2D of q,
        one step, D2H of q, timed with events on the same stream.
roofline  FP64-bound: algorithmic flops of the dominant kernel per launch over
        its event-timed launch duration (dg_solver_step_timed), against the DFMA
        peak measured live on this GPU.
--impl reference  the CPU oracle (the reference's user kernels, restated, driven
        OP2-openmp style on all host cores) on the same workload.
Multi-GPU: replicas only (the path is one mesh per GPU); each rank runs the
workload, times are maxed over ranks, value = total DOF-stages / time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_ORDER = 3
N_THETA, N_R = 256, 64
MACH, ALPHA, CFL = 0.4, 0.0, 0.5
METRIC = "DOF-stage updates/s FP64 on 1 GB300 (plain vs batched); adjoint/forward time at 1e-11"
WORKLOAD = "naca0012_ogrid_256x64_K32768_N3_M0.4_a0_cfl0.5"


def np_of(n):
    return (n + 1) * (n + 2) // 2


def elem_flops(n):
    """Algorithmic FP64 flops of elem_kernel per cell and stage (FMA = 2):
    volume contraction [Drw|Dsw] on metric-combined fluxes 16 Np^2, lift 24 Np Nfp,
    nodal flux + metric combine 36 Np, SSPRK3 combine 16 Np."""
    p, f = np_of(n), n + 1
    return 16 * p * p + 24 * p * f + 36 * p + 16 * p


def face_flops(n):
    """Algorithmic flops of face_kernel per face node: Roe flux (rotation, Roe averages,
    wave strengths, dissipation, rotation back; rsqrt/rcp counted as 1) plus fscale scaling."""
    return 150


def survey_flops(n):
    """The reference algorithm's flops per cell-stage (4-GEMV volume form, Roe on every
    cell face): 32 Np^2 + 24 Np Nfp + 60 Np + 330 Nfp."""
    p, f = np_of(n), n + 1
    return 32 * p * p + 24 * p * f + 60 * p + 330 * f


def algo_bytes(n):
    """Algorithmic HBM bytes per cell-stage of the fused path: 8 (32 Np/3 + 12 Nfp + 16)."""
    p, f = np_of(n), n + 1
    return 8 * (32 * p / 3 + 12 * f + 16)


class Clocks:
    """nvidia-smi sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world <= 1:
        return None, 0, 1
    import torch.distributed as dist
    backend = "gloo"
    dist.init_process_group(backend=backend)
    return dist, dist.get_rank(), world


def dist_max(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_oracle_rate(steps, nthreads, warmup=1):
    """DOF-stage/s of the CPU oracle on the bench workload (bounded sample of `steps` steps)."""
    import __graft_entry__ as g
    orc, om, oo = g.load_oracle()
    if not os.path.exists(orc.PORT_LIB):
        orc.build(ref=False)
    m = om.naca_ogrid(N_THETA, N_R, farfield="characteristic")
    o = orc.Oracle(m, oo.operators(N_ORDER), orc.freestream(MACH, ALPHA), kind="port")
    o.init(CFL)
    if warmup:
        o.run(warmup, nthreads=nthreads)
    t0 = time.perf_counter()
    o.run(steps, nthreads=nthreads)
    dt = time.perf_counter() - t0
    K = o.K
    return 3 * 4 * K * np_of(N_ORDER) * steps / dt, dt


def batched_measure(pkg, steps, n_inst=64, seed=20261203):
    """The batched sweep: 64 O-grid airfoil instances, alpha ~ U[-4,8], M ~ U[0.3,0.6] (seed
    20261203), grids 128x32 .. 384x96 (K 8192 .. 73728), N=3/4 alternating, CFL 0.5; one
    persistent kernel per RK stage (autotuned shape) vs the same instances on the plain path
    (each its own solver, all enqueued on their own streams, then synchronised)."""
    sc = pkg.sweep_config(n_inst, seed)
    meshes = [pkg.Mesh.naca_ogrid(c["n_theta"], c["n_r"]) for c in sc]
    cfgs = [pkg.config(N=c["N"], cfl=CFL, mach=c["mach"], alpha_deg=c["alpha_deg"]) for c in sc]
    cells = sum(m.size("cells") for m in meshes)
    dof = sum(m.size("cells") * np_of(c.N) * 4 for m, c in zip(meshes, cfgs))
    b = pkg.Batch(meshes, cfgs).init()
    tuned = b.autotune(2)
    b.run(3)
    b.sync()
    evs = [(pkg.Event(), pkg.Event()) for _ in range(steps)]
    for i in range(steps):  # inputs (~3.7 GB) far exceed L2: no flush needed
        evs[i][0].record(b.stream)
        b.run(1)
        evs[i][1].record(b.stream)
    b.sync()
    bms = sum(a.elapsed_ms(c) for a, c in evs) / steps
    solvers = [pkg.Solver(m, c).init() for m, c in zip(meshes, cfgs)]
    for s in solvers:
        s.run(2)
    for s in solvers:
        s.sync()
    psteps = max(3, steps // 4)
    t0 = time.perf_counter()
    for _ in range(psteps):
        for s in solvers:
            s.run(1)
        for s in solvers:
            s.sync()
    pms = (time.perf_counter() - t0) / psteps * 1e3
    # the plain path one instance at a time (each instance's steps, then the next)
    t0 = time.perf_counter()
    for s in solvers:
        s.run(psteps)
        s.sync()
    sms = (time.perf_counter() - t0) / psteps * 1e3
    del solvers
    return {"value": 3 * dof / (bms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": bms, "steps": steps,
            "instances": n_inst, "cells": cells, "dof_stage_per_step": 3 * dof, "shape": b.shape(),
            "autotune_ms_per_step": tuned,
            "plain_same_instances": {"value": 3 * dof / (pms * 1e-3), "ms_per_step": pms,
                                     "how": "64 plain solvers, each on its own stream, host-timed"},
            "plain_sequential": {"value": 3 * dof / (sms * 1e-3), "ms_per_step": sms,
                                 "how": "the 64 plain solvers one after another, host-timed"},
            "speedup_vs_plain": pms / bms, "speedup_vs_plain_sequential": sms / bms}


def batched_small_measure(pkg, steps=100, n_inst=64, seed=20261203):
    """Where batching pays: 64 small instances (O-grids 32x8 .. 64x16, K 512 .. 2048, N=3/4,
    the sweep's alpha and Mach), launch-bound on the plain path (7 launches per instance-step)."""
    sc = pkg.sweep_config(n_inst, seed)
    meshes, cfgs = [], []
    for i, c in enumerate(sc):
        f = i / (n_inst - 1)
        meshes.append(pkg.Mesh.naca_ogrid(int(round(32 + 32 * f)), int(round(8 + 8 * f))))
        cfgs.append(pkg.config(N=c["N"], cfl=CFL, mach=c["mach"], alpha_deg=c["alpha_deg"]))
    dof = sum(m.size("cells") * np_of(c.N) * 4 for m, c in zip(meshes, cfgs))
    b = pkg.Batch(meshes, cfgs).init()
    b.autotune(3)
    b.run(3)
    b.sync()
    e0, e1 = pkg.Event(), pkg.Event()
    e0.record(b.stream)
    b.run(steps)
    e1.record(b.stream)
    b.sync()
    bms = e0.elapsed_ms(e1) / steps
    solvers = [pkg.Solver(m, c).init() for m, c in zip(meshes, cfgs)]
    for s_ in solvers:
        s_.run(2)
    for s_ in solvers:
        s_.sync()
    t0 = time.perf_counter()
    for s_ in solvers:
        s_.run(steps)
    for s_ in solvers:
        s_.sync()
    pms = (time.perf_counter() - t0) / steps * 1e3
    t0 = time.perf_counter()
    for s_ in solvers:
        s_.run(steps)
        s_.sync()
    sms = (time.perf_counter() - t0) / steps * 1e3
    return {"value": 3 * dof / (bms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": bms, "instances": n_inst,
            "cells": sum(m.size("cells") for m in meshes), "shape": b.shape(),
            "plain_same_instances": {"value": 3 * dof / (pms * 1e-3), "ms_per_step": pms,
                                     "how": "64 plain solvers, graph launches on their own streams, host-timed"},
            "plain_sequential": {"value": 3 * dof / (sms * 1e-3), "ms_per_step": sms,
                                 "how": "the 64 plain solvers one after another, host-timed"},
            "speedup_vs_plain": pms / bms, "speedup_vs_plain_sequential": sms / bms}


def adjoint_measure(pkg, nsteps=2000, navg=100, C=50):
    """The adjoint case: NACA 0012 O-grid 256x64 (K=32768), N=3, M=0.5, alpha=2 deg, inflow /
    outflow farfield typing (the adjoint covers boundary types 0-2), J = mean C_l over the last
    100 of 2000 steps, checkpoints every 50 steps.  Reports forward and backward device times, the
    adjoint/forward cost ratio and a central-difference check of dJ/dalpha (h = 1e-6)."""
    mesh = pkg.Mesh.naca_ogrid(N_THETA, N_R, farfield="reference")
    cfg = pkg.config(N=N_ORDER, cfl=CFL, mach=0.5, alpha_deg=2.0)
    obj = pkg.LiftObjective(mesh, cfg, nsteps, navg, C)
    a, b, c = pkg.Event(), pkg.Event(), pkg.Event()
    a.record(obj.stream)
    J = obj.forward()
    b.record(obj.stream)
    ga, _ = obj.backward(want_q0=False)
    c.record(obj.stream)
    fwd_ms, bwd_ms = a.elapsed_ms(b), b.elapsed_ms(c)
    h = 1e-6
    fd = (obj.evaluate(2.0 + h) - obj.evaluate(2.0 - h)) / (2 * h)
    t0 = time.perf_counter()
    tan = obj.tangent(1.0)
    tan_s = time.perf_counter() - t0
    return {"J_mean_cl": J, "dJ_dalpha_deg": ga, "fd_dJ_dalpha_deg": fd,
            "fd_rel_diff": abs(ga - fd) / max(abs(fd), 1e-300),
            "tangent_dJ_dalpha_deg": tan, "tangent_rel_diff": abs(ga - tan) / max(abs(tan), 1e-300),
            "tangent_s": tan_s, "forward_ms": fwd_ms, "backward_ms": bwd_ms,
            "adjoint_over_forward": bwd_ms / fwd_ms, "steps": nsteps, "avg_last": navg,
            "checkpoint_every": C, "cells": mesh.size("cells"), "order": N_ORDER,
            "note": "backward = segment recomputation from checkpoints + reverse sweep"}


def advection_measure(pkg, steps=200, n=512, order=4, cpu_steps=40):
    """The scalar advection app (advec/src/advec.cpp) at scale: [0,10]^2 cut into 2 n^2 = 524288
    triangles, order 4, velocity (1, 1), dt = 1e-3, classical RK4 (four stages a step).  Device
    steps are CUDA-graph launches timed with events (q, W and the RK accumulator, 3 x 63 MB, exceed
    L2); per-kernel times from separately launched steps; the CPU oracle on the same mesh (all
    cores, a few steps) beside it."""
    mesh = pkg.Mesh.vortex_square(n, 0.0, 10.0)
    K = mesh.size("cells")
    Np = np_of(order)
    a = pkg.Advection(mesh, N=order, vel_x=1.0, vel_y=1.0, dt=1e-3).init()
    a.run(3)
    a.sync()
    evs = [(pkg.Event(), pkg.Event()) for _ in range(steps)]
    for i in range(steps):
        evs[i][0].record(a.stream)
        a.run(1)
        evs[i][1].record(a.stream)
    a.sync()
    ms = sum(x.elapsed_ms(y) for x, y in evs) / steps
    per = [a.step_timed() for _ in range(20)]
    face_ms = sum(sum(p[0::2]) for p in per) / len(per)
    elem_ms = sum(sum(p[1::2]) for p in per) / len(per)
    Nfp = order + 1
    # element kernel, per cell and stage: the contraction 2 (2 Np^2 + 3 Nfp Np), the metric
    # combine 2 Np + 6 and the RK4 combine 3 Np
    flops = K * (2 * (2 * Np * Np + 3 * Nfp * Np) + 5 * Np + 6)
    import __graft_entry__ as g
    orc, om, oo = g.load_oracle()
    if not os.path.exists(orc.PORT_LIB):
        orc.build(ref=False)
    o = orc.Advection(om.vortex_square(n, 0.0, 10.0), oo.operators(order), 1.0, 1.0)
    o.init(1e-3)
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o.run(cpu_steps, nthreads=nthreads)
    cpu_s = time.perf_counter() - t0
    dof_stage = 4 * K * Np
    return {"value": dof_stage / (ms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": ms, "steps": steps,
            "cells": K, "order": order, "kernels_per_step": 8,
            "face_kernel_ms_per_stage": face_ms / 4, "elem_kernel_ms_per_stage": elem_ms / 4,
            "elem_kernel_tflops_dense_equivalent": flops / (elem_ms / 4 * 1e-3) / 1e12,
            "flops_note": "dense-row count 2(2Np^2 + 3 Nfp Np) + 5Np + 6 per cell-stage; the even/odd kernel "
                          "executes about 0.6 of it",
            "cpu_oracle": {"value": cpu_steps * dof_stage / cpu_s, "unit": "DOF-stage/s", "cores": nthreads,
                           "sample": "%d RK4 steps of the same mesh (%.1f s)" % (cpu_steps, cpu_s)}}


def mesh_setup_measure(pkg, n=1024):
    """Edge-table construction for [0,10]^2 cut into 2 n^2 = 2,097,152 triangles: the host build
    (stable sort) against the device build (radix sort, scan, scatter), same tables."""
    m = pkg.Mesh.vortex_square(n, 0.0, 10.0).arrays()
    coords, cells = m["coords"], m["cell2nodes"]
    w = pkg.Mesh.vortex_square(8).arrays()
    pkg.Mesh.from_cells(w["coords"], w["cell2nodes"], device=True)  # warm the context and the sort
    t0 = time.perf_counter()
    h = pkg.Mesh.from_cells(coords, cells)
    host_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    d = pkg.Mesh.from_cells(coords, cells, device=True)
    call_ms = (time.perf_counter() - t0) * 1e3
    same = all(np.array_equal(a, b) for a, b in zip(h.arrays().values(), d.arrays().values()))
    return {"cells": len(cells), "host_build_ms": host_ms, "device_build_ms": d.build_ms,
            "device_call_ms": call_ms, "identical_tables": same,
            "note": "device_call_ms includes host<->device copies and host validation"}


def large_vortex_measure(pkg, n=512, orders=(1, 2, 3, 4, 5), steps=200, n_inst=16, grad_order=2, C=14,
                         seed=20261203):
    """Large vortex convergence plus batched gradient: [-5,5]^2 cut into 2 n^2 = 524288 triangles,
    the vortex (beta 5 at the origin, dt = 0.5/dt1 frozen) run 200 steps at each order N=1..5 with
    its L2 error against the analytic state; then 16 instances with beta ~ U[3,7] (numpy seed
    20261203), the gradient of each instance's final-time squared error with respect to beta in one
    batched forward and one batched backward (order 2, checkpoints every 14 steps), and a central
    difference check (h = 1e-6) of the first instance."""
    mesh = pkg.Mesh.vortex_square(n)
    conv = []
    for N in orders:
        cfg = pkg.config(N=N, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=CFL, vortex_x0=0.0, vortex_y0=0.0,
                         vortex_beta=5.0)
        s = pkg.Solver(mesh, cfg).init()
        s.run(1)
        s.sync()
        s = pkg.Solver(mesh, cfg).init()
        a, b = pkg.Event(), pkg.Event()
        a.record(s.stream)
        s.run(steps)
        b.record(s.stream)
        s.sync()
        ms = a.elapsed_ms(b)
        t, dt, _ = s.time()
        err = s.l2_error()
        dofs = mesh.size("cells") * np_of(N) * 4
        conv.append({"N": N, "dt": dt, "t_end": t, "l2_error_sums": [float(x) for x in err],
                     "rms_error": float(np.sqrt(err.sum() / dofs)), "ms": ms,
                     "dof_stage_per_s": 3 * dofs * steps / (ms * 1e-3)})
    betas = np.random.default_rng(seed).uniform(3.0, 7.0, n_inst)
    objs = [pkg.LiftObjective(mesh, pkg.config(N=grad_order, app=pkg.APP_VORTEX, dt_mode=pkg.DT_FROZEN, cfl=CFL,
                                               vortex_x0=0.0, vortex_y0=0.0, vortex_beta=float(bb)), steps, 1, C)
            for bb in betas]
    t0 = time.perf_counter()
    J = pkg.adjoint_batch_forward(objs)
    fwd_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    g, _ = pkg.adjoint_batch_backward(objs)
    bwd_s = time.perf_counter() - t0
    h = 1e-6
    fd = (objs[0].evaluate(betas[0] + h) - objs[0].evaluate(betas[0] - h)) / (2 * h)
    del objs
    return {"cells": mesh.size("cells"), "steps": steps, "convergence": conv,
            "batched_gradient": {"instances": n_inst, "order": grad_order, "checkpoint_every": C,
                                 "beta": [float(x) for x in betas], "J": [float(x) for x in J],
                                 "dJ_dbeta": [float(x) for x in g], "forward_s": fwd_s, "backward_s": bwd_s,
                                 "backward_over_forward": bwd_s / fwd_s,
                                 "fd_check_instance0": {"fd": fd, "adjoint": float(g[0]),
                                                        "rel_diff": abs(g[0] - fd) / max(abs(fd), 1e-300)}}}


def run_reference(args):
    """The reference arm: the reference's user kernels (restated; the reference's own build is
    N=4-only and cannot run this N=3 workload) on all host cores."""
    dist, rank, world = dist_init()
    if rank != 0:
        return 0
    import __graft_entry__ as g
    orc, om, oo = g.load_oracle()
    if not os.path.exists(orc.PORT_LIB):
        orc.build(ref=False)
    nthreads = os.cpu_count() or 1
    m = om.naca_ogrid(N_THETA, N_R, farfield="characteristic")
    o = orc.Oracle(m, oo.operators(N_ORDER), orc.freestream(MACH, ALPHA), kind="port")
    o.init(CFL)
    o.run(args.warmup, nthreads=nthreads)
    t0 = time.perf_counter()
    o.run(args.steps, nthreads=nthreads)
    el = time.perf_counter() - t0
    K = o.K
    value = 3 * 4 * K * np_of(N_ORDER) * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "DOF-stage/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "cells": K, "order": N_ORDER, "l2": "cpu (n/a)"},
        "cpu_baseline": {"value": value, "unit": "DOF-stage/s", "cores": nthreads, "kind": "port",
                         "sample": "%d SSPRK3 steps of the full K=%d N=3 workload" % (args.steps, K)},
        "e2e": {"value": value, "unit": "DOF-stage/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-steps", type=int, default=1500,
                    help="CPU-baseline sample size (steps; ~10 s on 16 Grace cores)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--batched-steps", type=int, default=20)
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-advection", action="store_true")
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--advection-steps", type=int, default=200)
    ap.add_argument("--large-vortex", action="store_true",
                    help="also run the large vortex convergence + 16-instance batched beta gradient (~1 min)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    dist, rank, world = dist_init()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:  # replicas: one GPU per rank
        vis = os.environ.get("CUDA_VISIBLE_DEVICES")
        devs = vis.split(",") if vis else [str(i) for i in range(world)]
        os.environ["CUDA_VISIBLE_DEVICES"] = devs[local % len(devs)]
    import __graft_entry__ as g
    pkg = g.load_package()
    pkg.lib()

    mesh = pkg.Mesh.naca_ogrid(N_THETA, N_R, farfield="characteristic")
    cfg = pkg.config(N=N_ORDER, cfl=CFL, mach=MACH, alpha_deg=ALPHA)
    s = pkg.Solver(mesh, cfg).init()
    K, Np = s.K, np_of(N_ORDER)
    dof_stage_per_step = 3 * 4 * K * Np
    stream = s.stream
    peak_gflops = pkg.fp64_peak_gflops()
    dmma_gflops = pkg.fp64_mma_peak_gflops()

    # warm-up (graph capture happens on the first run)
    s.run(args.warmup)
    s.sync()

    # timed region: device-resident steps, L2 flushed between steps outside the events
    evs = [(pkg.Event(), pkg.Event()) for _ in range(args.steps)]
    barrier(dist)
    clocks = Clocks(local)
    for i in range(args.steps):
        pkg.l2_flush(stream)
        evs[i][0].record(stream)
        s.run(1)
        evs[i][1].record(stream)
    s.sync()
    clk = clocks.stop()
    step_ms = [a.elapsed_ms(b) for a, b in evs]
    total_ms = dist_max(dist, sum(step_ms))
    barrier(dist)
    ms_per_step = total_ms / args.steps
    value = world * dof_stage_per_step * args.steps / (total_ms * 1e-3)

    # per-kernel durations (same workload, separate launches with events between kernels)
    nk = min(args.steps, 50)
    kt = np.zeros(7)
    for _ in range(nk):
        pkg.l2_flush(stream)
        kt += s.step_timed()
    kt /= nk
    face_ms = float(np.mean(kt[[0, 2, 4]]))
    elem_ms = float(np.mean(kt[[1, 3, 5]]))
    nf = (mesh.size("edges") + mesh.size("bedges")) * (N_ORDER + 1)
    elem_tf = elem_flops(N_ORDER) * K / (elem_ms * 1e-3) * 1e-12
    face_tf = face_flops(N_ORDER) * nf / (face_ms * 1e-3) * 1e-12
    step_tf = survey_flops(N_ORDER) * K / ((face_ms + elem_ms) * 1e-3) * 1e-12
    dominant = "elem_kernel" if elem_ms >= face_ms else "face_kernel"
    peak_tf = peak_gflops * 1e-3
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak = float(json.load(f)["hbm_gbs"])
        hbm_src = "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        hbm_peak, hbm_src = 6800.0, "fallback"
    traffic = None
    try:  # ncu-measured DRAM bytes per element-kernel launch (stage average), committed profile
        with open(os.path.join(ROOT, "profiles", "elem_kernel_sym_face_kernel_naca_ogrid_K32768_N3.md")) as f:
            for ln in f:
                if ln.startswith("traffic_bytes_per_launch_elem_kernel:"):
                    traffic = float(ln.split(":")[1])
    except OSError:
        traffic = None
    stage_bytes = algo_bytes(N_ORDER) * K
    hbm_gbs = stage_bytes / ((face_ms + elem_ms) * 1e-3) * 1e-9
    # the element kernel in its all-FP64 even/odd form on the same workload, for comparison
    variant = pkg.lib().dg_elem_variant()
    elem_ms_fp64 = None
    if variant >= 2:
        pkg.lib().dg_set_elem_variant(1)
        try:
            s64 = pkg.Solver(mesh, pkg.config(N=N_ORDER, cfl=CFL)).init()
            k64 = np.zeros(7)
            for _ in range(3):
                s64.step_timed()
            for _ in range(nk):
                pkg.l2_flush(stream)
                k64 += s64.step_timed()
            elem_ms_fp64 = float(np.mean(k64[[1, 3, 5]])) / nk
            del s64
        finally:
            pkg.lib().dg_set_elem_variant(variant)

    # end to end through the C ABI with pinned host buffers
    nq = K * Np * 4
    h_in, h_out = pkg.PinnedArray(nq), pkg.PinnedArray(nq)
    h_in.array[:] = s.get("q")
    e2e_steps = min(args.steps, 100)
    e2e_ms = 0.0
    for i in range(e2e_steps):
        pkg.l2_flush(stream)
        a, b = pkg.Event(), pkg.Event()
        a.record(stream)
        s.step_host(h_in.array, 1, h_out.array)
        b.record(stream)
        e2e_ms += a.elapsed_ms(b)
    e2e_ms = dist_max(dist, e2e_ms)
    e2e_value = world * dof_stage_per_step * e2e_steps / (e2e_ms * 1e-3)
    s.sync()

    line = {
        "metric": METRIC, "value": value, "unit": "DOF-stage/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (generated O-grid, freestream start)",
        "config": {"workload": WORKLOAD, "cells": K, "order": N_ORDER, "np": Np,
                   "dof_stage_per_step": dof_stage_per_step, "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between timed steps (512 MB write outside the events)",
                   "graph": "one CUDA graph launch per step (7 kernels)"},
        "gpu_launches": 7 * args.steps,
        "nodes_per_s": value / 4,
        "roofline": {"bound": "fp64", "kernel": dominant, "achieved": elem_tf if dominant == "elem_kernel" else face_tf,
                     "peak": peak_tf, "unit": "TFLOP/s",
                     "frac": (elem_tf if dominant == "elem_kernel" else face_tf) / peak_tf,
                     "traffic": traffic if dominant == "elem_kernel" else None,
                     "traffic_source": "ncu dram__bytes_read+write per launch, stage average (profiles/)",
                     "peak_source": "DFMA throughput measured live on this GPU (MEASURED_PEAKS.json has no FP64 figure)",
                     "elem_form": {3: "even/odd, contraction and butterfly on the bf16 tensor cores (exact integer product)",
                                   2: "even/odd, contraction on the bf16 tensor cores (exact integer product)",
                                   1: "even/odd, FP64", 0: "dense FP64"}[variant],
                     "frac_note": ("FP64-equivalent: algorithmic FP64 flops over the DFMA peak; the contraction "
                                   "runs on the tensor cores, so frac can exceed 1 (FP64 pipe busy 45-50 % of "
                                   "active cycles per ncu)") if variant >= 2 else "FP64 flops over the DFMA peak",
                     "elem_ms_fp64_form": elem_ms_fp64,
                     "fp64_tensor_peak_tflops": dmma_gflops * 1e-3,
                     "fp64_tensor_note": "DMMA (mma.sync m8n8k4 f64) measured live; below DFMA and on the same pipe, so unused",
                     "flops_per_unit": elem_flops(N_ORDER) if dominant == "elem_kernel" else face_flops(N_ORDER),
                     "unit_def": "cell-stage" if dominant == "elem_kernel" else "face node",
                     "kernel_ms": {"face": face_ms, "elem": elem_ms, "elem_stage2": float(kt[5]),
                                   "finalize": float(kt[6])},
                     "face_kernel_tflops": face_tf,
                     "step_tflops_survey_count": step_tf,
                     "hbm": {"achieved": hbm_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": hbm_gbs / hbm_peak,
                             "peak_source": hbm_src}},
        "e2e": {"value": e2e_value, "unit": "DOF-stage/s", "h2d_bytes_per_step": nq * 8,
                "d2h_bytes_per_step": nq * 8, "steps": e2e_steps,
                "call": "dg_solver_step_host (pinned host q in/out, 1 step per call)"},
        "clocks": clk,
    }
    if rank == 0 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        rate, secs = cpu_oracle_rate(args.cpu_steps, nthreads)
        line["cpu_baseline"] = {"value": rate, "unit": "DOF-stage/s", "cores": nthreads, "kind": "port",
                                "sample": "%d SSPRK3 steps of the full workload (%.1f s)" % (args.cpu_steps, secs)}
        one_steps = max(1, args.cpu_steps // 16)
        rate1, secs1 = cpu_oracle_rate(one_steps, 1)
        line["cpu_baseline"]["single_core"] = {"value": rate1, "cores": 1,
                                               "sample": "%d steps (%.1f s)" % (one_steps, secs1)}
    if not args.no_batched:
        line["batched"] = batched_measure(pkg, args.batched_steps)
        line["batched"]["small_instances"] = batched_small_measure(pkg)
    if not args.no_adjoint:
        steps = args.adjoint_steps
        line["adjoint"] = adjoint_measure(pkg, nsteps=steps, navg=min(100, max(1, steps // 2)))
    if not args.no_advection:
        line["advection"] = advection_measure(pkg, steps=args.advection_steps)
        line["mesh_setup"] = mesh_setup_measure(pkg)
    if args.large_vortex:
        line["large_vortex"] = large_vortex_measure(pkg)
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
