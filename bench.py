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
value_one_run  the same K steps as one dg_solver_run call (graphs of several steps,
        the next step's face launches overlapping the previous step's element
        launches), L2 flushed once before it; reported beside value.
e2e     the C-ABI call dg_solver_step_host with pinned host buffers: H2D of q,
        one step, D2H of q, timed with events on the same stream.
roofline  the dominant kernel's binding roof: its FP64-pipe instructions (per-unit
        counts from ncu, FP64_INST_*), algorithmic HBM bytes and mma flops over its
        event-timed duration (dg_solver_step_timed), against the FP64 pipe rate
        (half the DFMA peak, measured live), MEASURED_PEAKS.json's copy bandwidth
        and the mma.sync fp16 rate (measured live); plus the step's FP64-pipe
        fraction over the graph step time.
legs    the OP2 drop-in C++ application, the 64-instance batched sweep (and small
        instances), the adjoint case, the advection app, device mesh set-up and
        the large vortex case (each --no-<leg> skips it); clocks are sampled over
        all of them.
--impl reference  the CPU oracle (the reference's user kernels, restated, driven
        OP2-openmp style on all host cores) on the same workload.
Multi-GPU: replicas only (the path is one mesh per GPU); each rank runs the
workload, times are maxed over ranks, value = total DOF-stages / time.
"""
from __future__ import annotations

import argparse
import json
import math
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


def elem_bytes(n):
    """Algorithmic HBM bytes of the element kernel per cell-stage: W read and written
    (4 Np doubles each), q read in two stages of three and written in one (4 Np each), the face
    slots read (12 Nfp), the four metrics (and the fscale floats of the dt estimate)."""
    p, f = np_of(n), n + 1
    return 8 * (4 * p * (2 + 2 / 3 + 1 / 3) + 12 * f + 4 + 2 / 3)


def face_bytes(n):
    """Algorithmic HBM bytes of the face kernel per face node: the two traces read and the two
    scaled fluxes written (4 doubles each), the face normal and both fscale, the node indices
    and the edge record shared by the face's Nfp nodes."""
    return 8 * (4 * 4 + 4) + 2 * 4 + 16 / (n + 1)


def elem_mma(n):
    """mma.sync.m16n8k16 instructions of the element kernel per 32-cell tile: per parity block,
    8 row tiles (4 cells x 4 variables) x n-tiles of 8 operator rows x 28 digit products per
    k-step of 16 slots (orders 3-5); the dense rows at orders 1, 2."""
    sym = {3: (16, 16, 6, 4), 4: (23, 22, 9, 6), 5: (30, 30, 12, 9)}
    if n in sym:
        nue, nuo, nre, nro = sym[n]
        return 8 * 28 * (((nre + 7) // 8) * ((nue + 15) // 16) + ((nro + 7) // 8) * ((nuo + 15) // 16))
    if n in (1, 2):
        p, nk = np_of(n), 2 * np_of(n) + 3 * (n + 1)
        return 8 * 28 * ((p + 7) // 8) * ((nk + 15) // 16)
    return 0


# FP64-pipe thread instructions per unit (DFMA + DMUL + DADD and the rest of the FP64 pipe's
# instructions, smsp__thread_inst_executed_pipe_fp64_pred_on.sum per launch over the units the
# launch processes), counted by ncu on GB300 for the N = 3 kernels of this workload (profiles/
# fp64_instructions_naca_ogrid_K32768_N3.md).  They are properties of the compiled kernels, like
# the algorithmic bytes: re-count them when a kernel changes.
FP64_INST_PER_FACE_NODE = {3: 109.3}
FP64_INST_PER_CELL_STAGE = {3: 405.3}


def roofline(K, nf, face_ms, elem_ms, step_ms, peak_tf, hbm_peak, mma_tf=None):
    """Which roof binds, per kernel and for the overlapped step.

    The path is FP64 bound: the FP64 pipe issues one thread instruction per lane slot at the rate
    of half the DFMA flop peak (DFMA = 2 flops), measured live.  Each kernel's FP64 fraction is
    its FP64-pipe instructions (per unit, above) over its event-timed duration against that
    rate; its HBM fraction its algorithmic bytes over the same time against the measured copy
    bandwidth; the element kernel's tensor fraction its mma flops against the measured mma.sync
    fp16 rate.  frac is the largest (the binding roof) of the dominant kernel."""
    N = N_ORDER
    inst_rate = peak_tf * 1e12 / 2
    face_s, elem_s = face_ms * 1e-3, elem_ms * 1e-3
    fi, ei = FP64_INST_PER_FACE_NODE.get(N), FP64_INST_PER_CELL_STAGE.get(N)
    face_fp64 = fi * nf / face_s / inst_rate if fi else None
    elem_fp64 = ei * K / elem_s / inst_rate if ei else None
    face_hbm = face_bytes(N) * nf / face_s * 1e-9 / hbm_peak
    elem_hbm = elem_bytes(N) * K / elem_s * 1e-9 / hbm_peak
    tiles = (K + 31) // 32
    elem_tensor_tf = elem_mma(N) * tiles * 4096 / elem_s * 1e-12
    elem_tensor = elem_tensor_tf / mma_tf if mma_tf else None
    step_fp64 = ((3 * (fi * nf + ei * K)) / (step_ms * 1e-3) / inst_rate) if (fi and ei) else None
    # The dominant kernel: the element kernel unless the face kernel is clearly the longer (by more
    # than 2 %).  Separately launched they take about the same time per stage; inside the step graph
    # over cell ranges (what the timed step runs, and what the ncu launch list of it shows) the
    # element launches take the larger share, their range launches carrying longer tails.
    dominant = "elem_kernel" if elem_ms * 1.02 >= face_ms else "face_kernel"
    if dominant == "elem_kernel":
        roofs = {"fp64": elem_fp64, "hbm": elem_hbm, "tensor": elem_tensor}
        units, t = K, elem_s
    else:
        roofs = {"fp64": face_fp64, "hbm": face_hbm}
        units, t = nf, face_s
    bound = max((k for k in roofs if roofs[k] is not None), key=lambda k: roofs[k])
    if bound == "fp64":
        per = ei if dominant == "elem_kernel" else fi
        achieved, peak, unit = per * units / t * 1e-9, inst_rate * 1e-9, "G FP64-pipe thread-inst/s"
    elif bound == "hbm":
        per = elem_bytes(N) if dominant == "elem_kernel" else face_bytes(N)
        achieved, peak, unit = per * units / t * 1e-9, hbm_peak, "GB/s"
    else:
        achieved, peak, unit = elem_tensor_tf, mma_tf, "TFLOP/s"
    return {
        "bound": bound, "kernel": dominant, "achieved": achieved, "peak": peak, "unit": unit,
        "frac": achieved / peak, "traffic": None,
        "traffic_note": "DRAM bytes need hardware counters: measured by ncu, not in this run (profiles/)",
        "peak_source": {"fp64": "DFMA peak measured live on this GPU / 2 (instructions)",
                        "hbm": "MEASURED_PEAKS.json hbm_gbs", "tensor": "mma.sync fp16 measured live"}[bound],
        "hbm_frac": elem_hbm if dominant == "elem_kernel" else face_hbm,
        "fp64_pipe_frac": elem_fp64 if dominant == "elem_kernel" else face_fp64,
        "tensor_pipe_frac": elem_tensor if dominant == "elem_kernel" else 0.0,
        "face_fp64_pipe_frac": face_fp64, "face_hbm_frac": face_hbm,
        "elem_fp64_pipe_frac": elem_fp64, "elem_hbm_frac": elem_hbm, "elem_tensor_pipe_frac": elem_tensor,
        "elem_tensor_tflops": elem_tensor_tf, "f16_mma_peak_tflops": mma_tf,
        "step_fp64_pipe_frac": step_fp64,
        "step_note": "the graph step overlaps face and element launches of different cell ranges; "
                     "step_fp64_pipe_frac is both kernels' FP64-pipe instructions over the graph step time",
        "fp64_inst_per_face_node": fi, "fp64_inst_per_cell_stage": ei,
        "elem_bytes_per_cell_stage": elem_bytes(N), "face_bytes_per_face_node": face_bytes(N),
        "elem_flops_fp64_equivalent": elem_flops(N) * K / elem_s * 1e-12,
        "elem_flops_fp64_equivalent_note": "FP64-equivalent TFLOP/s of the element kernel: this build's count "
                                           "16Np^2 + 24NpNfp + 52Np = %d per cell-stage (the reference "
                                           "algorithm's, 32Np^2 + 24NpNfp + 60Np + 330Nfp = %d, covers "
                                           "the face kernel's Roe flux too); the contraction runs on the "
                                           "tensor cores, so this is not a fraction of any pipe"
                                           % (elem_flops(N), survey_flops(N)),
    }


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
    psteps = max(3, steps // 4)
    pms, sms = plain_device_times(pkg, solvers, psteps)
    del solvers
    tried = b.tried()
    best_persistent = min((t for t in tried if t[3] == "persistent"), key=lambda t: t[2], default=None)
    best_grouped = min((t for t in tried if t[3] == "grouped"), key=lambda t: t[2], default=None)
    return {"value": 3 * dof / (bms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": bms, "steps": steps,
            "instances": n_inst, "cells": cells, "dof_stage_per_step": 3 * dof, "shape": b.shape(),
            "autotune_ms_per_step": tuned,
            "persistent_ms_per_step": best_persistent[2] if best_persistent else None,
            "grouped_ms_per_step": best_grouped[2] if best_grouped else None,
            "shapes_timed": len(tried),
            "plain_concurrent_ms_per_step": pms, "plain_concurrent_value": 3 * dof / (pms * 1e-3),
            "plain_sequential_ms_per_step": sms, "plain_sequential_value": 3 * dof / (sms * 1e-3),
            "plain_how": "64 plain solvers (their step graphs); concurrent: each on its own stream, makespan "
                         "between CUDA events; sequential: sum of each solver's event-timed steps",
            "speedup_vs_plain": pms / bms, "speedup_vs_plain_sequential": sms / bms}


def plain_device_times(pkg, solvers, steps):
    """Device times per step of many plain solvers: all running at once on their own streams
    (makespan from the first start event to the last end event), and one after another (the
    sum of each solver's own event-timed steps, host gaps excluded)."""
    for s_ in solvers:
        s_.run(2)
    for s_ in solvers:
        s_.sync()
    starts = [pkg.Event() for _ in solvers]
    ends = [pkg.Event() for _ in solvers]
    for s_, a in zip(solvers, starts):
        a.record(s_.stream)
    for s_ in solvers:
        s_.run(steps)
    for s_, b in zip(solvers, ends):
        b.record(s_.stream)
    for s_ in solvers:
        s_.sync()
    t0 = starts[0]
    first = min(t0.elapsed_ms(a) for a in starts)
    last = max(t0.elapsed_ms(b) for b in ends)
    concurrent = (last - first) / steps
    seq = 0.0
    for s_ in solvers:
        a, b = pkg.Event(), pkg.Event()
        a.record(s_.stream)
        s_.run(steps)
        b.record(s_.stream)
        s_.sync()
        seq += a.elapsed_ms(b)
    return concurrent, seq / steps


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
    pms, sms = plain_device_times(pkg, solvers, steps)
    return {"value": 3 * dof / (bms * 1e-3), "unit": "DOF-stage/s", "ms_per_step": bms, "instances": n_inst,
            "cells": sum(m.size("cells") for m in meshes), "shape": b.shape(),
            "outside_config": "not the 64-instance sweep of the benchmark (O-grids 128x32..384x96): 64 small "
                              "O-grids 32x8..64x16, where the plain path is launch bound",
            "plain_concurrent_ms_per_step": pms, "plain_concurrent_value": 3 * dof / (pms * 1e-3),
            "plain_sequential_ms_per_step": sms, "plain_sequential_value": 3 * dof / (sms * 1e-3),
            "speedup_vs_plain": pms / bms, "speedup_vs_plain_sequential": sms / bms}


def adjoint_measure(pkg, nsteps=2000, navg=100, C=50):
    """The adjoint case: NACA 0012 O-grid 256x64 (K=32768), N=3, M=0.5, alpha=2 deg, the
    benchmark's boundary typing (slip wall, characteristic farfield), J = mean C_l over the last
    100 of 2000 steps, checkpoints every 50 steps.  Reports forward and backward device times, the
    adjoint/forward cost ratio, a central-difference check of dJ/dalpha (h = 1e-6) and the
    tangent-linear run's dJ/dalpha."""
    mesh = pkg.Mesh.naca_ogrid(N_THETA, N_R, farfield="characteristic")
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
            "boundaries": "slip wall + characteristic farfield (the benchmark's)",
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


def dropin_measure(pkg, steps=20):
    """The OP2 drop-in as its user runs it: the reference's airfoil main loop
    (src/airfoil.cpp:135-334: declarations from host arrays, the set-up loops, then per step
    get_neighbour_q, get_bedge_q, euler_rhs (x3), set_workingQ (x2), update_Q and calc_dt with
    its OP_MAX reduction back to the host) compiled in C++ against include/op2_gb300.h
    (apps/dropin_airfoil.cpp), on the benchmark's mesh and order (NACA 0012 O-grid 256 x 64,
    K = 32768, N = 3, M = 0.4) with the reference's own boundary typing (inflow / outflow by
    x < 0, wall) and dt = 1/dt1 (CFL 1, src/airfoil.cpp:237).  Wall-clock times from the
    application: from the first declaration to op_fetch_data(q), and the step loop alone."""
    import importlib
    import tempfile
    app = importlib.import_module(pkg.__name__ + ".dropin_app")
    mesh = pkg.Mesh.naca_ogrid(N_THETA, N_R, farfield="reference")
    m = mesh.arrays()
    ops = pkg.operators(N_ORDER)
    p = {"gam": 1.4, "bc_mach": MACH, "bc_alpha": ALPHA, "bc_p": 1.0, "bc_r": 1.0}
    p["bc_u"] = math.sqrt(1.4 * 1.0 / 1.0) * MACH
    p["bc_v"] = 0.0
    p["bc_e"] = 1.0 / (1.4 - 1.0) + 0.5 * 1.0 * p["bc_u"] ** 2
    with tempfile.TemporaryDirectory() as wd:
        exe = app.compile_app(wd, pkg.LIB_PATH)
        _, _, tm, _ = app.run_app(exe, m, ops, p, 2, wd)  # warm-up run (context, code load)
        q, dts, tm, _ = app.run_app(exe, m, ops, p, steps, wd)
    K = mesh.size("cells")
    dof = 3 * 4 * K * np_of(N_ORDER)
    return {"value": dof * steps / tm["steps_s"], "unit": "DOF-stage/s", "ms_per_step": tm["steps_s"] / steps * 1e3,
            "steps": steps, "end_to_end_s": tm["total_s"],
            "end_to_end_value": dof * steps / tm["total_s"],
            "loops_per_step": 13, "finite": bool(np.isfinite(q).all()),
            "how": "C++ application of the OP2 drop-in (host arrays in, op_fetch_data out); value over the step "
                   "loop, end_to_end from the first op_decl to op_fetch_data"}


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
    ap.add_argument("--no-dropin", action="store_true")
    ap.add_argument("--no-large-vortex", action="store_true",
                    help="skip the large vortex convergence + 16-instance batched beta gradient (~1 min)")
    ap.add_argument("--parts", type=int, default=0,
                    help="cell ranges of the step graph (0: the library's automatic choice; 1: one chain)")
    ap.add_argument("--adjoint-steps", type=int, default=2000)
    ap.add_argument("--advection-steps", type=int, default=200)
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
    pkg.set_step_parts(args.parts)
    # clocks sampled over every GPU leg of the run (the main timed region alone is a few ms,
    # shorter than the sampling interval)
    clocks = Clocks(local)
    t_gpu0 = time.perf_counter()

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
    for i in range(args.steps):
        pkg.l2_flush(stream)
        evs[i][0].record(stream)
        s.run(1)
        evs[i][1].record(stream)
    s.sync()
    step_ms = [a.elapsed_ms(b) for a, b in evs]
    total_ms = dist_max(dist, sum(step_ms))
    barrier(dist)
    ms_per_step = total_ms / args.steps
    value = world * dof_stage_per_step * args.steps / (total_ms * 1e-3)
    launches_per_step = s.kernels_per_step()

    # the same K steps as one run() call, as an application runs them: graphs of several steps,
    # the next step's face launches overlapping the previous step's element launches; L2 flushed
    # only before the call (the ~50 MB working set then stays in L2 from step to step)
    pkg.l2_flush(stream)
    ra, rb = pkg.Event(), pkg.Event()
    ra.record(stream)
    s.run(args.steps)
    rb.record(stream)
    s.sync()
    run_ms = dist_max(dist, ra.elapsed_ms(rb))
    run_value = world * dof_stage_per_step * args.steps / (run_ms * 1e-3)

    # per-kernel durations (same workload, the seven kernels of one step launched one after the
    # other with events between them: no overlap, so each kernel's own time)
    nk = min(args.steps, 50)
    kt = np.zeros(7)
    for _ in range(nk):
        pkg.l2_flush(stream)
        kt += s.step_timed()
    kt /= nk
    face_ms = float(np.mean(kt[[0, 2, 4]]))
    elem_ms = float(np.mean(kt[[1, 3, 5]]))
    nf = (mesh.size("edges") + mesh.size("bedges")) * (N_ORDER + 1)
    serial_ms = 3 * (face_ms + elem_ms) + float(kt[6])
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak = float(json.load(f)["hbm_gbs"])
        hbm_src = "measured (MEASURED_PEAKS.json)"
    except (OSError, KeyError, ValueError):
        hbm_peak, hbm_src = 6800.0, "fallback"
    peak_tf = peak_gflops * 1e-3
    roof = roofline(K, nf, face_ms, elem_ms, ms_per_step, peak_tf, hbm_peak, pkg.f16_mma_peak_gflops() * 1e-3)

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
                   "graph": "one CUDA graph launch per timed step: %d kernels over %d cell ranges"
                            % (launches_per_step, (launches_per_step - 1) // 6 if launches_per_step > 7 else 1)},
        "gpu_launches": launches_per_step * args.steps,
        "nodes_per_s": value / 4,
        "roofline": roof,
        "value_one_run": run_value, "ms_per_step_one_run": run_ms / args.steps,
        "one_run_note": "the K steps as one dg_solver_run call (graphs of %d steps), L2 flushed only before it"
                        % pkg.lib().dg_steps_per_graph(),
        "kernel_face_ms": face_ms, "kernel_elem_ms": elem_ms, "kernel_elem_stage2_ms": float(kt[5]),
        "kernel_finalize_ms": float(kt[6]), "serial_step_ms": serial_ms,
        "overlap_gain": serial_ms / ms_per_step,
        "fp64_dfma_peak_tflops": peak_tf, "fp64_mma_peak_tflops": dmma_gflops * 1e-3,
        "e2e": {"value": e2e_value, "unit": "DOF-stage/s", "h2d_bytes_per_step": nq * 8,
                "d2h_bytes_per_step": nq * 8, "steps": e2e_steps,
                "call": "dg_solver_step_host (pinned host q in/out, 1 step per call)"},
    }
    if not args.no_dropin:
        try:
            line["dropin"] = dropin_measure(pkg)
        except (RuntimeError, OSError) as exc:
            line["dropin"] = {"unavailable": str(exc)[:200]}
    if not args.no_batched:
        line["batched"] = batched_measure(pkg, args.batched_steps)
        line["batched"]["small_instances"] = batched_small_measure(pkg)
    if not args.no_adjoint:
        steps = args.adjoint_steps
        line["adjoint"] = adjoint_measure(pkg, nsteps=steps, navg=min(100, max(1, steps // 2)))
    if not args.no_advection:
        line["advection"] = advection_measure(pkg, steps=args.advection_steps)
        line["mesh_setup"] = mesh_setup_measure(pkg)
    if not args.no_large_vortex:
        line["large_vortex"] = large_vortex_measure(pkg)
    clk = clocks.stop()
    clk["window_s"] = time.perf_counter() - t_gpu0
    clk["window"] = "every GPU leg of this run"
    line["clocks"] = clk
    if rank == 0 and not args.no_cpu:
        nthreads = os.cpu_count() or 1
        rate, secs = cpu_oracle_rate(args.cpu_steps, nthreads)
        one_steps = max(1, args.cpu_steps // 16)
        rate1, secs1 = cpu_oracle_rate(one_steps, 1)
        line["cpu_baseline"] = {"value": rate, "unit": "DOF-stage/s", "cores": nthreads, "kind": "port",
                                "sample": "%d SSPRK3 steps of the full workload (%.1f s)" % (args.cpu_steps, secs),
                                "single_core_value": rate1,
                                "single_core_sample": "%d steps (%.1f s)" % (one_steps, secs1)}
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
