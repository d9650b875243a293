"""GB300-native DG Euler RHS + SSPRK3 step (Airfoil-OP2-FEM hot path).

Python front end over the C ABI of ``lib/libdg_gb300.so`` (include/dg_gb300.h
for the native fused solver, include/op2_gb300.h for the OP2 drop-in).  The
compute path is the CUDA library: nothing here computes on the CPU, and every
entry point raises if the library cannot be loaded.

The directory name is not a Python identifier; load it with
``importlib`` under the module name ``airfoil_op2_fem_gb300`` (see
``__graft_entry__.load_package``).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libdg_gb300.so")

APP_AIRFOIL, APP_VORTEX = 0, 1
DT_EVERY_STEP, DT_FROZEN = 0, 1
ERR_NONPHYSICAL = -200
ERR_TIMEOUT = -300
BATCH_GROUPED = 99  # dg_batch variant id of the grouped launches

_lib = None


class DGError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (code %d)" % (msg, code))
        self.code = code


class Config(C.Structure):
    """dg_config_t (include/dg_gb300.h)."""
    _fields_ = [("N", C.c_int), ("app", C.c_int), ("dt_mode", C.c_int), ("cfl", C.c_double),
                ("gam", C.c_double), ("mach", C.c_double), ("alpha_deg", C.c_double),
                ("p_inf", C.c_double), ("rho_inf", C.c_double), ("vortex_x0", C.c_double),
                ("vortex_y0", C.c_double), ("vortex_beta", C.c_double)]


def config(N=3, app=APP_AIRFOIL, dt_mode=DT_EVERY_STEP, cfl=1.0, gam=1.4, mach=0.4,
           alpha_deg=0.0, p_inf=1.0, rho_inf=1.0, vortex_x0=5.0, vortex_y0=0.0, vortex_beta=5.0):
    return Config(N, app, dt_mode, cfl, gam, mach, alpha_deg, p_inf, rho_inf, vortex_x0,
                  vortex_y0, vortex_beta)


def build():
    """Compile the CUDA library in-tree (sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_dg_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build()


def lib():
    """The loaded CUDA library; raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("CUDA library not built: %s (call build())" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    vp, ip, dp, cp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_char_p
    sig = {
        "dg_last_error": (cp, []),
        "dg_mesh_from_cells": (C.c_int, [C.c_int, dp, C.c_int, ip, C.POINTER(vp)]),
        "dg_mesh_from_tables": (C.c_int, [C.c_int, dp, C.c_int, ip, C.c_int, ip, ip, C.c_int, ip, ip, ip,
                                          C.POINTER(vp)]),
        "dg_mesh_read_vtk": (C.c_int, [cp, C.c_int, C.POINTER(vp)]),
        "dg_mesh_naca_ogrid": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, C.POINTER(vp)]),
        "dg_mesh_from_cells_device": (C.c_int, [C.c_int, dp, C.c_int, ip, C.POINTER(vp), C.POINTER(C.c_float)]),
        "dg_mesh_vortex_square": (C.c_int, [C.c_int, C.c_double, C.c_double, C.c_ulonglong, C.POINTER(vp)]),
        "dg_mesh_size": (C.c_int, [vp, C.c_int]),
        "dg_mesh_get": (C.c_int, [vp, cp, vp]),
        "dg_mesh_set_bedge_type": (C.c_int, [vp, ip]),
        "dg_mesh_free": (None, [vp]),
        "dg_operators": (C.c_int, [C.c_int, dp, dp, dp, dp, dp, dp, dp, ip]),
        "dg_solver_create": (C.c_int, [C.POINTER(Config), vp, C.POINTER(vp)]),
        "dg_solver_init": (C.c_int, [vp]),
        "dg_solver_run": (C.c_int, [vp, C.c_int]),
        "dg_solver_sync": (C.c_int, [vp]),
        "dg_solver_get": (C.c_int, [vp, cp, dp]),
        "dg_solver_set": (C.c_int, [vp, cp, dp]),
        "dg_solver_rhs": (C.c_int, [vp, dp, dp]),
        "dg_solver_time": (C.c_int, [vp, dp, dp, C.POINTER(C.c_ulonglong)]),
        "dg_solver_l2_error": (C.c_int, [vp, dp]),
        "dg_solver_record_dt": (C.c_int, [vp, C.c_int]),
        "dg_solver_dt_history": (C.c_int, [vp, dp, C.c_int]),
        "dg_solver_step_host": (C.c_int, [vp, dp, C.c_int, dp]),
        "dg_solver_device_ptr": (vp, [vp, cp]),
        "dg_solver_stream": (vp, [vp]),
        "dg_solver_step_timed": (C.c_int, [vp, C.POINTER(C.c_float)]),
        "dg_solver_free": (None, [vp]),
        "dg_solver_vertex_fields": (C.c_int, [vp, vp, dp, dp, dp, dp]),
        "dg_solver_write_vtk": (C.c_int, [vp, vp, cp]),
        "dg_mesh_write_vtk": (C.c_int, [vp, cp, dp, dp, dp, dp]),
        "dg_advec_create": (C.c_int, [vp, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(vp)]),
        "dg_advec_init": (C.c_int, [vp]),
        "dg_advec_run": (C.c_int, [vp, C.c_int]),
        "dg_advec_sync": (C.c_int, [vp]),
        "dg_advec_get": (C.c_int, [vp, cp, dp]),
        "dg_advec_set": (C.c_int, [vp, cp, dp]),
        "dg_advec_rhs": (C.c_int, [vp, dp, dp]),
        "dg_advec_time": (C.c_int, [vp, dp, C.POINTER(C.c_ulonglong)]),
        "dg_advec_step_timed": (C.c_int, [vp, C.POINTER(C.c_float)]),
        "dg_advec_vertex_values": (C.c_int, [vp, vp, dp]),
        "dg_advec_write_vtk": (C.c_int, [vp, vp, cp]),
        "dg_advec_stream": (vp, [vp]),
        "dg_advec_free": (None, [vp]),
        "dg_host_alloc": (vp, [C.c_size_t]),
        "dg_host_free": (None, [vp]),
        "dg_event_create": (vp, []),
        "dg_event_record": (C.c_int, [vp, vp]),
        "dg_event_elapsed_ms": (C.c_float, [vp, vp]),
        "dg_event_destroy": (None, [vp]),
        "dg_stream_sync": (C.c_int, [vp]),
        "dg_l2_flush": (C.c_int, [vp]),
        "dg_fp64_peak_gflops": (C.c_double, []),
        "dg_fp64_mma_peak_gflops": (C.c_double, []),
        "dg_kernels_per_step": (C.c_int, []),
        "dg_set_elem_variant": (None, [C.c_int]),
        "dg_set_elem_ws": (None, [C.c_int]),
        "dg_set_elem_blocks_per_sm": (None, [C.c_int]),
        "dg_elem_blocks_per_sm": (C.c_int, []),
        "dg_elem_ws": (C.c_int, []),
        "dg_elem_variant": (C.c_int, []),
        "dg_tc_operator_digits": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
        "dg_tc_round": (C.c_int, [C.c_longlong, C.c_longlong, C.c_int, C.c_void_p]),
        "dg_set_face_block": (None, [C.c_int]),
        "dg_set_face_regs64": (None, [C.c_int]),
        "dg_face_regs64": (C.c_int, []),
        "dg_set_pdl": (None, [C.c_int]),
        "dg_batch_create": (C.c_int, [C.c_int, C.POINTER(Config), C.POINTER(vp), C.POINTER(vp)]),
        "dg_batch_init": (C.c_int, [vp]),
        "dg_batch_autotune": (C.c_int, [vp, C.c_int, dp]),
        "dg_batch_run": (C.c_int, [vp, C.c_int]),
        "dg_batch_sync": (C.c_int, [vp]),
        "dg_batch_get": (C.c_int, [vp, C.c_int, cp, dp]),
        "dg_batch_time": (C.c_int, [vp, C.c_int, dp, dp, C.POINTER(C.c_ulonglong)]),
        "dg_batch_shape": (C.c_int, [vp, ip, ip, ip, ip]),
        "dg_batch_uses_graph": (C.c_int, [vp]),
        "dg_batch_use_shape": (C.c_int, [vp, C.c_int, C.c_int]),
        "dg_batch_inject_barrier_timeout": (C.c_int, [vp]),
        "dg_batch_tried": (C.c_int, [vp, C.c_int, ip, ip, dp]),
        "dg_batch_set_barrier_limit": (C.c_int, [vp, C.c_ulonglong]),
        "dg_batch_barrier_check": (C.c_int, [vp, C.c_ulonglong]),
        "dg_batch_stream": (vp, [vp]),
        "dg_batch_free": (None, [vp]),
        "dg_batch_last_error": (cp, []),
        "dg_sweep_config": (C.c_int, [C.c_int, C.c_ulonglong, ip, ip, ip, dp, dp]),
        "dg_adjoint_create": (C.c_int, [C.POINTER(Config), vp, C.c_int, C.c_int, C.c_int, C.POINTER(vp)]),
        "dg_adjoint_forward": (C.c_int, [vp, dp]),
        "dg_adjoint_backward": (C.c_int, [vp, C.c_double, dp, dp]),
        "dg_adjoint_evaluate": (C.c_int, [vp, C.c_double, dp, dp]),
        "dg_adjoint_dt_sequence": (C.c_int, [vp, dp, C.c_int]),
        "dg_adjoint_rhs_vjp": (C.c_int, [vp, dp, dp, dp, dp]),
        "dg_adjoint_stream": (vp, [vp]),
        "dg_adjoint_tangent": (C.c_int, [vp, C.c_double, dp, dp]),
        "dg_adjoint_batch_forward": (C.c_int, [C.POINTER(vp), C.c_int, dp]),
        "dg_adjoint_batch_backward": (C.c_int, [C.POINTER(vp), C.c_int, C.c_double, dp, C.POINTER(dp)]),
        "dg_adjoint_free": (None, [vp]),
        "dg_adjoint_last_error": (cp, []),
        "dg_order_tables_loaded": (C.c_int, [C.c_int, C.c_int]),
        "dg_solver_kernels_per_step": (C.c_int, [vp]),
        "dg_f16_mma_peak_gflops": (C.c_double, []),
        "dg_set_step_parts": (None, [C.c_int]),
        "dg_step_parts": (C.c_int, []),
        "dg_set_steps_per_graph": (None, [C.c_int]),
        "dg_steps_per_graph": (C.c_int, []),
        "dg_set_step_graph_flags": (None, [C.c_int]),
        "dg_step_graph_flags": (C.c_int, []),
        "dg_boundary_state": (C.c_int, [C.POINTER(Config), C.c_int, C.c_int, dp, dp, dp]),
        "dg_boundary_state_error": (cp, []),
        "dg_rhs_noalloc_ready": (C.c_int, [C.c_int]),
        "dg_once_table_selftest": (C.c_int, [C.c_int, C.c_int, ip, ip]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _check(rc):
    if rc != 0:
        raise DGError(rc, lib().dg_last_error().decode())


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class Mesh:
    """A triangle mesh with the reference's connectivity tables (dg_mesh_t)."""

    def __init__(self, handle):
        self.h = handle

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dg_mesh_free(self.h)
            self.h = None

    @classmethod
    def from_cells(cls, coords, cells, device=False):
        """Edge tables from cells + coordinates, on the host or (device=True) on the GPU; the
        two give identical tables.  After a device build, `build_ms` holds its device time."""
        coords, cells = _f64(coords), _i32(cells)
        h = C.c_void_p()
        if device:
            ms = C.c_float()
            _check(lib().dg_mesh_from_cells_device(coords.shape[0], _dp(coords), cells.shape[0], _ip(cells),
                                                   C.byref(h), C.byref(ms)))
            out = cls(h)
            out.build_ms = ms.value
            return out
        _check(lib().dg_mesh_from_cells(coords.shape[0], _dp(coords), cells.shape[0], _ip(cells), C.byref(h)))
        return cls(h)

    @classmethod
    def from_tables(cls, m):
        a = {k: (_f64(v) if k == "coords" else _i32(v)) for k, v in m.items()}
        bt = a.get("bedge_type")
        h = C.c_void_p()
        _check(lib().dg_mesh_from_tables(
            a["coords"].shape[0], _dp(a["coords"]), a["cell2nodes"].shape[0], _ip(a["cell2nodes"]),
            a["edge2cells"].shape[0], _ip(a["edge2cells"]), _ip(a["edgeNum"]), a["bedge2cell"].shape[0],
            _ip(a["bedge2cell"]), _ip(a["bedgeNum"]), _ip(bt) if bt is not None else None, C.byref(h)))
        return cls(h)

    @classmethod
    def read_vtk(cls, path, classify_box=True):
        h = C.c_void_p()
        _check(lib().dg_mesh_read_vtk(path.encode(), int(classify_box), C.byref(h)))
        return cls(h)

    @classmethod
    def naca_ogrid(cls, n_theta=256, n_r=64, stretch=1.1, radius=20.0, farfield="characteristic"):
        h = C.c_void_p()
        _check(lib().dg_mesh_naca_ogrid(n_theta, n_r, stretch, radius,
                                        1 if farfield == "characteristic" else 0, C.byref(h)))
        return cls(h)

    @classmethod
    def vortex_square(cls, n=32, lo=-5.0, hi=5.0, seed=20261203):
        h = C.c_void_p()
        _check(lib().dg_mesh_vortex_square(n, lo, hi, seed, C.byref(h)))
        return cls(h)

    def size(self, what):
        idx = {"nodes": 0, "cells": 1, "edges": 2, "bedges": 3}[what]
        n = lib().dg_mesh_size(self.h, idx)
        if n < 0:
            _check(n)
        return n

    def arrays(self):
        nn, nc, ne, nb = (self.size(w) for w in ("nodes", "cells", "edges", "bedges"))
        shapes = {"coords": (np.float64, (nn, 2)), "cell2nodes": (np.int32, (nc, 3)),
                  "edge2nodes": (np.int32, (ne, 2)), "edge2cells": (np.int32, (ne, 2)),
                  "edgeNum": (np.int32, (ne, 2)), "bedge2nodes": (np.int32, (nb, 2)),
                  "bedge2cell": (np.int32, (nb,)), "bedgeNum": (np.int32, (nb,)),
                  "bedge_type": (np.int32, (nb,))}
        out = {}
        for name, (dt, shp) in shapes.items():
            a = np.empty(shp, dtype=dt)
            _check(lib().dg_mesh_get(self.h, name.encode(), a.ctypes.data_as(C.c_void_p)))
            out[name] = a
        return out

    def set_bedge_type(self, types):
        t = _i32(types)
        _check(lib().dg_mesh_set_bedge_type(self.h, _ip(t)))

    def write_vtk(self, path, rho, u, v, p):
        """Legacy-VTK file of per-vertex fields (host arrays of n_nodes)."""
        a = [np.ascontiguousarray(x, dtype=np.float64) for x in (rho, u, v, p)]
        n = self.size("nodes")
        if any(x.size != n for x in a):
            raise ValueError("fields must have one value per mesh vertex")
        _check(lib().dg_mesh_write_vtk(self.h, str(path).encode(), *[_dp(x) for x in a]))


def operators(N):
    """Nodal operators of order N (dict like the reference's constants headers)."""
    np_, nfp = (N + 1) * (N + 2) // 2, N + 1
    o = {k: np.empty(sz) for k, sz in (("r", np_), ("s", np_), ("Dr", np_ * np_), ("Ds", np_ * np_),
                                         ("Drw", np_ * np_), ("Dsw", np_ * np_), ("LIFT", np_ * 3 * nfp))}
    fm = np.empty(3 * nfp, dtype=np.int32)
    _check(lib().dg_operators(N, *(_dp(o[k]) for k in ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT")), _ip(fm)))
    o["FMASK"] = fm
    o.update(N=N, Np=np_, Nfp=nfp)
    for k in ("Dr", "Ds", "Drw", "Dsw"):
        o[k] = o[k].reshape(np_, np_)
    o["LIFT"] = o["LIFT"].reshape(np_, 3 * nfp)
    return o


class Solver:
    """The native fused solver (dg_solver_t): state stays on the GPU between calls."""

    def __init__(self, mesh: Mesh, cfg: Config):
        self.mesh = mesh
        self.cfg = cfg
        self.N = cfg.N
        self.Np = (cfg.N + 1) * (cfg.N + 2) // 2
        self.K = mesh.size("cells")
        h = C.c_void_p()
        _check(lib().dg_solver_create(C.byref(cfg), mesh.h, C.byref(h)))
        self.h = h

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dg_solver_free(self.h)
            self.h = None

    def init(self):
        _check(lib().dg_solver_init(self.h))
        return self

    def run(self, nsteps):
        _check(lib().dg_solver_run(self.h, nsteps))

    def sync(self):
        _check(lib().dg_solver_sync(self.h))

    def get(self, name="q"):
        n = self.K * 16 if name == "geo" else (self.K * 3 * (self.N + 1) * 4 if name == "flux" else self.K * self.Np * 4)
        out = np.empty(n)
        _check(lib().dg_solver_get(self.h, name.encode(), _dp(out)))
        return out

    def set(self, name, arr):
        a = _f64(arr).ravel()
        assert a.size == self.K * self.Np * 4
        _check(lib().dg_solver_set(self.h, name.encode(), _dp(a)))

    def rhs(self, W):
        a = _f64(W).ravel()
        out = np.empty_like(a)
        _check(lib().dg_solver_rhs(self.h, _dp(a), _dp(out)))
        return out

    def time(self):
        t, dt, st = C.c_double(), C.c_double(), C.c_ulonglong()
        _check(lib().dg_solver_time(self.h, C.byref(t), C.byref(dt), C.byref(st)))
        return t.value, dt.value, st.value

    def l2_error(self):
        out = np.empty(4)
        _check(lib().dg_solver_l2_error(self.h, _dp(out)))
        return out

    def record_dt(self, max_steps):
        _check(lib().dg_solver_record_dt(self.h, max_steps))

    def dt_history(self, n):
        out = np.empty(n)
        _check(lib().dg_solver_dt_history(self.h, _dp(out), n))
        return out

    def step_host(self, q_in, nsteps, q_out):
        _check(lib().dg_solver_step_host(self.h, _dp(q_in) if q_in is not None else None, nsteps,
                                         _dp(q_out) if q_out is not None else None))

    def step_timed(self):
        ms = (C.c_float * 7)()
        _check(lib().dg_solver_step_timed(self.h, ms))
        return np.array(ms[:], dtype=np.float64)

    @property
    def stream(self):
        return lib().dg_solver_stream(self.h)

    def kernels_per_step(self):
        """Kernel launches of one run() step (the step graph's nodes)."""
        return lib().dg_solver_kernels_per_step(self.h)

    def vertex_fields(self):
        """rho, u, v, p per mesh vertex (src/save_solution.cpp's sampling)."""
        n = self.mesh.size("nodes")
        out = [np.empty(n) for _ in range(4)]
        _check(lib().dg_solver_vertex_fields(self.h, self.mesh.h, *[_dp(a) for a in out]))
        return out

    def write_vtk(self, path):
        """The current solution as a legacy-VTK file (vertex_fields' values)."""
        _check(lib().dg_solver_write_vtk(self.h, self.mesh.h, str(path).encode()))


class Batch:
    """Many instances advanced together by one persistent kernel per RK stage (dg_batch_t)."""

    def __init__(self, meshes, cfgs):
        assert len(meshes) == len(cfgs) and meshes
        self.meshes, self.cfgs = list(meshes), list(cfgs)
        arr = (Config * len(cfgs))(*cfgs)
        hs = (C.c_void_p * len(meshes))(*[m.h for m in meshes])
        h = C.c_void_p()
        self._check(lib().dg_batch_create(len(cfgs), arr, hs, C.byref(h)))
        self.h = h

    @staticmethod
    def _check(rc):
        if rc != 0:
            raise DGError(rc, lib().dg_batch_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dg_batch_free(self.h)
            self.h = None

    def init(self):
        self._check(lib().dg_batch_init(self.h))
        return self

    def autotune(self, steps=2):
        ms = C.c_double()
        self._check(lib().dg_batch_autotune(self.h, steps, C.byref(ms)))
        return ms.value

    def run(self, nsteps):
        self._check(lib().dg_batch_run(self.h, nsteps))

    def sync(self):
        self._check(lib().dg_batch_sync(self.h))

    def get(self, k, name="q"):
        N = self.cfgs[k].N
        n = self.meshes[k].size("cells") * (N + 1) * (N + 2) // 2 * 4
        out = np.empty(n)
        self._check(lib().dg_batch_get(self.h, k, name.encode(), _dp(out)))
        return out

    def time(self, k):
        t, dt, st = C.c_double(), C.c_double(), C.c_ulonglong()
        self._check(lib().dg_batch_time(self.h, k, C.byref(t), C.byref(dt), C.byref(st)))
        return t.value, dt.value, st.value

    def shape(self):
        v = [C.c_int() for _ in range(4)]
        self._check(lib().dg_batch_shape(self.h, *[C.byref(x) for x in v]))
        return dict(variant=v[0].value, block=v[1].value, face_tile=v[2].value, grid=v[3].value,
                    kind="grouped" if v[0].value == BATCH_GROUPED else "persistent",
                    graph=bool(lib().dg_batch_uses_graph(self.h)))

    def use_shape(self, variant, face_tile):
        """Select a launch shape without timing (variant BATCH_GROUPED for grouped launches)."""
        self._check(lib().dg_batch_use_shape(self.h, variant, face_tile))

    def tried(self):
        """Every shape the last autotune timed: [(variant, face_tile, ms_per_step, kind)]."""
        n = lib().dg_batch_tried(self.h, -1, None, None, None)
        out = []
        for i in range(max(0, n)):
            v, f, ms = C.c_int(), C.c_int(), C.c_double()
            lib().dg_batch_tried(self.h, i, C.byref(v), C.byref(f), C.byref(ms))
            out.append((v.value, f.value, ms.value, "grouped" if v.value == BATCH_GROUPED else "persistent"))
        return out

    @property
    def stream(self):
        return lib().dg_batch_stream(self.h)


class LiftObjective:
    """An objective with its discrete adjoint (dg_adjoint_t), used like torch.autograd.Function:
    J = forward(); grad_param, grad_q0 = backward(grad_J).  Airfoil (cfg.app 0): mean lift
    coefficient over the last navg steps, parameter alpha (degrees).  Vortex (cfg.app 1):
    final-time squared error against the analytic vortex, parameter beta."""

    def __init__(self, mesh, cfg, nsteps, navg, checkpoint_every=50):
        self.mesh, self.cfg, self.nsteps = mesh, cfg, nsteps
        self.param = cfg.vortex_beta if cfg.app == APP_VORTEX else cfg.alpha_deg
        self.K = mesh.size("cells")
        self.nq = self.K * (cfg.N + 1) * (cfg.N + 2) // 2 * 4
        h = C.c_void_p()
        self._check(lib().dg_adjoint_create(C.byref(cfg), mesh.h, nsteps, navg, checkpoint_every, C.byref(h)))
        self.h = h

    @staticmethod
    def _check(rc):
        if rc != 0:
            raise DGError(rc, lib().dg_adjoint_last_error().decode())

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dg_adjoint_free(self.h)
            self.h = None

    def forward(self):
        J = C.c_double()
        self._check(lib().dg_adjoint_forward(self.h, C.byref(J)))
        return J.value

    def backward(self, grad_J=1.0, want_q0=True):
        ga = C.c_double()
        gq = np.empty(self.nq) if want_q0 else None
        self._check(lib().dg_adjoint_backward(self.h, grad_J, C.byref(ga), _dp(gq) if want_q0 else None))
        return ga.value, gq

    def evaluate(self, alpha_deg, q0=None):
        J = C.c_double()
        q = None if q0 is None else _f64(q0).ravel()
        self._check(lib().dg_adjoint_evaluate(self.h, alpha_deg, _dp(q) if q is not None else None, C.byref(J)))
        return J.value

    def tangent(self, d_param, dq0=None):
        """Tangent-linear run: dJ along (d_param, dq0), independent of the reverse kernels."""
        dJ = C.c_double()
        q = None if dq0 is None else _f64(dq0).ravel()
        self._check(lib().dg_adjoint_tangent(self.h, d_param, _dp(q) if q is not None else None, C.byref(dJ)))
        return dJ.value

    def dt_sequence(self):
        out = np.empty(self.nsteps)
        self._check(lib().dg_adjoint_dt_sequence(self.h, _dp(out), self.nsteps))
        return out

    def rhs_vjp(self, W, v):
        W, v = _f64(W).ravel(), _f64(v).ravel()
        out, ap = np.empty(self.nq), C.c_double()
        self._check(lib().dg_adjoint_rhs_vjp(self.h, _dp(W), _dp(v), _dp(out), C.byref(ap)))
        return out, ap.value

    @property
    def stream(self):
        return lib().dg_adjoint_stream(self.h)


def torch_objective(obj):
    """A torch.autograd.Function over a LiftObjective: f(p) -> J, with p the objective's scalar
    parameter (alpha in degrees for the airfoil, beta for the vortex) as a 0-d float64 tensor.
    forward() runs the recording forward solve at p; backward() the discrete adjoint, so
    torch.autograd composes it with other torch code.  The solve itself stays in the library;
    torch only carries the scalars."""
    import torch

    class _Objective(torch.autograd.Function):
        @staticmethod
        def forward(ctx, p):
            if float(p) != obj.param:
                raise ValueError("the objective was created at parameter %g" % obj.param)
            J = obj.forward()
            return torch.tensor(J, dtype=torch.float64, device=p.device)

        @staticmethod
        def backward(ctx, grad_J):
            g, _ = obj.backward(float(grad_J), want_q0=False)
            return torch.tensor(g, dtype=torch.float64, device=grad_J.device)

    return _Objective.apply


def adjoint_batch_forward(objs):
    """forward() of every objective at once (concurrent, one stream and host thread each)."""
    hs = (C.c_void_p * len(objs))(*[o.h.value for o in objs])
    J = np.empty(len(objs))
    LiftObjective._check(lib().dg_adjoint_batch_forward(hs, len(objs), _dp(J)))
    return J


def adjoint_batch_backward(objs, grad_J=1.0, want_q0=False):
    """backward(grad_J) of every objective at once: (grad_param[n], [grad_q0] or None)."""
    hs = (C.c_void_p * len(objs))(*[o.h.value for o in objs])
    g = np.empty(len(objs))
    gq = [np.empty(o.nq) for o in objs] if want_q0 else None
    ptrs = (C.POINTER(C.c_double) * len(objs))(*[_dp(a) for a in gq]) if want_q0 else None
    LiftObjective._check(lib().dg_adjoint_batch_backward(hs, len(objs), grad_J, _dp(g), ptrs))
    return g, gq


def sweep_config(n=64, seed=20261203):
    """The batched sweep's per-instance (n_theta, n_r, order, alpha_deg, mach)."""
    nt, nr, od = (np.empty(n, dtype=np.int32) for _ in range(3))
    al, ma = np.empty(n), np.empty(n)
    _check(lib().dg_sweep_config(n, seed, _ip(nt), _ip(nr), _ip(od), _dp(al), _dp(ma)))
    return [dict(n_theta=int(nt[i]), n_r=int(nr[i]), N=int(od[i]), alpha_deg=float(al[i]), mach=float(ma[i]))
            for i in range(n)]


class Advection:
    """The scalar advection app (advec/src/advec.cpp) on the GPU: q has one value per node,
    classical RK4 with a fixed dt, velocity (vel_x, vel_y) (the app's -vx/-vy)."""

    def __init__(self, mesh, N=4, vel_x=1.0, vel_y=1.0, dt=1e-3):
        self.mesh, self.N, self.dt = mesh, N, dt
        self.h = C.c_void_p()
        _check(lib().dg_advec_create(mesh.h, N, vel_x, vel_y, dt, C.byref(self.h)))
        self.n = mesh.size("cells") * (N + 1) * (N + 2) // 2

    def __del__(self):
        if getattr(self, "h", None):
            lib().dg_advec_free(self.h)
            self.h = None

    def init(self):
        _check(lib().dg_advec_init(self.h))
        return self

    def run(self, nsteps):
        _check(lib().dg_advec_run(self.h, nsteps))

    def sync(self):
        _check(lib().dg_advec_sync(self.h))

    def get(self, name="q"):
        n = self.mesh.size("cells") * 16 if name == "geo" else self.n
        out = np.empty(n)
        _check(lib().dg_advec_get(self.h, name.encode(), _dp(out)))
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        if a.size != self.n:
            raise ValueError("expected %d values" % self.n)
        _check(lib().dg_advec_set(self.h, name.encode(), _dp(a)))

    def rhs(self, W):
        a = np.ascontiguousarray(W, dtype=np.float64).ravel()
        if a.size != self.n:
            raise ValueError("expected %d values" % self.n)
        out = np.empty(self.n)
        _check(lib().dg_advec_rhs(self.h, _dp(a), _dp(out)))
        return out

    def time(self):
        t, k = C.c_double(), C.c_ulonglong()
        _check(lib().dg_advec_time(self.h, C.byref(t), C.byref(k)))
        return t.value, k.value

    def step_timed(self):
        ms = (C.c_float * 8)()
        _check(lib().dg_advec_step_timed(self.h, ms))
        return list(ms)

    def vertex_values(self):
        out = np.empty(self.mesh.size("nodes"))
        _check(lib().dg_advec_vertex_values(self.h, self.mesh.h, _dp(out)))
        return out

    def write_vtk(self, path):
        _check(lib().dg_advec_write_vtk(self.h, self.mesh.h, str(path).encode()))

    @property
    def stream(self):
        return lib().dg_advec_stream(self.h)


class PinnedArray:
    """A float64 numpy view of pinned host memory (dg_host_alloc)."""

    def __init__(self, n):
        self.ptr = lib().dg_host_alloc(n * 8)
        if not self.ptr:
            raise MemoryError("pinned allocation failed")
        self.array = np.ctypeslib.as_array(C.cast(self.ptr, C.POINTER(C.c_double)), shape=(n,))

    def __del__(self):
        if getattr(self, "ptr", None) and _lib is not None:
            _lib.dg_host_free(self.ptr)
            self.ptr = None


class Event:
    def __init__(self):
        self.h = lib().dg_event_create()

    def record(self, stream):
        _check(lib().dg_event_record(self.h, stream))

    def elapsed_ms(self, end):
        return lib().dg_event_elapsed_ms(self.h, end.h)

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.dg_event_destroy(self.h)


def l2_flush(stream):
    _check(lib().dg_l2_flush(stream))


def fp64_peak_gflops():
    return lib().dg_fp64_peak_gflops()


def f16_mma_peak_gflops():
    return lib().dg_f16_mma_peak_gflops()


def fp64_mma_peak_gflops():
    """FP64 tensor-core (DMMA, mma.sync m8n8k4) throughput measured on this GPU, GFLOP/s."""
    return lib().dg_fp64_mma_peak_gflops()


def boundary_state(cfg, bc_type, qi, nrm):
    """The device's ghost state (dg_boundary_state) of boundary type bc_type for interior states
    qi [n][4] and unit normals nrm [n][2]; returns [n][4]."""
    qi = _f64(np.asarray(qi).reshape(-1, 4))
    nrm = _f64(np.asarray(nrm).reshape(-1, 2))
    out = np.empty_like(qi)
    rc = lib().dg_boundary_state(C.byref(cfg), int(bc_type), qi.shape[0], _dp(qi), _dp(nrm), _dp(out))
    if rc != 0:
        raise DGError(rc, lib().dg_boundary_state_error().decode())
    return out


def set_step_parts(parts):
    """Cell ranges of step graphs built from now on (0 automatic, 1 one chain, 2..32)."""
    lib().dg_set_step_parts(int(parts))


def step_parts():
    return lib().dg_step_parts()
