"""ctypes front end of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Loads ``oracle/liboracle.so`` (the restated kernels, kind "port") or
``oracle/_ref/libref.so`` (the reference's own kernel headers, kind
"reference"), both exporting the C API of ``oracle/dg_oracle.h``.  Only tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref.so")
# Where the reference source tree is read from (the reference build and the golden fixtures):
# the environment variable DG_REFERENCE_TREE, else the checkout location of this build machine.
REFERENCE_TREE = os.environ.get("DG_REFERENCE_TREE", "/root/reference")

APP_AIRFOIL, APP_VORTEX = 0, 1
DT_EVERY_STEP, DT_FROZEN = 0, 1


class _Ops(C.Structure):
    _fields_ = [("N", C.c_int)] + [(n, C.POINTER(C.c_double)) for n in
                                   ("r", "s", "Dr", "Ds", "Drw", "Dsw", "LIFT")] + \
               [("FMASK", C.POINTER(C.c_int))]


class _Phys(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("gam", "bc_mach", "bc_alpha", "bc_p", "bc_r", "bc_u",
                                          "bc_v", "bc_e", "vortex_x0", "vortex_y0", "vortex_beta")]


class _Mesh(C.Structure):
    _fields_ = [("n_nodes", C.c_int), ("n_cells", C.c_int), ("n_edges", C.c_int),
                ("n_bedges", C.c_int), ("coords", C.POINTER(C.c_double))] + \
               [(n, C.POINTER(C.c_int)) for n in ("cell2nodes", "edge2cells", "edgeNum",
                                                 "bedge2cell", "bedgeNum", "bedge_type")]


def build(ref: bool = None):
    """Compile the oracle libraries with make; the reference build only if its tree exists."""
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref is None:
        ref = os.path.isdir(REFERENCE_TREE)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "REF=" + REFERENCE_TREE], check=True)


_LIBS = {}


def load(kind: str = "port"):
    path = PORT_LIB if kind == "port" else REF_LIB
    if path not in _LIBS:
        if not os.path.exists(path):
            raise FileNotFoundError(path + " (run oracle.build())")
        lib = C.CDLL(path)
        lib.orc_create.restype = C.c_void_p
        lib.orc_create.argtypes = [C.POINTER(_Ops), C.POINTER(_Phys), C.POINTER(_Mesh), C.c_int]
        lib.orc_destroy.argtypes = [C.c_void_p]
        lib.orc_last_error.restype = C.c_char_p
        lib.orc_kind.restype = C.c_char_p
        lib.orc_init.argtypes = [C.c_void_p, C.c_double]
        lib.orc_get.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
        lib.orc_set.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
        lib.orc_rhs.argtypes = [C.c_void_p, C.c_int, C.c_double]
        lib.orc_run.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.POINTER(C.c_double)]
        lib.orc_dt.restype = C.c_double
        lib.orc_dt.argtypes = [C.c_void_p]
        lib.orc_time.restype = C.c_double
        lib.orc_time.argtypes = [C.c_void_p]
        lib.orc_l2_error.argtypes = [C.c_void_p, C.POINTER(C.c_double)]
        lib.orc_refresh_dt.argtypes = [C.c_void_p]
        lib.adv_create.restype = C.c_void_p
        lib.adv_create.argtypes = [C.POINTER(_Ops), C.POINTER(_Mesh), C.c_double, C.c_double]
        lib.adv_destroy.argtypes = [C.c_void_p]
        lib.adv_init.argtypes = [C.c_void_p, C.c_double]
        lib.adv_get.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
        lib.adv_set.argtypes = [C.c_void_p, C.c_char_p, C.POINTER(C.c_double)]
        lib.adv_rhs.argtypes = [C.c_void_p, C.c_int]
        lib.adv_run.argtypes = [C.c_void_p, C.c_int, C.c_int]
        lib.adv_time.restype = C.c_double
        lib.adv_time.argtypes = [C.c_void_p]
        _LIBS[path] = lib
    return _LIBS[path]


def freestream(mach=0.4, alpha_deg=0.0, gam=1.4, p=1.0, rho=1.0):
    """Boundary/freestream constants as src/airfoil.cpp:79-99 computes them."""
    if alpha_deg != 0.0:
        u = math.sin((math.pi / 2.0) - (alpha_deg * math.pi / 180.0)) * math.sqrt(gam * p / rho) * mach
        v = math.cos((math.pi / 2.0) - (alpha_deg * math.pi / 180.0)) * math.sqrt(gam * p / rho) * mach
        e = p / (gam - 1.0) + 0.5 * rho * (u * u + v * v)
    else:
        u = math.sqrt(gam * p / rho) * mach
        v = 0.0
        e = p / (gam - 1.0) + 0.5 * rho * (u * u)
    return dict(gam=gam, bc_mach=mach, bc_alpha=alpha_deg, bc_p=p, bc_r=rho, bc_u=u, bc_v=v,
                bc_e=e, vortex_x0=5.0, vortex_y0=0.0, vortex_beta=5.0)


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _structs(mesh, ops):
    """(_Ops, _Mesh, arrays to keep alive) from an operator dict and a mesh dict."""
    keep = {}
    N = int(ops["N"])

    def f64(name):
        a = np.ascontiguousarray(ops[name], dtype=np.float64).ravel()
        keep[name] = a
        return _dp(a)

    fm = np.ascontiguousarray(ops["FMASK"], dtype=np.int32).ravel()
    keep["FMASK"] = fm
    o = _Ops(N, f64("r"), f64("s"), f64("Dr"), f64("Ds"), f64("Drw"), f64("Dsw"), f64("LIFT"), _ip(fm))
    m = {k: np.ascontiguousarray(v) for k, v in mesh.items()}
    if "bedge_type" not in m:
        m["bedge_type"] = np.full(m["bedge2cell"].shape[0], 2, dtype=np.int32)
    keep.update(m)
    ms = _Mesh(int(m["coords"].shape[0]), int(m["cell2nodes"].shape[0]), int(m["edge2cells"].shape[0]),
               int(m["bedge2cell"].shape[0]), _dp(m["coords"]), _ip(m["cell2nodes"]),
               _ip(m["edge2cells"]), _ip(m["edgeNum"]), _ip(m["bedge2cell"]),
               _ip(m["bedgeNum"]), _ip(m["bedge_type"]))
    return o, ms, keep


class Oracle:
    """One oracle instance over a mesh dict (oracle.mesh layout) and an operator dict
    (oracle.operators layout)."""

    def __init__(self, mesh, ops, phys, app=APP_AIRFOIL, kind="port"):
        self.lib = load(kind)
        self.N = int(ops["N"])
        self.Np = (self.N + 1) * (self.N + 2) // 2
        self.Nfp = self.N + 1
        self._ops, self._mesh, self._keep = _structs(mesh, ops)
        self._phys = _Phys(**{k: float(phys[k]) for k, _ in _Phys._fields_})
        self.K = int(self._mesh.n_cells)
        self.h = self.lib.orc_create(C.byref(self._ops), C.byref(self._phys), C.byref(self._mesh), app)
        if not self.h:
            raise RuntimeError(self.lib.orc_last_error().decode())

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.orc_destroy(h)
            self.h = None

    _DIMS = None

    def dim(self, name):
        np_, nfp = self.Np, self.Nfp
        return {"nodeX": 3, "nodeY": 3, "nx": 3 * nfp, "ny": 3 * nfp, "fscale": 3 * nfp,
                "exteriorQ": 12 * nfp, "q": 4 * np_, "workingQ": 4 * np_, "rk1": 4 * np_,
                "rk2": 4 * np_, "rk3": 4 * np_}.get(name, np_)

    def init(self, cfl=1.0):
        self._check(self.lib.orc_init(self.h, cfl))

    def get(self, name):
        out = np.empty(self.K * self.dim(name))
        self._check(self.lib.orc_get(self.h, name.encode(), _dp(out)))
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        assert a.size == self.K * self.dim(name)
        self._check(self.lib.orc_set(self.h, name.encode(), _dp(a)))

    def rhs(self, stage=0, t_stage=0.0):
        self._check(self.lib.orc_rhs(self.h, stage, t_stage))
        return self.get("rk%d" % (stage + 1))

    def run(self, iters, dt_mode=DT_EVERY_STEP, nthreads=0):
        hist = np.empty(max(iters, 1))
        self._check(self.lib.orc_run(self.h, iters, dt_mode, nthreads, _dp(hist)))
        return hist[:iters]

    @property
    def dt(self):
        return self.lib.orc_dt(self.h)

    @property
    def t(self):
        return self.lib.orc_time(self.h)

    def refresh_dt(self):
        self._check(self.lib.orc_refresh_dt(self.h))

    def l2_error(self):
        out = np.empty(4)
        self._check(self.lib.orc_l2_error(self.h, _dp(out)))
        return out

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.orc_last_error().decode())


class Advection:
    """The scalar advection app (advec/src/advec.cpp) on the oracle: q has one value per node."""

    def __init__(self, mesh, ops, vel_x=1.0, vel_y=1.0, kind="port"):
        self.lib = load(kind)
        self.N = int(ops["N"])
        self.Np = (self.N + 1) * (self.N + 2) // 2
        self.Nfp = self.N + 1
        self._ops, self._mesh, self._keep = _structs(mesh, ops)
        self.K = int(self._mesh.n_cells)
        self.h = self.lib.adv_create(C.byref(self._ops), C.byref(self._mesh), vel_x, vel_y)
        if not self.h:
            raise RuntimeError(self.lib.orc_last_error().decode())

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.adv_destroy(h)
            self.h = None

    def dim(self, name):
        return {"nodeX": 3, "nodeY": 3, "nx": 3 * self.Nfp, "ny": 3 * self.Nfp, "fscale": 3 * self.Nfp,
                "exteriorQ": 3 * self.Nfp}.get(name, self.Np)

    def init(self, dt=1e-3):
        self._check(self.lib.adv_init(self.h, dt))

    def get(self, name):
        out = np.empty(self.K * self.dim(name))
        self._check(self.lib.adv_get(self.h, name.encode(), _dp(out)))
        return out

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).ravel()
        assert a.size == self.K * self.dim(name)
        self._check(self.lib.adv_set(self.h, name.encode(), _dp(a)))

    def rhs(self, stage=0):
        self._check(self.lib.adv_rhs(self.h, stage))
        return self.get("rk%d" % (stage + 1))

    def run(self, iters, nthreads=0):
        self._check(self.lib.adv_run(self.h, iters, nthreads))

    @property
    def t(self):
        return self.lib.adv_time(self.h)

    def _check(self, rc):
        if rc != 0:
            raise RuntimeError(self.lib.orc_last_error().decode())


def vertex_fields(cells, q, N, gam=1.4, n_nodes=None):
    """rho, u, v, p per mesh vertex, restating src/save_solution.cpp:13-46: cells visited in
    ascending order, vertex k of a cell takes local node (0, N, Np-1)[k], a later cell
    overwrites an earlier one."""
    cells = np.asarray(cells, dtype=np.int64).reshape(-1, 3)
    Np = (N + 1) * (N + 2) // 2
    q = np.asarray(q, dtype=np.float64).reshape(len(cells), Np, 4)
    n_nodes = int(cells.max()) + 1 if n_nodes is None else n_nodes
    out = np.zeros((4, n_nodes))
    local = (0, N, Np - 1)
    node = cells.reshape(-1)                         # visiting order: cell-major, vertex 0..2
    qv = q[np.repeat(np.arange(len(cells)), 3), np.tile(local, len(cells))]
    last = len(node) - 1 - np.unique(node[::-1], return_index=True)[1]   # last visit per vertex
    n, qq = node[last], qv[last]
    r = qq[:, 0]
    u = qq[:, 1] / r
    v = qq[:, 2] / r
    out[0, n], out[1, n], out[2, n] = r, u, v
    out[3, n] = (gam - 1) * (qq[:, 3] - 0.5 * (qq[:, 1] * u + qq[:, 2] * v))
    return out


def read_vtk_point_data(path):
    """The POINT_DATA arrays of a legacy-ASCII VTK file as {name: array}."""
    tok = open(path).read().split()
    i, out = tok.index("POINT_DATA"), {}
    n = int(tok[i + 1])
    i += 2
    while i < len(tok):
        if tok[i] == "SCALARS":
            name, i = tok[i + 1], i + 6           # SCALARS name type 1 LOOKUP_TABLE default
            out[name] = np.array(tok[i:i + n], dtype=np.float64)
            i += n
        elif tok[i] == "VECTORS":
            name, i = tok[i + 1], i + 3
            out[name] = np.array(tok[i:i + 3 * n], dtype=np.float64).reshape(n, 3)
            i += 3 * n
        else:
            raise ValueError("unexpected token " + tok[i])
    return out


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64).ravel()
    b = np.asarray(b, dtype=np.float64).ravel()
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))
