"""Python mirror of the OP2 drop-in surface (include/op2_gb300.h).

Same names, argument meanings and order as OP2's C++ API as the reference's
driver uses it (src/airfoil.cpp:135-331), so a driver written against it reads
like the reference's own.  Errors raise Op2Error instead of exiting.

    import op2  # airfoil_op2_fem_gb300.op2
    op2.op_init(0)
    cells = op2.op_decl_set(K, "cells")
    q = op2.op_decl_dat(cells, 60, "double", q_host, "q")
    op2.op_par_loop_euler_rhs("euler_rhs", cells, op2.op_arg_dat(workingQ, -1, op2.OP_ID, 60, "double", op2.OP_READ), ...)
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import lib as _lib_loader

OP_READ, OP_WRITE, OP_RW, OP_INC, OP_MIN, OP_MAX = range(6)
OP_ID = None
OP_GBL = None


class Op2Error(RuntimeError):
    pass


class op_arg(C.Structure):
    _fields_ = [("dat", C.c_void_p), ("map", C.c_void_p), ("idx", C.c_int), ("dim", C.c_int),
                ("size", C.c_int), ("acc", C.c_int), ("argtype", C.c_int), ("data", C.c_void_p),
                ("type", C.c_char_p)]


# argument counts per loop: the airfoil app's, and the vortex and advection apps' where they
# differ (vortex/src/vortex.cpp:210-318, advec/src/advec.cpp:191-260)
_LOOPS = {"init_grid": (18,), "set_ic": (2, 4, 5), "neighbour_zero": (1,), "calc_dt": (3,),
          "get_neighbour_q": (9, 11), "get_bedge_q": (6, 8, 9), "euler_rhs": (10,), "set_workingQ": (5, 6),
          "update_Q": (6, 7), "l2_error": (9,), "advec_rhs": (10,)}
_configured = False
_keep = []  # host buffers whose addresses op_arg_gbl hands to the library


def _L():
    global _configured
    L = _lib_loader()
    if not _configured:
        vp, cp, ip = C.c_void_p, C.c_char_p, C.c_int
        L.op_init.argtypes = [ip, C.c_void_p, ip]
        L.op_exit.argtypes = []
        L.op_decl_set.restype = vp
        L.op_decl_set.argtypes = [ip, cp]
        L.op_decl_map.restype = vp
        L.op_decl_map.argtypes = [vp, vp, ip, vp, cp]
        L.op_decl_dat.restype = vp
        L.op_decl_dat.argtypes = [vp, ip, cp, vp, cp]
        L.op_decl_const2.argtypes = [cp, ip, cp, vp]
        L.op_fetch_data.argtypes = [vp, vp]
        L.op_get_size.restype = ip
        L.op_get_size.argtypes = [vp]
        L.op_timing_output.argtypes = []
        L.op2_gb300_last_error.restype = cp
        L.op2_gb300_set_exit_on_error.argtypes = [ip]
        L.op2_gb300_clear_error.argtypes = []
        L.op2_gb300_sync.restype = ip
        L.op2_gb300_reset.argtypes = []
        # Loops go through op2_gb300_par_loop (arguments in an array): passing many
        # structures by value through a foreign-function layer is not portable.
        L.op2_gb300_par_loop.restype = None
        L.op2_gb300_par_loop.argtypes = [cp, cp, vp, ip, C.POINTER(op_arg)]
        L.op2_gb300_set_exit_on_error(0)
        _configured = True
    return L


def _call(fn, *args):
    L = _L()
    L.op2_gb300_clear_error()
    r = fn(*args)
    msg = L.op2_gb300_last_error()
    if msg:
        raise Op2Error(msg.decode())
    return r


def op_init(diags=0):
    _L().op2_gb300_reset()
    _L().op_init(0, None, diags)


def op_exit():
    _L().op_exit()
    _keep.clear()


def op_decl_set(size, name):
    return _call(_L().op_decl_set, int(size), name.encode())


def op_decl_map(frm, to, dim, imap, name):
    a = np.ascontiguousarray(imap, dtype=np.int32)
    return _call(_L().op_decl_map, frm, to, int(dim), a.ctypes.data, name.encode())


def op_decl_dat(st, dim, typ, data, name):
    dt = np.float64 if typ == "double" else np.int32
    a = None if data is None else np.ascontiguousarray(data, dtype=dt)
    return _call(_L().op_decl_dat, st, int(dim), typ.encode(), None if a is None else a.ctypes.data, name.encode())


def op_decl_const2(name, dim, typ, data):
    dt = np.float64 if typ == "double" else np.int32
    a = np.ascontiguousarray(np.atleast_1d(data), dtype=dt).ravel()
    assert a.size >= dim
    _call(_L().op_decl_const2, name.encode(), int(dim), typ.encode(), a.ctypes.data)


_TYPES = {"double": b"double", "int": b"int"}  # kept alive: op_arg.type points at them


def op_arg_dat(dat, idx, mp, dim, typ, acc):
    """Same fields as the library's op_arg_dat, filled here (no structure return through FFI)."""
    return op_arg(dat, mp, int(idx) if mp else -1, int(dim), int(dim) * (4 if typ == "int" else 8),
                  int(acc), 0, None, _TYPES[typ])


def op_arg_gbl(var, dim, typ, acc):
    """var: a numpy array (1 element per dim) that the loop reads or (OP_MAX) writes."""
    assert isinstance(var, np.ndarray) and var.flags["C_CONTIGUOUS"]
    _keep.append(var)
    return op_arg(None, None, -1, int(dim), int(dim) * (4 if typ == "int" else 8), int(acc), 1,
                  var.ctypes.data, _TYPES[typ])


def op_fetch_data(dat, out):
    assert out.flags["C_CONTIGUOUS"]
    _call(_L().op_fetch_data, dat, out.ctypes.data)


def op_get_size(st):
    return _L().op_get_size(st)


def op_timing_output():
    _L().op_timing_output()


def _loop(name):
    def f(loop_name, st, *args):
        if len(args) not in _LOOPS[name]:
            raise Op2Error("op_par_loop_%s takes %s arguments" % (name, " or ".join(map(str, _LOOPS[name]))))
        arr = (op_arg * len(args))(*args)
        _call(_L().op2_gb300_par_loop, name.encode(), loop_name.encode(), st, len(args), arr)
    f.__name__ = "op_par_loop_" + name
    return f


op_par_loop_init_grid = _loop("init_grid")
op_par_loop_set_ic = _loop("set_ic")
op_par_loop_neighbour_zero = _loop("neighbour_zero")
op_par_loop_calc_dt = _loop("calc_dt")
op_par_loop_get_neighbour_q = _loop("get_neighbour_q")
op_par_loop_get_bedge_q = _loop("get_bedge_q")
op_par_loop_euler_rhs = _loop("euler_rhs")
op_par_loop_set_workingQ = _loop("set_workingQ")
op_par_loop_update_Q = _loop("update_Q")
op_par_loop_l2_error = _loop("l2_error")
op_par_loop_advec_rhs = _loop("advec_rhs")
