"""The C-ABI libraries load on a host without a GPU and export every symbol their headers
declare; calls that need a device fail with an error code, not a crash."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = set()
    for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text):
        name = m.group(1)
        if name.startswith(("dg_", "op_")) and not name.endswith("_t"):
            names.add(name)
    return names


def test_dg_header_symbols_exported(pkg):
    lib = ctypes.CDLL(pkg.LIB_PATH)
    names = declared_functions("dg_gb300.h")
    assert len(names) > 30
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_no_device_is_an_error_not_a_crash(pkg):
    import __graft_entry__ as g
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    mesh = pkg.Mesh.vortex_square(4)
    with pytest.raises(pkg.DGError):
        pkg.Solver(mesh, pkg.config())


def test_bad_config_rejected(pkg):
    mesh = pkg.Mesh.vortex_square(4)
    for cfg in (pkg.config(N=0), pkg.config(N=7), pkg.config(cfl=0.0), pkg.config(gam=1.0), pkg.config(app=5)):
        with pytest.raises(pkg.DGError):
            pkg.Solver(mesh, cfg)


def test_element_form_selector(pkg):
    """Host logic of the element-kernel form selector: 3 (the tensor-core forms) by default,
    0..3 taken as given, anything else back to the default."""
    lib = pkg.lib()
    prev = lib.dg_elem_variant()
    try:
        assert prev == 3
        for v in (0, 1, 2, 3):
            lib.dg_set_elem_variant(v)
            assert lib.dg_elem_variant() == v
        for v in (-1, 4, 99):
            lib.dg_set_elem_variant(v)
            assert lib.dg_elem_variant() == 3
    finally:
        lib.dg_set_elem_variant(prev)


def test_once_table_bookkeeping(pkg):
    """Host logic behind the per-(device, order) operator uploads: threads racing through every
    (device, slot) pair upload each pair exactly once, a failed upload is retried by a later call,
    and nothing is marked loaded before it is."""
    lib = pkg.lib()
    devices, slots = 4, 7
    ups = (ctypes.c_int * (devices * slots))()
    tries = (ctypes.c_int * (devices * slots))()
    assert lib.dg_once_table_selftest(8, devices, ups, tries) == 0
    assert list(ups) == [1] * (devices * slots)
    assert list(tries) == [2 if k % 3 == 0 else 1 for k in range(devices * slots)]
    assert lib.dg_once_table_selftest(0, devices, ups, tries) != 0


def test_order_tables_query_without_device(pkg):
    """With no device nothing is loaded on any (device, order); out-of-range pairs are -1."""
    lib = pkg.lib()
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    for dev in (0, 1, 63):
        for N in range(1, 7):
            assert lib.dg_order_tables_loaded(dev, N) == 0
        assert lib.dg_rhs_noalloc_ready(dev) == 0
    for dev, N in ((-1, 3), (64, 3), (0, 0), (0, 7)):
        assert lib.dg_order_tables_loaded(dev, N) == -1
    assert lib.dg_rhs_noalloc_ready(64) == -1


def test_persistent_element_kernel_selector(pkg):
    """Host logic of the warp-specialised element kernel switch: off (0) by default, 0..2 taken
    as given, anything else back to off."""
    lib = pkg.lib()
    prev = lib.dg_elem_ws()
    try:
        assert prev == 0
        for v in (0, 1, 2):
            lib.dg_set_elem_ws(v)
            assert lib.dg_elem_ws() == v
        for v in (-1, 3, 77):
            lib.dg_set_elem_ws(v)
            assert lib.dg_elem_ws() == 0
    finally:
        lib.dg_set_elem_ws(prev)
