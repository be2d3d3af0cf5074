"""The C-ABI library loads and exports every symbol the header declares (CPU, no compute)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "discoeb_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(deb_[a-z0-9_]+)\s*\(", txt)))


def test_header_declares_the_entry_points():
    syms = declared_symbols()
    for s in ("deb_plan_create", "deb_forward", "deb_get_power", "deb_plan_destroy"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from discoeb_gb300 import _native, build  # noqa: F401
    import discoeb_gb300.build as b

    b.build()
    lib = ctypes.CDLL(_native.LIB_PATH)
    for s in declared_symbols():
        assert hasattr(lib, s), s
    assert set(_native.EXPORTS) <= set(declared_symbols())


def test_host_side_argument_checks_without_gpu():
    """Calls that fail argument validation return before touching the device."""
    from discoeb_gb300 import _native

    L = _native.load()
    assert L.deb_version() == 1
    bad = _native.DebDims(2, 12, 17, 8, 3, 1, 0, 0)  # lmaxg < 3
    plan = ctypes.c_void_p()
    assert L.deb_plan_create(ctypes.byref(bad), 8, ctypes.byref(plan)) == -1
    assert L.deb_forward(None, None, 1, 40, None, None, 4, None, None, None, None, None, None) == -1
    assert L.deb_error_string(-5) == b"plan capacity exceeded"
    assert L.deb_nvar(ctypes.byref(_native.DebDims(12, 12, 17, 17, 15, 1, 0, 0))) == 323


def test_new_entry_points_check_their_arguments_without_gpu():
    """Argument checks of the launch-shape, grouped and table-producer entry
    points return before touching the device."""
    from discoeb_gb300 import _native, tables_gpu

    L = _native.load()
    dims = _native.DebDims(12, 12, 17, 17, 15, 1, 0, 0, 0)
    plan = ctypes.c_void_p()
    bad_shape = _native.DebLaunchCfg(7, 0)
    assert L.deb_plan_create_ex(ctypes.byref(dims), 8, ctypes.byref(bad_shape), ctypes.byref(plan)) == -1
    assert L.deb_plan_create_ex(ctypes.byref(dims), 8, ctypes.byref(_native.DebLaunchCfg(0, -1)),
                                ctypes.byref(plan)) == -1
    for bs in (0, 33):
        assert L.deb_plan_create_grouped(ctypes.byref(dims), 64, bs, ctypes.byref(plan)) == -1
    dense = _native.DebDims(12, 12, 17, 17, 15, 1, 0, 1, 0)
    assert L.deb_plan_create_grouped(ctypes.byref(dense), 64, 16, ctypes.byref(plan)) == -1
    assert L.deb_forward_grouped(None, None, 1, 40, None, None, 16, None, None, None, None, None, None) == -1
    assert L.deb_plan_launch_info(None, None, None) == -1
    assert L.deb_tables_blob_len(2, 512, 15) == -1
    assert L.deb_tables_blob_len(256, 512, 15) == tables_gpu.blob_len(256, 15)
    cfg = tables_gpu.DebBgCfg(256, 512, 8, 15, 128, 1e-9, 1e-3, 1e-6)
    # wrong blob length is refused by both producers
    assert L.deb_evolve_background(ctypes.byref(cfg), 1, 1, 1, 1, 1, 123, None, None) == -1
    assert L.deb_evolve_background_host(ctypes.byref(cfg), 1, 1, 1, 1, 1, 123, None, 1) == -1
    assert L.deb_tau_of_a(None, 1, 100, None, 1, None, None) == -1


def test_adjoint_and_frozen_producer_check_their_arguments_without_gpu():
    """The adjoint entry points and the frozen producer refuse bad arguments
    before touching the device."""
    from discoeb_gb300 import _native, tables_gpu

    L = _native.load()
    vp = ctypes.c_void_p
    plan = vp()
    small = _native.DebDims(4, 12, 17, 17, 15, 1, 0, 0, 0)           # lmaxg < 5: no adjoint
    assert L.deb_plan_create_adjoint(ctypes.byref(small), 8, 4, ctypes.byref(plan)) == -1
    full = _native.DebDims(12, 12, 17, 17, 15, 1, 1, 0, 0)           # return_full: no adjoint
    assert L.deb_plan_create_adjoint(ctypes.byref(full), 8, 4, ctypes.byref(plan)) == -1
    # deb_adjoint without a plan, and with npar out of range
    args = [None, None, None, 1, 6, 1000, None, None, None, 1, None, None, None, 10, None, None, 32, None, None,
            None, 1, None, None, None]
    assert L.deb_adjoint(*args) == -1
    # the record with checkpoints needs its buffers
    assert L.deb_forward_record_ckpt(None, None, 1, 1000, None, None, 1, None, None, None, None, None, None, 10,
                                     None, None, 32, None, None, None, None) == -1
    # the frozen producers need a leader array (and the device one its step buffer)
    cfg = tables_gpu.DebBgCfg(256, 512, 8, 3, 128, 1e-9, 1e-3, 1e-6)
    bl = tables_gpu.blob_len(256, 3)
    import numpy as np

    from discoeb_gb300.workloads import fiducial_mnu_param

    pm = np.ascontiguousarray(tables_gpu.param_matrix([fiducial_mnu_param()]))
    c = lambda a: vp(a.ctypes.data)
    tabs = np.zeros((1, bl))
    st = np.zeros(1, np.int32)
    consts, grd = tables_gpu.constants(), tables_gpu.grid(256, 3)
    assert L.deb_evolve_background_frozen_host(ctypes.byref(cfg), c(pm), 1, None, c(consts), c(grd), None, 0,
                                               c(tabs), bl, c(st), 1) == -1
    assert L.deb_evolve_background_frozen(ctypes.byref(cfg), 1, 1, None, 1, 1, None, 0, 1, bl, None, None) == -1
