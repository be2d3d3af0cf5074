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
