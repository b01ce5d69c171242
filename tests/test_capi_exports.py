"""libpfgb.so builds for sm_103a, loads without a GPU and exports every
function that include/pfgb.h declares (no compute calls here)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"PFGB_API\s+[\w\s\*]+?\b(pfgb_\w+)\s*\(", txt)
    return names


@pytest.fixture(scope="module")
def lib():
    from pyflow_solver_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "pfgb_step" in names and "pfgb_cg_solve" in names and len(names) >= 15


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_signatures_cover_the_header():
    from pyflow_solver_gb300 import _capi
    assert set(declared_symbols()) == set(_capi.SIGNATURES)


def test_version_and_error_channel(lib):
    lib.pfgb_version.restype = ctypes.c_int
    assert lib.pfgb_version() >= 100
    buf = ctypes.create_string_buffer(64)
    assert lib.pfgb_last_error(buf, 64) == 0
    # invalid arguments are rejected before any CUDA call
    from pyflow_solver_gb300 import _capi
    p = _capi.Params()
    p.nx, p.ny, p.dx, p.dy = 1, 5, 1.0, 1.0
    h = ctypes.c_void_p()
    lib.pfgb_create.argtypes = [ctypes.POINTER(_capi.Params), ctypes.POINTER(ctypes.c_void_p)]
    assert lib.pfgb_create(ctypes.byref(p), ctypes.byref(h)) == -1
    lib.pfgb_last_error(buf, 64)
    assert b"nx and ny" in buf.value
