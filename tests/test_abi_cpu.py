"""CPU checks of the C-ABI library: it loads, and it exports every entry
point that include/icep_gb300.h declares (no GPU work is launched)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(icep_[A-Za-z0-9_]+)\s*\(", src):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from icep_kapsel_gb300.build import build
    return ctypes.CDLL(build())


def test_header_declares_entry_points():
    names = declared_functions()
    assert "icep_create" in names and "icep_step" in names and "icep_Ax" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_create_rejects_bad_mesh_without_gpu_work(lib):
    from icep_kapsel_gb300 import abi
    lib.icep_create.restype = ctypes.c_void_p
    lib.icep_create.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
    p = abi.make_params(nx=24, ny=32, nz=32)  # not a power of two
    st = ctypes.c_int(0)
    ctx = lib.icep_create(ctypes.byref(p), None, 0, ctypes.byref(st))
    assert not ctx
    assert st.value != 0
