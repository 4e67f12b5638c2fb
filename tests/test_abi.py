"""The C-ABI library loads and exports every symbol include/*.h declares."""
import ctypes as C
import os
import re

import pytest

from sem2dpack_gb300 import _lib, abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in ("sem2d_gpu.h", "sem2d_host.h"):
        src = open(os.path.join(ROOT, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"\b(sem2d_\w+)\s*\(", src):
            names.add(m.group(1))
    return names


def test_all_declared_symbols_exported():
    L = _lib.lib()
    names = declared_functions()
    assert len(names) > 25
    missing = [n for n in sorted(names) if not hasattr(L, n)]
    assert not missing, missing
    # and the ctypes prototype table covers exactly the declared functions
    assert {p[0] for p in _lib.PROTOTYPES} == names


def test_struct_layouts_match():
    a, b = C.c_int(), C.c_int()
    assert _lib.lib().sem2d_abi_struct_sizes(C.byref(a), C.byref(b)) == 0
    assert a.value == C.sizeof(abi.ProblemDesc)
    assert b.value == C.sizeof(abi.Deck)


def test_version_and_errors_without_device():
    L = _lib.lib()
    assert L.sem2d_gpu_version() == 1
    # bad arguments are rejected before any device work
    h = C.c_void_p()
    assert L.sem2d_gpu_create(None, C.byref(h)) == abi.SEM2D_E_ARG
    assert b"null" in L.sem2d_gpu_last_error(None)
    assert L.sem2d_gpu_step(None, 1) == abi.SEM2D_E_ARG
