"""CPU: libgbpt builds, loads and exports every entry point declared in include/gbpt.h; argument
checks answer without touching the GPU."""
import ctypes
import os
import re

import pytest

import gbpt
from gbpt import _lib

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for h in sorted(os.listdir(INCLUDE)):
        if h.endswith(".h"):
            text = open(os.path.join(INCLUDE, h)).read()
            names |= set(re.findall(r"GBPT_API\s+[^;]*?\b(gbpt_\w+)\s*\(", text, re.S))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    lib = gbpt.load()
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    from gbpt import render
    bound = {n for n, _, _ in _lib.SIGNATURES} | {n for n, _, _ in render.RENDER_SIGNATURES}
    assert bound == set(names)


def test_status_strings_and_version():
    lib = gbpt.load()
    assert lib.gbpt_version() >= 1
    assert lib.gbpt_status_string(0) == b"ok"
    assert lib.gbpt_status_string(2) == b"out of memory"


def test_invalid_arguments_are_reported_not_fatal():
    lib = gbpt.load()
    assert lib.gbpt_bvh_build(None, None, 0, 0, None, None) == 1
    assert b"out is NULL" in lib.gbpt_last_error()
    assert lib.gbpt_trace_closest(None, None, None, None, 10, None, None) == 1
    assert b"bvh is NULL" in lib.gbpt_last_error()
    h = ctypes.c_void_p()
    assert lib.gbpt_bvh_build(None, None, 0, 5, None, ctypes.byref(h)) == 1
    with pytest.raises(gbpt.GbptError):
        _lib.check(1)
