"""CPU: libgbpt builds, loads and exports every entry point declared in include/gbpt.h; argument
checks answer without touching the GPU."""
import ctypes
import os
import re

import pytest

import gbpt
from gbpt import _lib

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "gbpt.h")


def declared_symbols():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"GBPT_API\s+[^;]*?\b(gbpt_\w+)\s*\(", text, re.S)))


def test_library_exports_every_declared_symbol():
    lib = gbpt.load()
    names = declared_symbols()
    assert len(names) >= 10
    for n in names:
        assert hasattr(lib, n), n
    assert {n for n, _, _ in _lib.SIGNATURES} == set(names)


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
