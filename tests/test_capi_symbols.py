"""The C-ABI library builds here, loads, and exports every function that
include/bgo.h declares; the tools library exports those of include/bgo_tools.h
(no device calls: this runs without a GPU)."""
import ctypes
import os
import re

import pytest

from beguidedoff_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header="bgo.h"):
    txt = open(os.path.join(ROOT, "include", header)).read()
    return sorted(set(re.findall(r"^int (bgo_\w+)\(", txt, flags=re.M)))


def test_header_and_binding_agree():
    assert _declared() == sorted(_native.EXPORTED)
    assert _declared("bgo_tools.h") == sorted(_native.TOOLS_EXPORTED)


def test_library_exports_every_declared_symbol():
    try:
        path = build.build()
    except (RuntimeError, FileNotFoundError) as e:  # no nvcc on this host
        pytest.skip(f"cannot build: {e}")
    lib = ctypes.CDLL(path)
    for name in _declared():
        assert hasattr(lib, name), name
    tools = ctypes.CDLL(build.TOOLS_PATH)
    for name in _declared("bgo_tools.h"):
        assert hasattr(tools, name), name
        assert not hasattr(lib, name), f"{name} is a tool, not in the product library"
    lib.bgo_version.restype = ctypes.c_int
    assert lib.bgo_version() >= 100
    buf = ctypes.create_string_buffer(64)
    assert lib.bgo_last_error(buf, 64) == 0
