"""The C-ABI library loads and exports every entry point include/arc/*.h declares (no GPU needed)."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include", "arc")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            text = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^\s*int\s+(arc_\w+)\s*\(", text, re.M))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_symbols()
    assert "arc_trace_frame" in names and "arc_upload_world" in names and len(names) >= 30


def test_library_exports_every_declared_symbol(native_lib):
    lib = ctypes.CDLL(native_lib.LIB_PATH)
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_wrapper_signatures_cover_headers(native_lib):
    assert set(declared_symbols()) <= set(native_lib.SIGNATURES)


def test_null_arguments_are_rejected_without_a_device(native_lib):
    L = native_lib.lib()
    assert L.arc_create(0, None) == -1
    assert L.arc_world_build(None, None, 0, ctypes.byref(ctypes.c_void_p())) == -1
    assert L.arc_default_palette(None) == -1
    assert L.arc_destroy(None) == 0


def test_builder_rejects_bad_grid(native_lib):
    from arcadia_gb300.layout import SceneParams

    with pytest.raises(native_lib.ArcError):
        native_lib.build_world(SceneParams(grid=(0, 1, 1)))


def test_python_bindings_fail_loudly_without_library(native_lib, monkeypatch):
    monkeypatch.setattr(native_lib, "LIB_PATH", "/nonexistent/libarc_trace.so")
    monkeypatch.setattr(native_lib, "_lib", None)
    with pytest.raises(native_lib.ArcError):
        native_lib.lib()
