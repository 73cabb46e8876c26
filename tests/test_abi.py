"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: these run without a GPU)."""
from __future__ import annotations

import ctypes as C
import re
import subprocess

import pytest

from conftest import ROOT


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(cloth_[a-z0-9_]+)\s*\(", text))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    assert "cloth_step" in names and "cloth_create" in names and "cloth_batch_step" in names


def test_library_exports_every_declared_symbol(built):
    from acousticsim_gb300 import _native
    lib = _native.load()
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", str(_native.LIB_PATH)],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (cloth_[a-z0-9_]+)", out))
    assert declared_functions() <= exported


def test_bindings_cover_every_declared_symbol(built):
    from acousticsim_gb300 import _native
    assert declared_functions() <= set(_native.SIGNATURES)


def test_abi_version_and_errors(built):
    from acousticsim_gb300 import _native
    lib = _native.load()
    assert lib.cloth_abi_version() == 2
    assert lib.cloth_status_string(0) == b"ok"
    # NULL arguments are rejected with a status, not a crash
    assert lib.cloth_step(None, 0.0, None, None) == 1
    assert lib.cloth_grid_build(None, None, None, None, None, None, None, None) == 1
    assert b"NULL" in lib.cloth_last_error() or len(lib.cloth_last_error()) > 0


def test_no_device_is_an_error_not_a_crash(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from acousticsim_gb300 import _native
    lib = _native.load()
    h = C.c_void_p()
    assert lib.cloth_ctx_create(0, C.byref(h)) == 2  # CLOTH_ERR_CUDA


def test_graft_entry_build_is_importable():
    import importlib
    mod = importlib.import_module("__graft_entry__")
    assert callable(mod.build) and callable(mod.smoke)
