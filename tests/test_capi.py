"""The C-ABI library loads on a machine without a GPU and exports every entry
point declared in include/sfx.h; argument checks fail loudly without touching
a device."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:const\s+)?\w+\*?\s+\**(sfx_\w+)\s*\(", text, re.M))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for n in ("sfx_residual", "sfx_jvp", "sfx_jvp_f32", "sfx_linearize", "sfx_assemble_csr", "sfx_csr_graph"):
        assert n in names


def test_library_exports_every_declared_symbol():
    from serac_gb300 import _lib

    lib = _lib.load()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.SIGNATURES) >= declared_symbols()


def test_invalid_arguments_fail_loudly():
    from serac_gb300 import _lib

    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.sfx_mesh_create_structured_hex(0, 1, 1, None, ctypes.byref(h)) == -1
    assert b"dimensions" in lib.sfx_last_error()
    assert lib.sfx_residual(None, 0.0, None, None, None) == -1
    with pytest.raises(_lib.SfxError):
        _lib.call("sfx_form_create", None, 2, 3, ctypes.byref(h))
