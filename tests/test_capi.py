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


def test_new_entry_points_validate_before_touching_a_device():
    """QoI, adjoint, sensitivity, element-table and tangent-storage entry
    points reject bad arguments on the host (no GPU needed)."""
    import numpy as np

    from serac_gb300 import _lib

    lib = _lib.load()
    h = ctypes.c_void_p()
    i32 = ctypes.POINTER(ctypes.c_int32)
    dp = ctypes.POINTER(ctypes.c_double)
    table = np.zeros((1, 8), dtype=np.int32)
    corners = np.zeros((1, 8, 3))
    # order 3 is not built; node id out of range; empty table; null tables
    assert lib.sfx_form_create_from_table(3, 1, 1, 8, table.ctypes.data_as(i32), corners.ctypes.data_as(dp),
                                          ctypes.byref(h)) == -5
    bad = table.copy()
    bad[0, 3] = 9
    assert lib.sfx_form_create_from_table(1, 1, 1, 8, bad.ctypes.data_as(i32), corners.ctypes.data_as(dp),
                                          ctypes.byref(h)) == -1
    assert b"out of range" in lib.sfx_last_error()
    assert lib.sfx_form_create_from_table(1, 1, 0, 8, table.ctypes.data_as(i32), corners.ctypes.data_as(dp),
                                          ctypes.byref(h)) == -1
    assert lib.sfx_form_create_from_table(1, 1, 1, 8, None, None, ctypes.byref(h)) == -1
    assert lib.sfx_qoi_create_from_table(2, 2, 1, 27, None, None, ctypes.byref(h)) == -5
    for call in (lambda: lib.sfx_jvp_transpose(None, None, None, None),
                 lambda: lib.sfx_jvp_transpose_f32(None, None, None, None),
                 lambda: lib.sfx_qoi_add_domain_integral(None, 0, None),
                 lambda: lib.sfx_qoi_evaluate(None, 0.0, None, None, None),
                 lambda: lib.sfx_qoi_gradient(None, 0.0, None, None, None, None),
                 lambda: lib.sfx_qoi_action(None, 0.0, None, None, None, None),
                 lambda: lib.sfx_qoi_shape_gradient(None, 0.0, None, None, None),
                 lambda: lib.sfx_shape_vjp(None, 0.0, None, None, None, None),
                 lambda: lib.sfx_form_set_tangent_storage(None, 1),
                 lambda: lib.sfx_form_add_boundary_integral_faces(None, 0, 0, None, None, None),
                 lambda: lib.sfx_form_add_face_set_faces(None, 0, None, None, None),
                 lambda: lib.sfx_solver_solve_adjoint(None, 0.0, None, None, None, None),
                 lambda: lib.sfx_set_param_field(None, 0, None, 0)):
        assert call() == -1


def test_python_side_validation():
    """QoI parameter counts and face lists are validated in Python before any
    call into the library."""
    from serac_gb300 import functional as F

    assert F._qoi_nparams(F.QOI_FIELD, 3, False) == 3
    assert F._qoi_nparams(F.QOI_NEOHOOKEAN_ENERGY, 3, False) == 2
    assert F._qoi_nparams(F.QOI_NORMAL_FIELD, 3, True) == 0
    with pytest.raises(ValueError):
        F._qoi_nparams(F.QOI_NORMAL_FIELD, 1, True)  # needs 3 components
    with pytest.raises(ValueError):
        F._qoi_nparams(F.QOI_NEOHOOKEAN_ENERGY, 3, True)  # domain only
    with pytest.raises(ValueError):
        F._face_arrays(([0, 1], [3]))
    e, s = F._face_arrays(([0, 1], [3, 6]))
    assert e.dtype.name == "int32" and list(s) == [3, 6]


def test_table_rejects_inverted_elements():
    """An element whose corners are left-handed in its lexicographic frame
    (for instance a wrong native -> lexicographic permutation) is rejected on
    the host."""
    import numpy as np

    from serac_gb300 import _lib

    lib = _lib.load()
    h = ctypes.c_void_p()
    table = np.arange(8, dtype=np.int32).reshape(1, 8)
    corners = np.array([[x, y, z] for z in (0.0, 1.0) for y in (0.0, 1.0) for x in (0.0, 1.0)]).reshape(1, 8, 3)
    corners[0, :, 0] = 1.0 - corners[0, :, 0]  # mirrored in x
    rc = lib.sfx_form_create_from_table(1, 1, 1, 8, table.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                        corners.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.byref(h))
    assert rc == -1
    assert b"inverted" in lib.sfx_last_error()


def test_missing_library_fails_loudly(monkeypatch):
    """No CPU fallback: without the built CUDA library the package refuses to
    run instead of computing elsewhere."""
    from serac_gb300 import _lib

    monkeypatch.setattr(_lib, "_LIB", None)
    monkeypatch.setattr(_lib, "LIB_PATH", "/nonexistent/libsfx_gb300.so")
    with pytest.raises(ImportError):
        _lib.load()
    with pytest.raises(ImportError):
        _lib.call("sfx_version")
