"""ctypes binding of the sfx C ABI (include/sfx.h).

The library is the in-tree ``serac_gb300/libsfx_gb300.so`` built by
``serac_gb300/build.py``.  There is no fallback: if the library is missing or
a call fails, an exception is raised.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libsfx_gb300.so")

SFX_OK = 0
STATUS = {
    -1: "SFX_ERR_INVALID",
    -2: "SFX_ERR_CUDA",
    -3: "SFX_ERR_NONFINITE",
    -4: "SFX_ERR_TIMEOUT",
    -5: "SFX_ERR_UNSUPPORTED",
    -6: "SFX_ERR_NOMEM",
}

_c = ctypes
_vp = _c.c_void_p
_i64p = _c.POINTER(_c.c_int64)
_dp = _c.POINTER(_c.c_double)

# name -> (restype, argtypes); every entry point declared in include/sfx.h
SIGNATURES = {
    "sfx_last_error": (_c.c_char_p, []),
    "sfx_version": (_c.c_int, []),
    "sfx_mesh_create_structured_hex": (_c.c_int, [_c.c_int, _c.c_int, _c.c_int, _dp, _c.POINTER(_vp)]),
    "sfx_mesh_destroy": (_c.c_int, [_vp]),
    "sfx_mesh_num_elements": (_c.c_int, [_vp, _i64p]),
    "sfx_form_create": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.POINTER(_vp)]),
    "sfx_form_destroy": (_c.c_int, [_vp]),
    "sfx_form_num_dofs": (_c.c_int, [_vp, _i64p]),
    "sfx_form_add_domain_integral": (_c.c_int, [_vp, _c.c_int, _dp, _c.c_int]),
    "sfx_form_add_boundary_integral": (_c.c_int, [_vp, _c.c_int, _c.c_int, _dp]),
    "sfx_form_set_shape_displacement": (_c.c_int, [_vp, _vp, _vp]),
    "sfx_shape_jvp": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp, _vp]),
    "sfx_residual": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp]),
    "sfx_linearize": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp]),
    "sfx_form_set_jvp_mode": (_c.c_int, [_vp, _c.c_int]),
    "sfx_jvp": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_jvp_host": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_set_param_field": (_c.c_int, [_vp, _c.c_int, _vp, _c.c_int]),
    "sfx_form_set_tangent_storage": (_c.c_int, [_vp, _c.c_int]),
    "sfx_jvp_transpose": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_jvp_transpose_f32": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_qoi_create": (_c.c_int, [_vp, _c.c_int, _c.c_int, _vp]),
    "sfx_form_create_from_table": (_c.c_int, [_c.c_int, _c.c_int, _c.c_int64, _c.c_int64, _vp, _vp, _vp]),
    "sfx_qoi_create_from_table": (_c.c_int, [_c.c_int, _c.c_int, _c.c_int64, _c.c_int64, _vp, _vp, _vp]),
    "sfx_form_add_boundary_integral_faces": (_c.c_int, [_vp, _c.c_int, _c.c_int64, _vp, _vp, _vp]),
    "sfx_form_add_face_set_faces": (_c.c_int, [_vp, _c.c_int64, _vp, _vp, _vp]),
    "sfx_qoi_add_boundary_integral_faces": (_c.c_int, [_vp, _c.c_int, _c.c_int64, _vp, _vp, _vp]),
    "sfx_qoi_add_domain_integral": (_c.c_int, [_vp, _c.c_int, _vp]),
    "sfx_qoi_add_boundary_integral": (_c.c_int, [_vp, _c.c_int, _c.c_int, _vp]),
    "sfx_qoi_evaluate": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp]),
    "sfx_qoi_gradient": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp, _vp]),
    "sfx_qoi_action": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp, _vp]),
    "sfx_qoi_shape_gradient": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp]),
    "sfx_shape_vjp": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp, _vp]),
    "sfx_jvp_f32": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_jvp_element": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_jvp_element_f32": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_selftest_bounded_wait": (_c.c_int, [_c.c_uint]),
    "sfx_selftest_umma_tile": (_c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _vp]),
    "sfx_csr_nnz": (_c.c_int, [_vp, _i64p]),
    "sfx_csr_graph": (_c.c_int, [_vp, _vp, _vp, _vp]),
    "sfx_assemble_csr": (_c.c_int, [_vp, _vp, _vp]),
    "sfx_assemble_diagonal": (_c.c_int, [_vp, _vp, _vp]),
    "sfx_residual_structured_noalloc": (_c.c_int, [_c.c_int] * 5 + [_dp, _vp, _vp, _vp, _c.c_double, _vp]),
    "sfx_form_get_layout": (_c.c_int, [_vp, _vp]),
    "sfx_form_add_face_set": (_c.c_int, [_vp, _c.c_int, _c.POINTER(_c.c_int)]),
    "sfx_form_get_face_layout": (_c.c_int, [_vp, _c.c_int, _vp]),
    "sfx_scatter_add": (_c.c_int, [_vp, _vp, _vp, _c.c_int, _vp]),
    "sfx_scatter_add_f32": (_c.c_int, [_vp, _vp, _vp, _c.c_int, _vp]),
    "sfx_update_qdata": (_c.c_int, [_vp, _c.c_int]),
    "sfx_qdata_size": (_c.c_int, [_vp, _i64p]),
    "sfx_set_qdata": (_c.c_int, [_vp, _dp]),
    "sfx_get_qdata": (_c.c_int, [_vp, _dp]),
    "sfx_mform_create": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _c.POINTER(_c.c_int), _c.POINTER(_vp)]),
    "sfx_mform_destroy": (_c.c_int, [_vp]),
    "sfx_mform_num_nodes": (_c.c_int, [_vp, _i64p]),
    "sfx_mform_add_domain_integral": (_c.c_int, [_vp, _c.c_int, _c.POINTER(_c.c_int), _c.c_int, _dp, _c.c_int]),
    "sfx_mform_residual": (_c.c_int, [_vp, _c.c_double, _c.POINTER(_vp), _vp, _vp]),
    "sfx_mform_linearize": (_c.c_int, [_vp, _c.c_double, _c.POINTER(_vp), _c.c_int, _vp]),
    "sfx_mform_jvp": (_c.c_int, [_vp, _c.c_int, _vp, _vp, _vp]),
    "sfx_mform_jvp_transpose": (_c.c_int, [_vp, _c.c_int, _vp, _vp, _vp]),
    # include/sfx_learned.h
    "sfx_lnet_create": (_c.c_int, [_c.c_uint64, _c.POINTER(_vp)]),
    "sfx_lnet_destroy": (_c.c_int, [_vp]),
    "sfx_lnet_num_params": (_c.c_int, [_vp, _i64p]),
    "sfx_lnet_get_params": (_c.c_int, [_vp, _c.POINTER(_c.c_float), _c.c_int64]),
    "sfx_lnet_set_params": (_c.c_int, [_vp, _c.POINTER(_c.c_float), _c.c_int64]),
    "sfx_lnet_apply": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _vp, _vp, _vp]),
    "sfx_lnet_gradient": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _vp, _vp, _vp, _c.POINTER(_c.c_float),
                                     _c.POINTER(_c.c_float), _vp]),
    "sfx_lnet_train_step": (_c.c_int, [_vp, _c.c_int, _c.c_int, _c.c_int, _c.c_int, _vp, _vp, _vp, _c.c_float,
                                       _c.POINTER(_c.c_float), _vp]),
    # include/sfx_solver.h (struct arguments passed by address)
    "sfx_solver_default_options": (_c.c_int, [_vp]),
    "sfx_solver_create": (_c.c_int, [_vp, _vp, _c.POINTER(_vp)]),
    "sfx_solver_destroy": (_c.c_int, [_vp]),
    "sfx_solver_set_essential": (_c.c_int, [_vp, _i64p, _c.c_int64]),
    "sfx_solver_solve": (_c.c_int, [_vp, _c.c_double, _vp, _vp]),
    "sfx_solver_solve_linear": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp, _vp]),
    "sfx_solver_solve_adjoint": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp, _vp]),
    "sfx_solver_warm_start": (_c.c_int, [_vp, _c.c_double, _vp, _vp, _vp]),
    "sfx_solver_get_stats": (_c.c_int, [_vp, _vp]),
    "sfx_solver_set_learned": (_c.c_int, [_vp, _vp, _c.c_int, _c.c_int, _c.c_int, _vp]),
}

_LIB = None


class SfxError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


def load():
    """Load the library (once) and declare every entry point."""
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"sfx CUDA library not built: {LIB_PATH} (run serac_gb300/build.py)")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = lib
    return _LIB


def check(rc):
    if rc != SFX_OK:
        msg = load().sfx_last_error()
        raise SfxError(rc, msg.decode() if msg else "")
    return rc


def call(name, *args):
    return check(getattr(load(), name)(*args))
