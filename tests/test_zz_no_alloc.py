"""The no-allocation residual entry point (sfx_residual_structured_noalloc).

It exists for callers that cannot allocate device memory: the caller brings
the vertex coordinates, the field and the output vector, and the library's
element-residual scratch is a fixed device array.  This test calls it through
the C ABI, twice in a row on the same inputs, and checks each result against
the regular entry point (sfx_residual, whose scratch comes from the form) and
against the CPU oracle, at the tolerance of the other FP64 parity tests
(1e-12 relative), plus the size limit.  Collected last so that a failure here stops a -x run only after
every other test has run; it also passes alone in a fresh process.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

TOL64 = 1e-12


def _noalloc(lib, dims, order, material, params, V_dev, u, r):
    prm = np.ascontiguousarray(params, dtype=np.float64)
    return lib.sfx_residual_structured_noalloc(
        dims[0], dims[1], dims[2], order, material, prm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
        ctypes.c_void_p(V_dev.data_ptr()), ctypes.c_void_p(u.data_ptr()), ctypes.c_void_p(r.data_ptr()),
        ctypes.c_double(0.0), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("material,order,comps,params", [
    (0, 2, 1, [1.3, 0.7]),   # SFX_MAT_HEAT
    (0, 1, 1, [1.0, 1.0]),
    (1, 2, 3, [5.0, 0.25]),  # SFX_MAT_NEOHOOKEAN
    (1, 1, 3, [5.0, 0.25]),
])
def test_noalloc_residual_matches_regular_entry_point(cuda, material, order, comps, params):
    import serac_gb300 as sg
    from serac_gb300 import _lib

    lib = _lib.load()
    lib.sfx_residual_structured_noalloc.restype = ctypes.c_int
    lib.sfx_residual_structured_noalloc.argtypes = [ctypes.c_int] * 5 + [
        ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
        ctypes.c_void_p]
    dims = (5, 4, 3)
    V = sg.box_vertices(*dims, perturb=0.1, seed=3)
    f = sg.Functional(sg.Mesh.structured_hex(*dims, V), sg.H1(order, comps))
    f.AddDomainIntegral(material, params)
    rng = np.random.default_rng(17)
    V_dev = torch.tensor(V, device=cuda)
    for call in range(2):
        u = torch.tensor(rng.standard_normal(f.ndofs) * 0.01, device=cuda)
        expected = f.residual(0.0, u)
        r = torch.full_like(u, float("nan"))
        rc = _noalloc(lib, dims, order, material, params, V_dev, u, r)
        assert rc == 0, lib.sfx_last_error()
        torch.cuda.synchronize()
        assert torch.isfinite(r).all()
        err = (torch.linalg.norm(r - expected) / torch.linalg.norm(expected)).item()
        assert err <= TOL64, (call, err)


def test_noalloc_residual_matches_oracle(cuda):
    """The same entry point against the CPU oracle (serac's residual
    restated), Neo-Hookean Q2 on a perturbed mesh, two calls in a row."""
    import serac_gb300 as sg
    from oracle import oracle as O
    from serac_gb300 import _lib

    lib = _lib.load()
    lib.sfx_residual_structured_noalloc.restype = ctypes.c_int
    lib.sfx_residual_structured_noalloc.argtypes = [ctypes.c_int] * 5 + [
        ctypes.POINTER(ctypes.c_double), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
        ctypes.c_void_p]
    dims, params = (6, 5, 4), [5.0, 0.25]
    V = sg.box_vertices(*dims, perturb=0.1, seed=5)
    orc = O.OracleFunctional(O.StructuredHexMesh(*dims, V), 2, 3)
    orc.add_domain_integral(O.MAT_NEOHOOKEAN, params)
    V_dev = torch.tensor(V, device=cuda)
    rng = np.random.default_rng(23)
    for call in range(2):
        u = rng.standard_normal(orc.ndofs) * 0.005  # keeps det F > 0 at every point
        u_dev = torch.tensor(u, device=cuda)
        r = torch.full_like(u_dev, float("nan"))
        assert _noalloc(lib, dims, 2, 1, params, V_dev, u_dev, r) == 0, lib.sfx_last_error()
        torch.cuda.synchronize()
        ref = orc.residual(u)
        err = np.linalg.norm(r.cpu().numpy() - ref) / np.linalg.norm(ref)
        assert err <= TOL64, (call, err)


def test_noalloc_rejects_meshes_beyond_the_scratch(cuda):
    from serac_gb300 import _lib

    lib = _lib.load()
    lib.sfx_residual_structured_noalloc.restype = ctypes.c_int
    dummy = torch.zeros(8, dtype=torch.float64, device=cuda)
    prm = np.array([5.0, 0.25])
    # 40^3 vector Q2 elements need 40^3 * 81 > 4,194,304 doubles of scratch
    rc = lib.sfx_residual_structured_noalloc(
        40, 40, 40, 2, 1, prm.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), ctypes.c_void_p(dummy.data_ptr()),
        ctypes.c_void_p(dummy.data_ptr()), ctypes.c_void_p(dummy.data_ptr()), ctypes.c_double(0.0), None)
    assert rc == -5
    assert b"scratch" in lib.sfx_last_error()
