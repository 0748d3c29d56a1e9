"""The Jacobian action between host buffers (sfx_jvp_host, Gradient.mult on
CPU tensors): the copies in, the kernels and the copies out are pipelined
over slabs of element layers, and the result must be bitwise that of
sfx_jvp on device buffers, and within 1e-12 of the oracle.  Slab counts that
do not divide the layer count, a single layer, order 1, the fallback for a
form with a boundary integral, pinned and pageable host memory.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, fields, mesh, rel

pytestmark = pytest.mark.gpu


def _form(mat, p, dims, boundary=False):
    import serac_gb300 as sg

    m = mesh(*dims, perturb=0.1, seed=5)
    c = O.COMPONENTS[mat]
    orc = O.OracleFunctional(m, p, c, nthreads=8)
    orc.add_domain_integral(mat, PARAMS[mat])
    f = sg.Functional(sg.Mesh.structured_hex(*dims, m.vertices), sg.H1(p, c))
    f.AddDomainIntegral(mat, PARAMS[mat])
    if boundary:
        bp = [0.1, 0.2, 0.3, 0.5, -0.4, 0.2]
        orc.add_boundary_integral(O.BMAT_TRACTION, (2, 6), bp)
        f.AddBoundaryIntegral(O.BMAT_TRACTION, (2, 6), bp)
    return orc, f


@pytest.mark.parametrize("mat,p,dims,boundary,pinned", [
    (O.MAT_NEOHOOKEAN, 2, (4, 3, 9), False, True),    # 8 slabs over 9 layers
    (O.MAT_NEOHOOKEAN, 2, (3, 4, 5), False, False),   # 5 slabs, pageable memory
    (O.MAT_J2, 2, (5, 4, 1), False, True),            # one layer
    (O.MAT_HEAT, 1, (6, 5, 11), False, True),         # order 1 (four elements per warp)
    (O.MAT_NEOHOOKEAN, 1, (4, 4, 7), False, True),
    (O.MAT_NEOHOOKEAN, 2, (4, 3, 6), True, True),     # boundary integral: unpipelined fallback
])
def test_host_jvp_matches_device_and_oracle(cuda, mat, p, dims, boundary, pinned):
    import serac_gb300 as sg

    orc, f = _form(mat, p, dims, boundary)
    # displacement amplitude well below the node spacing of these meshes (no inverted element)
    u, du = fields(orc.ndofs, mat, seed=11, scale=0.1)
    ut = torch.tensor(u, device=cuda)
    _, grad = f(0.0, sg.differentiate_wrt(ut))
    dev = grad.mult(torch.tensor(du, device=cuda)).cpu()
    assert bool(torch.isfinite(dev).all())
    h_du = torch.tensor(du)
    h_out = torch.empty(orc.ndofs, dtype=torch.float64)
    if pinned:
        h_du, h_out = h_du.pin_memory(), h_out.pin_memory()
    out = grad.mult(h_du, out=h_out)
    assert out.data_ptr() == h_out.data_ptr()
    assert torch.equal(out, dev), "host-buffer action differs from the device action"
    assert rel(out.numpy(), orc.jvp(u, du)) <= 1e-12
    # repeated calls reuse the pipeline's buffers and give the same bits
    again = grad.mult(h_du)
    assert torch.equal(again, dev)


def test_host_jvp_rejects_wrong_buffers(cuda):
    import serac_gb300 as sg

    orc, f = _form(O.MAT_NEOHOOKEAN, 2, (2, 2, 2))
    u, du = fields(orc.ndofs, O.MAT_NEOHOOKEAN, seed=1)
    _, grad = f(0.0, sg.differentiate_wrt(torch.tensor(u, device=cuda)))
    with pytest.raises(ValueError):
        grad.mult(torch.tensor(du, dtype=torch.float32))
    with pytest.raises(ValueError):
        grad.mult(torch.tensor(du[:-1]))
