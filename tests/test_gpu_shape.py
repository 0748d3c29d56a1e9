"""Shape-aware functional (shape displacement held fixed) on the GPU against
the oracle's shape path (itself pinned on the CPU to the moved-mesh
identity): residual, stored-tangent Jacobian action and CSR assembly with a
non-trilinear order-2 shape field, with domain and boundary integrals."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, rel

pytestmark = pytest.mark.gpu


def _build(mat, c, bmat=None, n=3, p=2):
    import serac_gb300 as sg

    V = O.box_vertices(n, n, n, 0.1, 4)
    m = O.StructuredHexMesh(n, n, n, V)
    orc = O.OracleFunctional(m, p, c)
    orc.add_domain_integral(mat, PARAMS[mat])
    mesh = sg.Mesh.structured_hex(n, n, n, V)
    saf = sg.ShapeAwareFunctional(mesh, sg.H1(p, 3), sg.H1(p, c))
    saf.AddDomainIntegral(mat, PARAMS[mat])
    if bmat is not None:
        bp = [0.3, -0.2, 0.5] if bmat == O.BMAT_TRACTION else [0.7]
        orc.add_boundary_integral(bmat, [3, 6], bp)
        saf.AddBoundaryIntegral(bmat, [3, 6], bp)
    rng = np.random.default_rng(21)
    shape = rng.uniform(-0.04, 0.04, 3 * orc.nnodes) / n
    orc.set_shape(shape)
    return orc, saf, shape, rng


@pytest.mark.parametrize("mat,c,bmat", [(O.MAT_HEAT, 1, O.BMAT_HEAT_FLUX), (O.MAT_NEOHOOKEAN, 3, O.BMAT_TRACTION),
                                        (O.MAT_NEOHOOKEAN, 3, O.BMAT_PRESSURE), (O.MAT_ELASTIC_TEST, 3, None)])
def test_shape_aware_matches_oracle(cuda, mat, c, bmat):
    import serac_gb300 as sg

    orc, saf, shape, rng = _build(mat, c, bmat)
    u = rng.standard_normal(orc.ndofs) * (0.02 if c == 3 else 0.3)
    du = rng.standard_normal(orc.ndofs)
    sh = torch.tensor(shape, device=cuda)
    ut = torch.tensor(u, device=cuda)
    r = saf(0.0, sh, ut).cpu().numpy()
    assert rel(r, orc.residual(u)) <= 1e-12
    _, J = saf(0.0, sh, sg.differentiate_wrt(ut))
    assert rel(J(torch.tensor(du, device=cuda)).cpu().numpy(), orc.jvp(u, du)) <= 1e-12
    row_ptr, col, val = sg.assemble(J)
    A = orc.assemble(u)
    assert np.array_equal(row_ptr.cpu().numpy(), A.indptr) and np.array_equal(col.cpu().numpy(), A.indices)
    assert rel(val.cpu().numpy(), A.data) <= 1e-12


def test_zero_shape_and_reset(cuda):
    import serac_gb300 as sg

    orc, saf, shape, rng = _build(O.MAT_NEOHOOKEAN, 3, O.BMAT_PRESSURE)
    u = torch.tensor(rng.standard_normal(orc.ndofs) * 0.02, device=cuda)
    f = saf.functional
    r_plain = f.residual(0.0, u)
    f.set_shape_displacement(torch.zeros(3 * f.num_nodes, dtype=torch.float64, device=cuda))
    assert torch.equal(f.residual(0.0, u), r_plain)
    f.set_shape_displacement(torch.tensor(shape, device=cuda))
    assert not torch.equal(f.residual(0.0, u), r_plain)
    f.set_shape_displacement(None)
    assert torch.equal(f.residual(0.0, u), r_plain)
