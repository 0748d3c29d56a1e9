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
        bp = {O.BMAT_TRACTION: [0.3, -0.2, 0.5, 0.1, 0.0, -0.2], O.BMAT_HEAT_FLUX: [0.7, 0.2, 0.4],
              O.BMAT_PRESSURE: [0.7]}[bmat]
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


@pytest.mark.parametrize("mat,c", [(O.MAT_HEAT, 1), (O.MAT_THERMAL_TEST, 1), (O.MAT_NEOHOOKEAN, 3),
                                   (O.MAT_ELASTIC_TEST, 3), (O.MAT_J2, 3)])
def test_shape_derivative_matches_finite_differences(cuda, mat, c):
    """dR/dp dshape on the GPU against central differences of the oracle's
    shape-aware residual (h = 1e-6), at a non-zero shape displacement."""
    import serac_gb300 as sg

    orc, saf, shape, rng = _build(mat, c)
    u = rng.standard_normal(orc.ndofs) * (0.02 if c == 3 else 0.3)
    dp = rng.uniform(-1.0, 1.0, 3 * orc.nnodes) / 3
    h = 1e-6
    orc.set_shape(shape + h * dp)
    rp = orc.residual(u)
    orc.set_shape(shape - h * dp)
    rm = orc.residual(u)
    fd = (rp - rm) / (2 * h)
    sh = torch.tensor(shape, device=cuda)
    ut = torch.tensor(u, device=cuda)
    r, dRdp = saf(0.0, sg.differentiate_wrt(sh), ut)
    orc.set_shape(shape)
    assert rel(r.cpu().numpy(), orc.residual(u)) <= 1e-12
    got = dRdp(torch.tensor(dp, device=cuda)).cpu().numpy()
    assert rel(got, fd) <= 1e-6


def test_shape_derivative_at_zero_shape_and_linearity(cuda):
    import serac_gb300 as sg

    orc, saf, shape, rng = _build(O.MAT_NEOHOOKEAN, 3)
    f = saf.functional
    u = torch.tensor(rng.standard_normal(orc.ndofs) * 0.02, device=cuda)
    zero = torch.zeros(3 * f.num_nodes, dtype=torch.float64, device=cuda)
    _, dRdp = saf(0.0, sg.differentiate_wrt(zero), u)
    a = torch.tensor(rng.standard_normal(3 * f.num_nodes), device=cuda)
    b = torch.tensor(rng.standard_normal(3 * f.num_nodes), device=cuda)
    lin = dRdp(2.0 * a - 3.0 * b)
    assert torch.allclose(lin, 2.0 * dRdp(a) - 3.0 * dRdp(b), rtol=1e-11, atol=1e-13)
    # at p = 0 the derivative equals that of the plain functional on moved vertices
    h = 1e-6
    orc.set_shape(h * a.cpu().numpy())
    rp = orc.residual(u.cpu().numpy())
    orc.set_shape(-h * a.cpu().numpy())
    rm = orc.residual(u.cpu().numpy())
    assert rel(dRdp(a).cpu().numpy(), (rp - rm) / (2 * h)) <= 1e-6


@pytest.mark.parametrize("mat,c,bmat", [(O.MAT_HEAT, 1, O.BMAT_HEAT_FLUX), (O.MAT_NEOHOOKEAN, 3, O.BMAT_TRACTION),
                                        (O.MAT_NEOHOOKEAN, 3, O.BMAT_PRESSURE)])
def test_shape_derivative_with_boundary_integrals(cuda, mat, c, bmat):
    """dR/dp dshape of a form with domain and boundary integrals (the boundary
    part carries the area correction and the shape-displaced position) against
    central differences of the oracle's shape-aware residual."""
    import serac_gb300 as sg

    orc, saf, shape, rng = _build(mat, c, bmat)
    u = rng.standard_normal(orc.ndofs) * (0.02 if c == 3 else 0.3)
    dp = rng.uniform(-1.0, 1.0, 3 * orc.nnodes) / 3
    h = 1e-6
    orc.set_shape(shape + h * dp)
    rp = orc.residual(u)
    orc.set_shape(shape - h * dp)
    rm = orc.residual(u)
    orc.set_shape(shape)
    _, dRdp = saf(0.0, sg.differentiate_wrt(torch.tensor(shape, device=cuda)), torch.tensor(u, device=cuda))
    got = dRdp(torch.tensor(dp, device=cuda)).cpu().numpy()
    assert rel(got, (rp - rm) / (2 * h)) <= 1e-6
