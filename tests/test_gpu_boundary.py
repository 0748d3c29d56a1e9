"""Boundary integrals (AddBoundaryIntegral) against the oracle: residual,
Jacobian action (FP64 and FP32), CSR values and diagonal, alone and together
with a domain integral."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, mesh, rel

pytestmark = pytest.mark.gpu

BCASES = [
    (O.BMAT_HEAT_FLUX, 2, (1, 3, 6), [0.3, 0.7, 1.1]),
    (O.BMAT_HEAT_FLUX, 1, (2, 5), [0.1, -0.2, 0.5]),
    (O.BMAT_TRACTION, 1, (2, 5, 6), [0.1, 0.2, 0.3, 0.5, -0.4, 0.2]),
    (O.BMAT_TRACTION, 2, (4,), [0.0, 0.0, -1.0, 0.2, 0.1, 0.0]),
    (O.BMAT_PRESSURE, 2, (1, 2, 3, 4, 5, 6), [0.7]),
    (O.BMAT_PRESSURE, 1, (6,), [-0.4]),
]


def _pair(bmat, p, sides, params, domain=None, dims=(3, 2, 2)):
    import serac_gb300 as sg

    m = mesh(*dims, perturb=0.1, seed=5)
    c = O.BCOMPONENTS[bmat]
    orc = O.OracleFunctional(m, p, c)
    f = sg.Functional(sg.Mesh.structured_hex(*dims, m.vertices), sg.H1(p, c))
    if domain is not None:
        orc.add_domain_integral(domain, PARAMS[domain])
        f.AddDomainIntegral(domain, PARAMS[domain])
    orc.add_boundary_integral(bmat, sides, params)
    f.AddBoundaryIntegral(bmat, sides, params)
    return orc, f


@pytest.mark.parametrize("bmat,p,sides,params", BCASES)
@pytest.mark.parametrize("with_domain", [False, True])
def test_boundary_integrals(cuda, bmat, p, sides, params, with_domain):
    import serac_gb300 as sg

    domain = None
    if with_domain:
        domain = O.MAT_HEAT if O.BCOMPONENTS[bmat] == 1 else O.MAT_NEOHOOKEAN
    orc, f = _pair(bmat, p, sides, params, domain)
    rng = np.random.default_rng(31)
    u = rng.standard_normal(orc.ndofs) * 0.02
    du = rng.standard_normal(orc.ndofs)
    ut = torch.tensor(u, device=cuda)
    assert rel(f.residual(0.0, ut).cpu().numpy(), orc.residual(u)) <= 1e-12
    r, g = f(0.0, sg.differentiate_wrt(ut))
    assert rel(r.cpu().numpy(), orc.residual(u)) <= 1e-12
    ref = orc.jvp(u, du)
    dut = torch.tensor(du, device=cuda)
    if np.linalg.norm(ref) > 0:
        assert rel(g(dut).cpu().numpy(), ref) <= 1e-12
        assert rel(g(dut.float()).double().cpu().numpy(), ref) <= 1e-5
    else:
        assert float(torch.abs(g(dut)).max()) == 0.0
    row_ptr, col, val = sg.assemble(g)
    A = orc.assemble(u)
    assert np.array_equal(row_ptr.cpu().numpy(), A.indptr) and np.array_equal(col.cpu().numpy(), A.indices)
    if np.linalg.norm(A.data) > 0:
        assert rel(val.cpu().numpy(), A.data) <= 1e-12
        assert rel(f.assemble_diagonal().cpu().numpy(), A.diagonal()) <= 1e-12
