"""Assembled dR/du (CSR) and its diagonal against the oracle.

The graph must be identical to serac's (every element's test x trial vdof
pair, sorted: dof_numbering.hpp:290-351) and the values within 1e-12
relative; the matrix times a vector must equal the matrix-free Jacobian
action (check_gradient.hpp:28-34).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import fields, rel
from tests.test_gpu_parity import _pair

pytestmark = pytest.mark.gpu

CASES = [(O.MAT_HEAT, 2), (O.MAT_HEAT, 1), (O.MAT_NEOHOOKEAN, 2), (O.MAT_NEOHOOKEAN, 1), (O.MAT_J2, 2),
         (O.MAT_THERMAL_TEST, 2), (O.MAT_ELASTIC_TEST, 1), (O.MAT_NONLINEAR_HEAT, 2)]


@pytest.mark.parametrize("mat,p", CASES)
def test_csr_graph_and_values(cuda, mat, p):
    import serac_gb300 as sg

    orc, f = _pair(mat, p, dims=(3, 2, 2))
    u, du = fields(orc.ndofs, mat, seed=21)
    ut = torch.tensor(u, device=cuda)
    r, g = f(0.0, sg.differentiate_wrt(ut))
    row_ptr, col, val = sg.assemble(g)
    A = orc.assemble(u)
    assert np.array_equal(row_ptr.cpu().numpy(), A.indptr)
    assert np.array_equal(col.cpu().numpy(), A.indices)
    assert rel(val.cpu().numpy(), A.data) <= 1e-12
    # matrix-free action equals the assembled matrix times the vector
    jv = g(torch.tensor(du, device=cuda)).cpu().numpy()
    assert rel(A @ du, jv) <= 1e-12
    d = f.assemble_diagonal().cpu().numpy()
    assert rel(d, A.diagonal()) <= 1e-12


def test_assembly_is_bitwise_reproducible(cuda):
    import serac_gb300 as sg

    orc, f = _pair(O.MAT_NEOHOOKEAN, 2, dims=(4, 4, 3))
    u, _ = fields(orc.ndofs, O.MAT_NEOHOOKEAN, seed=22, scale=0.5)
    f.linearize(0.0, torch.tensor(u, device=cuda))
    a = f.assemble_values().clone()
    b = f.assemble_values().clone()
    assert torch.isfinite(a).all()
    assert torch.equal(a, b)
