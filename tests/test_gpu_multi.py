"""Multi-field forms on the GPU (sfx_mform_*: Functional<test(displacement,
acceleration, dK, dG)>, the residual SolidMechanics builds with
DependsOn<0, 1, parameters...>, solid_mechanics.hpp:243, 880-893) against the
oracle: residual, Jacobian action and transposed action with respect to each
argument field, FP64 1e-12, orders 1 and 2; the DependsOn mapping with the
form's fields in another order; a field no integral depends on."""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.golden.make_golden import multi_fields
from tests.problems import rel

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _pair(p, dims=(3, 3, 2), params=(1.3, 5.0, 0.25), order=(0, 1, 2, 3)):
    """order[k]: the form field holding material argument k."""
    import serac_gb300 as sg

    V = sg.box_vertices(*dims, perturb=0.1, seed=17)
    mesh = sg.Mesh.structured_hex(*dims, V)
    comps = [0] * 4
    for k, fld in enumerate(order):
        comps[fld] = O.MULTI_COMPONENTS[k]
    f = sg.MultiFunctional(mesh, sg.H1(p, 3), [sg.H1(p, c) for c in comps])
    f.AddDomainIntegral(sg.PARAM_NEOHOOKEAN, list(order), params)
    orc = O.OracleMultiFunctional(O.StructuredHexMesh(*dims, V), p, params)
    return f, orc


@pytest.mark.parametrize("p", [1, 2])
def test_multi_field_operators_match_oracle(cuda, p):
    import serac_gb300 as sg

    f, orc = _pair(p)
    flds = multi_fields(orc.nnodes, 60 + p)
    dev = [torch.tensor(x, device=cuda) for x in flds]
    assert rel(f(0.0, *dev).cpu().numpy(), orc.residual(flds)) <= TOL
    rng = np.random.default_rng(p)
    for w, c in enumerate(O.MULTI_COMPONENTS):
        args = list(dev)
        args[w] = sg.differentiate_wrt(dev[w])
        r, J = f(0.0, *args)
        assert rel(r.cpu().numpy(), orc.residual(flds)) <= TOL
        d = rng.standard_normal(c * orc.nnodes)
        jv = J(torch.tensor(d, device=cuda)).cpu().numpy()
        assert rel(jv, orc.jvp(flds, w, d)) <= TOL, w
        v = rng.standard_normal(3 * orc.nnodes)
        jt = J.mult_transpose(torch.tensor(v, device=cuda)).cpu().numpy()
        assert rel(jt, orc.jvp_transpose(flds, w, v)) <= TOL, w


def test_depends_on_maps_material_arguments_to_form_fields(cuda):
    """The form's fields in the order (dG, u, dK, a): DependsOn<1, 3, 2, 0>."""
    order = (1, 3, 2, 0)
    f, orc = _pair(2, dims=(2, 3, 2), order=order)
    flds = multi_fields(orc.nnodes, 71)
    form_fields = [None] * 4
    for k, fld in enumerate(order):
        form_fields[fld] = torch.tensor(flds[k], device=cuda)
    assert rel(f.residual(0.0, form_fields).cpu().numpy(), orc.residual(flds)) <= TOL
    rng = np.random.default_rng(3)
    for k, fld in enumerate(order):
        J = f.linearize(0.0, form_fields, fld)
        d = rng.standard_normal(O.MULTI_COMPONENTS[k] * orc.nnodes)
        assert rel(J.mult(torch.tensor(d, device=cuda)).cpu().numpy(), orc.jvp(flds, k, d)) <= TOL, k


def test_field_without_dependence_has_zero_derivative(cuda):
    import serac_gb300 as sg

    dims = (2, 2, 2)
    V = sg.box_vertices(*dims, perturb=0.1, seed=2)
    mesh = sg.Mesh.structured_hex(*dims, V)
    # five fields; the integral reads fields 0-3, field 4 is unused
    f = sg.MultiFunctional(mesh, sg.H1(2, 3), [sg.H1(2, c) for c in (3, 3, 1, 1, 1)])
    f.AddDomainIntegral(sg.PARAM_NEOHOOKEAN, [0, 1, 2, 3], [1.0, 5.0, 0.25])
    N = f.num_nodes
    flds = [torch.tensor(x, device=cuda) for x in multi_fields(N, 5)] + [torch.ones(N, dtype=torch.float64, device=cuda)]
    J = f.linearize(0.0, flds, 4)
    out = J.mult(torch.randn(N, dtype=torch.float64, device=cuda))
    assert torch.count_nonzero(out).item() == 0
    out_t = J.mult_transpose(torch.randn(3 * N, dtype=torch.float64, device=cuda))
    assert torch.count_nonzero(out_t).item() == 0


def test_multi_field_is_bitwise_reproducible(cuda):
    import serac_gb300 as sg

    f, orc = _pair(2)
    flds = [torch.tensor(x, device=cuda) for x in multi_fields(orc.nnodes, 80)]
    args = list(flds)
    args[2] = sg.differentiate_wrt(flds[2])
    _, J = f(0.0, *args)
    v = torch.randn(3 * orc.nnodes, dtype=torch.float64, device=cuda)
    a = J.mult_transpose(v).clone()
    b = J.mult_transpose(v).clone()
    assert torch.equal(a, b)
