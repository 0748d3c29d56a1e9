"""Parity of the sfx CUDA kernels (through the C ABI) with the oracle.

FP64 residual and Jacobian action: relative l2 error <= 1e-12 against the
oracle's restatement of serac's element arithmetic (pinned to serac's own
kernels in test_oracle.py).  FP32 Jacobian action: relative l2 error <= 1e-5
against the FP64 oracle.  Repeated calls are bit-identical (no atomics).
"""
import numpy as np
import pytest
import torch

from oracle import oracle as O
from tests.problems import PARAMS, fields, mesh, rel

pytestmark = pytest.mark.gpu

TOL64 = 1e-12
TOL32 = 1e-5

CASES = [(mat, p) for mat in (O.MAT_HEAT, O.MAT_NONLINEAR_HEAT, O.MAT_THERMAL_TEST, O.MAT_NEOHOOKEAN, O.MAT_J2,
                              O.MAT_ELASTIC_TEST) for p in (1, 2)]


def _pair(mat, p, dims=(4, 3, 2), perturb=0.1, per_element=False, seed=0):
    import serac_gb300 as sg

    m = mesh(*dims, perturb=perturb, seed=seed + 1)
    c = O.COMPONENTS[mat]
    orc = O.OracleFunctional(m, p, c, nthreads=8)
    params = PARAMS[mat]
    if per_element and params is not None:
        rng = np.random.default_rng(seed + 7)
        pe = np.tile(np.asarray(params, dtype=np.float64), (m.ne, 1))
        pe[:, -1] *= np.exp(0.5 * rng.standard_normal(m.ne))
        params = pe
    orc.add_domain_integral(mat, params)
    mesh_g = sg.Mesh.structured_hex(*dims, m.vertices)
    f = sg.Functional(mesh_g, sg.H1(p, c))
    if params is not None:
        f.AddDomainIntegral(mat, params, per_element=per_element)
    else:
        f.AddDomainIntegral(mat)
    return orc, f


@pytest.mark.parametrize("mode", [0, 1], ids=["stored", "recompute"])
@pytest.mark.parametrize("mat,p", CASES)
def test_residual_and_jvp_fp64(cuda, mat, p, mode):
    orc, f = _pair(mat, p)
    f.set_jvp_mode(mode)
    u, du = fields(orc.ndofs, mat, seed=3)
    ut = torch.tensor(u, device=cuda)
    dut = torch.tensor(du, device=cuda)
    r = f.residual(0.0, ut).cpu().numpy()
    assert rel(r, orc.residual(u)) <= TOL64
    r2, grad = f(0.0, sg_wrt(ut))
    assert rel(r2.cpu().numpy(), orc.residual(u)) <= TOL64
    jv = grad(dut).cpu().numpy()
    ref = orc.jvp(u, du)
    assert rel(jv, ref) <= TOL64
    # FP32 inner Jacobian action against the FP64 oracle
    jv32 = grad(dut.float()).double().cpu().numpy()
    assert rel(jv32, ref) <= TOL32


def sg_wrt(u):
    import serac_gb300 as sg

    return sg.differentiate_wrt(u)


@pytest.mark.parametrize("mode", [0, 1], ids=["stored", "recompute"])
@pytest.mark.parametrize("mat", [O.MAT_HEAT, O.MAT_NEOHOOKEAN, O.MAT_J2])
def test_per_element_parameters(cuda, mat, mode):
    orc, f = _pair(mat, 2, dims=(3, 3, 3), per_element=True, seed=5)
    f.set_jvp_mode(mode)
    u, du = fields(orc.ndofs, mat, seed=9)
    ut = torch.tensor(u, device=cuda)
    f.linearize(0.0, ut)
    assert rel(f.residual(0.0, ut).cpu().numpy(), orc.residual(u)) <= TOL64
    assert rel(f.gradient(torch.tensor(du, device=cuda)).cpu().numpy(), orc.jvp(u, du)) <= TOL64


@pytest.mark.parametrize("mode", [0, 1], ids=["stored", "recompute"])
def test_bitwise_reproducible(cuda, mode):
    orc, f = _pair(O.MAT_NEOHOOKEAN, 2, dims=(6, 5, 4))
    f.set_jvp_mode(mode)
    u, du = fields(orc.ndofs, O.MAT_NEOHOOKEAN, seed=11, scale=0.25)
    ut = torch.tensor(u, device=cuda)
    dut = torch.tensor(du, device=cuda)
    f.linearize(0.0, ut)
    a = f.gradient(dut).clone()
    b = f.gradient(dut).clone()
    assert torch.isfinite(a).all()
    assert torch.equal(a, b)
    assert rel(a.cpu().numpy(), orc.jvp(u, du)) <= TOL64
    ra = f.residual(0.0, ut).clone()
    rb = f.residual(0.0, ut).clone()
    assert torch.equal(ra, rb)


@pytest.mark.parametrize("mode", [0, 1], ids=["stored", "recompute"])
def test_j2_state_update_matches_oracle(cuda, mode):
    orc, f = _pair(O.MAT_J2, 1, dims=(3, 2, 2))
    f.set_jvp_mode(mode)
    u, du = fields(orc.ndofs, O.MAT_J2, seed=13)
    ut = torch.tensor(u, device=cuda)
    # commit plastic state at u, then evaluate at 1.5 u with that state
    f.updateQdata(True)
    f.residual(0.0, ut)
    f.updateQdata(False)
    orc.residual(u, update_state=True)
    st = f.qdata().reshape(orc.state.shape)
    assert np.max(np.abs(st - orc.state)) <= 1e-12 * max(1.0, np.max(np.abs(orc.state)))
    assert np.max(orc.state[..., 9]) > 0.0  # some points yielded
    u2 = 1.5 * u
    ut2 = torch.tensor(u2, device=cuda)
    f.linearize(0.0, ut2)
    assert rel(f.residual(0.0, ut2).cpu().numpy(), orc.residual(u2)) <= TOL64
    assert rel(f.gradient(torch.tensor(du, device=cuda)).cpu().numpy(), orc.jvp(u2, du)) <= TOL64


def test_config1_heat_q2_16cubed(cuda):
    """Steady heat, 16^3 Q2 scalar (35,937 DOF), k = 1, f = 1: residual at u = 0
    and Jv with a seeded N(0,1) vector."""
    import serac_gb300 as sg

    n = 16
    m = O.StructuredHexMesh(n, n, n, O.box_vertices(n, n, n))
    orc = O.OracleFunctional(m, 2, 1, nthreads=8)
    orc.add_domain_integral(O.MAT_HEAT, [1.0, 1.0])
    f = sg.Functional(sg.Mesh.structured_hex(n, n, n, m.vertices), sg.H1(2, 1))
    f.AddDomainIntegral(sg.HEAT, [1.0, 1.0])
    assert f.ndofs == 35937
    u = np.zeros(f.ndofs)
    du = np.random.default_rng(0).standard_normal(f.ndofs)
    ut = torch.tensor(u, device=cuda)
    r, g = f(0.0, sg.differentiate_wrt(ut))
    assert rel(r.cpu().numpy(), orc.residual(u)) <= TOL64
    assert rel(g(torch.tensor(du, device=cuda)).cpu().numpy(), orc.jvp(u, du)) <= TOL64


@pytest.mark.parametrize("mat", [O.MAT_HEAT, O.MAT_NEOHOOKEAN, O.MAT_J2])
def test_set_parameters_in_place(cuda, mat):
    """sfx_set_param_field (BasePhysics::setParameter as per-element values):
    a form whose parameters are replaced in place reproduces, bit for bit, a
    form built with those parameters, and matches the oracle."""
    import serac_gb300 as sg

    orc, fresh = _pair(mat, 2, dims=(3, 3, 2), per_element=True, seed=11)
    m = mesh(3, 3, 2, perturb=0.1, seed=12)
    f = sg.Functional(sg.Mesh.structured_hex(3, 3, 2, m.vertices), sg.H1(2, O.COMPONENTS[mat]))
    f.AddDomainIntegral(mat, PARAMS[mat])
    u, du = fields(orc.ndofs, mat, seed=13)
    ut, dut = torch.tensor(u, device=cuda), torch.tensor(du, device=cuda)
    f.linearize(0.0, ut)  # with the old parameters
    rng = np.random.default_rng(11 + 7)
    pe = np.tile(np.asarray(PARAMS[mat], dtype=np.float64), (m.ne, 1))
    pe[:, -1] *= np.exp(0.5 * rng.standard_normal(m.ne))
    f.set_parameters(pe, per_element=True)
    r = f.residual(0.0, ut)
    assert torch.equal(r, fresh.residual(0.0, ut))
    assert rel(r.cpu().numpy(), orc.residual(u)) <= TOL64
    _, g = f(0.0, sg.differentiate_wrt(ut))
    _, g0 = fresh(0.0, sg.differentiate_wrt(ut))
    assert torch.equal(g(dut), g0(dut))
