"""Size-independent properties at the configurations' full sizes, alongside
the direct comparisons with the oracle at those sizes in
tests/test_gpu_configs.py: the Neo-Hookean 32^3 Q2 problem (823,875 DOF) and
the heterogeneous 64^3 Q2 problem (6,440,067 DOF).

* the assembled CSR matrix applied to a vector equals the Jacobian action;
* the hyperelastic tangent is symmetric: w . J v = v . J w;
* the Jacobian action is linear and bitwise reproducible;
* the FP32 action agrees with the FP64 one to 1e-5;
* patch test: an affine displacement gives a uniform stress, so the residual
  vanishes at interior nodes (relative to the boundary reactions)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _c2():
    import serac_gb300 as sg
    from oracle.oracle import box_vertices

    n = 32
    mesh = sg.Mesh.structured_hex(n, n, n, box_vertices(n, n, n, 0.1, 1))
    f = sg.Functional(mesh, sg.H1(2, 3))
    f.AddDomainIntegral(sg.NEOHOOKEAN, [5.0, 0.25])
    return mesh, f


def _state(mesh, f, seed=2):
    X = mesh.node_coordinates(2)
    u = np.zeros((3, X.shape[0]))
    u[2] = -0.005 * X[:, 2]
    u += 1e-4 * np.random.default_rng(seed).standard_normal(u.shape)
    return torch.tensor(u.ravel(), device="cuda")


def _rel(a, b):
    return float(torch.linalg.norm(a - b) / torch.linalg.norm(b))


def test_c2_csr_times_vector_equals_jacobian_action(cuda):
    import serac_gb300 as sg

    mesh, f = _c2()
    u = _state(mesh, f)
    _, J = f(0.0, sg.differentiate_wrt(u))
    v = torch.randn(f.ndofs, dtype=torch.float64, device=cuda)
    jv = J(v).clone()
    row_ptr, col, val = sg.assemble(J)
    assert int(row_ptr[-1]) == val.numel() == 152_771_337  # 9 * 257^3, the C2 nnz
    A = torch.sparse_csr_tensor(row_ptr, col.to(torch.int64), val, size=(f.ndofs, f.ndofs))
    av = (A @ v.unsqueeze(1)).squeeze(1)
    assert _rel(av, jv) <= 1e-12


def test_c2_tangent_symmetric_linear_reproducible(cuda):
    import serac_gb300 as sg

    mesh, f = _c2()
    u = _state(mesh, f)
    _, J = f(0.0, sg.differentiate_wrt(u))
    g = torch.Generator(device="cuda").manual_seed(3)
    v = torch.randn(f.ndofs, dtype=torch.float64, device=cuda, generator=g)
    w = torch.randn(f.ndofs, dtype=torch.float64, device=cuda, generator=g)
    jv, jw = J(v).clone(), J(w).clone()
    a, b = float(w @ jv), float(v @ jw)
    assert abs(a - b) <= 1e-12 * float(torch.linalg.norm(w) * torch.linalg.norm(jv))
    lin = J(2.0 * v - 3.0 * w).clone()
    assert _rel(lin, 2.0 * jv - 3.0 * jw) <= 1e-13
    assert torch.equal(J(v), jv)
    jv32 = J(v.float()).double()
    assert _rel(jv32, jv) <= 1e-5


def test_c2_patch_test_affine_displacement(cuda):
    mesh, f = _c2()
    X = torch.tensor(mesh.node_coordinates(2).T.copy(), device=cuda)  # (3, N)
    A = torch.tensor([[0.010, -0.004, 0.002], [0.003, 0.008, -0.001], [-0.002, 0.005, -0.012]],
                     dtype=torch.float64, device=cuda)
    u = (A @ X).reshape(-1).contiguous()
    r = f.residual(0.0, u).reshape(3, -1)
    b = mesh.boundary_nodes(2, [1, 2, 3, 4, 5, 6])
    interior = torch.ones(f.num_nodes, dtype=torch.bool, device=cuda)
    interior[torch.as_tensor(b, device=cuda)] = False
    assert float(r[:, interior].abs().max()) <= 1e-12 * float(r[:, ~interior].abs().max())


def test_c3_64cubed_heterogeneous_action_properties(cuda):
    """The 64^3 heterogeneous Neo-Hookean problem (per-element shear modulus
    0.25 exp(g), bulk modulus 20 G): symmetry, FP32 vs FP64, reproducibility."""
    import serac_gb300 as sg
    from serac_gb300 import learned as LP

    prob = LP.neohookean_problem(64, 2, sigma_log=1.0, ell=0.1, strain=0.05, steps=10, bulk_ratio=20.0)
    S = LP.SolidSetup(prob, 2)
    u = torch.zeros(S.f.ndofs, dtype=torch.float64, device=cuda)
    S.load(u, 1)
    _, J = S.f(0.0, sg.differentiate_wrt(u))
    g = torch.Generator(device="cuda").manual_seed(5)
    v = torch.randn(S.f.ndofs, dtype=torch.float64, device=cuda, generator=g)
    w = torch.randn(S.f.ndofs, dtype=torch.float64, device=cuda, generator=g)
    jv, jw = J(v).clone(), J(w).clone()
    assert abs(float(w @ jv) - float(v @ jw)) <= 1e-12 * float(torch.linalg.norm(w) * torch.linalg.norm(jv))
    assert torch.equal(J(v), jv)
    assert _rel(J(v.float()).double(), jv) <= 1e-5
