"""serac's functional_comparisons.cpp checks Functional against hand-assembled
mass / diffusion / load integrators at 1e-14.  mfem is absent here, so the
comparison is restated analytically: on an unperturbed box every element is
the same axis-aligned brick, its diffusion stiffness is the Kronecker sum
k (Kx (x) My (x) Mz + Mx (x) Ky (x) Mz + Mx (x) My (x) Kz) of 1-D matrices built
from the same Gauss-Legendre points and Gauss-Lobatto basis, and the source
load is -f (Mx (x) My (x) Mz) 1.  The oracle's heat material (pinned against
the reference kernels) must reproduce both, element by element and assembled."""
import numpy as np
import pytest

from oracle import oracle as O
from tests.problems import rel


def _one_d(p, h):
    B, G = O.basis_1d(p)
    _, w = np.polynomial.legendre.leggauss(p + 1)
    w = 0.5 * w
    M = (B * (w * h)[:, None]).T @ B
    K = (G * (w / h)[:, None]).T @ G
    return M, K


@pytest.mark.parametrize("p", [1, 2])
def test_heat_matches_kronecker_integrators(p):
    nx, ny, nz = 3, 2, 4
    m = O.StructuredHexMesh(nx, ny, nz, O.box_vertices(nx, ny, nz, perturb=0.0))
    k, f = 1.7, 2.1
    hx, hy, hz = 1.0 / nx, 1.0 / ny, 1.0 / nz
    Mx, Kx = _one_d(p, hx)
    My, Ky = _one_d(p, hy)
    Mz, Kz = _one_d(p, hz)
    Ke = k * (np.kron(Mz, np.kron(My, Kx)) + np.kron(Mz, np.kron(Ky, Mx)) + np.kron(Kz, np.kron(My, Mx)))
    Me = np.kron(Mz, np.kron(My, Mx))

    orc = O.OracleFunctional(m, p, 1)
    orc.add_domain_integral(O.MAT_HEAT, [k, f])
    rng = np.random.default_rng(0)
    u = rng.standard_normal(orc.ndofs)
    # element matrices
    uE = O.gather(u, orc.conn, 1, orc.nnodes)
    K = O.element_kernel(O.MAT_HEAT, p, 2, uE, orc.Xq, orc.Jq, [k, f])
    for e in (0, m.ne // 2, m.ne - 1):
        assert np.abs(K[e] - Ke).max() <= 1e-13 * np.abs(Ke).max()
    # assembled residual R = K u - f M 1 and the assembled matrix
    Kg = np.zeros((orc.ndofs, orc.ndofs))
    load = np.zeros(orc.ndofs)
    for e in range(m.ne):
        idx = orc.conn[e]
        Kg[np.ix_(idx, idx)] += Ke
        load[idx] += Me.sum(axis=1)
    assert rel(orc.residual(u), Kg @ u - f * load) <= 1e-13
    assert rel(orc.assemble(u).toarray(), Kg) <= 1e-13
    # Jacobian action of the linear form is the matrix (check_gradient.hpp semantics)
    du = rng.standard_normal(orc.ndofs)
    assert rel(orc.jvp(u, du), Kg @ du) <= 1e-13


@pytest.mark.parametrize("p", [1, 2])
@pytest.mark.parametrize("mat", [O.MAT_HEAT, O.MAT_NEOHOOKEAN])
def test_patch_test_perturbed_mesh(p, mat):
    """Patch tests (solid_statics_patch.cpp, thermal_statics_patch.cpp) on a
    perturbed mesh: a field affine in X is reproduced exactly by the trilinear
    geometry and the H1 basis, its gradient is uniform, so the residual of a
    source-free material vanishes at every interior node."""
    m = O.StructuredHexMesh(3, 3, 3, O.box_vertices(3, 3, 3, perturb=0.25, seed=4))
    c = O.COMPONENTS[mat]
    f = O.OracleFunctional(m, p, c)
    f.add_domain_integral(mat, [1.3, 0.0] if mat == O.MAT_HEAT else [5.0, 0.25])
    X = m.node_coordinates(p)
    G = np.array([[0.01, 0.02, -0.01], [0.0, -0.015, 0.01], [0.005, 0.0, 0.02]])[:c]
    u = (X @ G.T + np.array([0.3, -0.2, 0.1])[:c]).T.ravel()
    r = f.residual(u).reshape(c, -1)
    interior = np.setdiff1d(np.arange(f.nnodes), m.boundary_nodes(p, [1, 2, 3, 4, 5, 6]))
    scale = np.abs(r).max()
    assert scale > 1e-6
    assert np.abs(r[:, interior]).max() <= 1e-13 * scale


def _one_d_mixed(p, h):
    """D[i, j] = int phi_i' phi_j over one 1-D element of length h."""
    B, G = O.basis_1d(p)
    _, w = np.polynomial.legendre.leggauss(p + 1)
    w = 0.5 * w
    return (G * w[:, None]).T @ B


@pytest.mark.parametrize("p", [1, 2])
def test_neohookean_tangent_at_rest_is_linear_elasticity(p):
    """The vector half of functional_comparisons.cpp (StressFunctor at
    1e-14): the Neo-Hookean element stiffness at u = 0 equals isotropic
    linear elasticity with lambda = K - 2G/3, mu = G, built on an unperturbed
    box from the 1-D integrals of phi phi, phi' phi' and phi' phi."""
    nx, ny, nz = 2, 3, 2
    m = O.StructuredHexMesh(nx, ny, nz, O.box_vertices(nx, ny, nz, perturb=0.0))
    Kb, G = 5.0, 0.25
    lam = Kb - 2.0 * G / 3.0
    hs = (1.0 / nx, 1.0 / ny, 1.0 / nz)
    one = [_one_d(p, h) for h in hs]  # (M, S) per direction
    Dm = [_one_d_mixed(p, h) for h in hs]
    npe = (p + 1) ** 3

    def grad_pair(k, l):
        """int d_k phi_a d_l phi_b (a: test node, b: trial node), lexicographic."""
        f = []
        for d in range(3):
            M, S = one[d]
            if d == k and d == l:
                f.append(S)
            elif d == k:
                f.append(Dm[d])
            elif d == l:
                f.append(Dm[d].T)
            else:
                f.append(M)
        return np.kron(f[2], np.kron(f[1], f[0]))

    Gkl = [[grad_pair(k, l) for l in range(3)] for k in range(3)]
    lap = Gkl[0][0] + Gkl[1][1] + Gkl[2][2]
    A = np.zeros((3 * npe, 3 * npe))  # [test (i, a)][trial (j, b)]
    for i in range(3):
        for j in range(3):
            blk = lam * Gkl[i][j] + G * Gkl[j][i] + (G * lap if i == j else 0.0)
            A[i * npe:(i + 1) * npe, j * npe:(j + 1) * npe] = blk
    orc = O.OracleFunctional(m, p, 3)
    orc.add_domain_integral(O.MAT_NEOHOOKEAN, [Kb, G])
    uE = np.zeros((m.ne, 3 * npe))
    K = O.element_kernel(O.MAT_NEOHOOKEAN, p, 2, uE, orc.Xq, orc.Jq, [Kb, G])
    for e in range(m.ne):
        assert np.abs(K[e].T - A).max() <= 1e-13 * np.abs(A).max()
