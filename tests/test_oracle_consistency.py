"""Operator-level checks of the CPU oracle that need no reference golden.

The reference pins no vmult vector, no 3D case and no degree above 1 (solid)
or 2 (heat), so the oracle's matrix-free operators are checked two more ways,
at every degree 1-6 (the assembled operators also in 2D):

* tangent consistency: the central finite difference of the oracle's
  residual (mf_elasticity.h:1649-1908, internal force + inertia) along v
  equals minus the tangent vmult (mf_nh_operator.h:545-625) for every
  caching variant, within 1e-7 relative;
* an assembled operator: element matrices integrated here in numpy with the
  full (non-sum-factorized) Q_p basis on QGauss(p+1) and the closed-form
  derivative of P = mu F - (mu - 2 lambda ln J) F^{-T}
  (material.h:116-161), assembled densely with identity rows and zero
  columns for the Dirichlet DoFs, give the same A x as the oracle's
  matrix-free vmult within 1e-12; likewise the heat operator M + k dt K
  (heat_transfer.h:236-250).
"""
import numpy as np
import pytest

import oracle as O
import workloads as W


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


# --- numpy reference element (independent of the oracle's kernels) --------

def lagrange_1d(nodes, x):
    """Values and derivatives of the Lagrange basis on `nodes` at points x."""
    n = len(nodes)
    V = np.ones((n, len(x)))
    dV = np.zeros((n, len(x)))
    for i in range(n):
        others = [j for j in range(n) if j != i]
        for j in others:
            V[i] *= (x - nodes[j]) / (nodes[i] - nodes[j])
        for k in others:
            term = np.ones(len(x)) / (nodes[i] - nodes[k])
            for j in others:
                if j != k:
                    term = term * (x - nodes[j]) / (nodes[i] - nodes[j])
            dV[i] += term
    return V, dV


def element_basis(p, h):
    """phi[q, a] and physical grad[q, a, d] on the reference cell (lexicographic
    local nodes, x fastest) at the tensor Gauss points; JxW[q]."""
    nodes = W.gauss_lobatto(p)
    xg, wg = np.polynomial.legendre.leggauss(p + 1)
    xg, wg = (xg + 1) / 2, wg / 2
    V, dV = lagrange_1d(nodes, xg)
    N, Q = p + 1, p + 1
    phi = np.einsum("aq,br,cs->qrsabc", V, V, V).reshape(Q ** 3, N ** 3)
    gx = np.einsum("aq,br,cs->qrsabc", dV, V, V).reshape(Q ** 3, N ** 3) / h[0]
    gy = np.einsum("aq,br,cs->qrsabc", V, dV, V).reshape(Q ** 3, N ** 3) / h[1]
    gz = np.einsum("aq,br,cs->qrsabc", V, V, dV).reshape(Q ** 3, N ** 3) / h[2]
    # the einsum orders (qz, qy, qx) slowest to fastest when reshaping with
    # (q, r, s) = (x, y, z) first: reorder to x fastest for both q and a
    def to_lex(t):
        t = t.reshape(Q, Q, Q, N, N, N)            # qx, qy, qz, a, b, c
        t = t.transpose(2, 1, 0, 5, 4, 3)          # qz, qy, qx, c, b, a
        return t.reshape(Q ** 3, N ** 3)
    phi, gx, gy, gz = map(to_lex, (phi, gx, gy, gz))
    w = np.einsum("i,j,k->kji", wg, wg, wg).reshape(-1) * h[0] * h[1] * h[2]
    return phi, np.stack([gx, gy, gz], axis=2), w


def mesh_geometry(spec):
    p = spec["degree"]
    C = [spec["rep"][d] << spec["n_ref"] for d in range(3)]
    Nn = [C[d] * p + 1 for d in range(3)]
    h = [(spec["hi"][d] - spec["lo"][d]) / C[d] for d in range(3)]
    return p, C, Nn, h


def cell_nodes(p, C, Nn, cx, cy, cz):
    a = np.arange(p + 1)
    ix = cx * p + a[None, None, :]
    iy = cy * p + a[None, :, None]
    iz = cz * p + a[:, None, None]
    return (ix + Nn[0] * (iy + Nn[1] * iz)).reshape(-1)


def constrained_nodes(spec, Nn, comp):
    """Nodes constrained in component `comp` (face bitmask semantics)."""
    X = np.arange(Nn[0])[None, None, :] + 0 * np.zeros((Nn[2], Nn[1], 1), int)
    Y = np.arange(Nn[1])[None, :, None] + 0 * np.zeros((Nn[2], 1, Nn[0]), int)
    Z = np.arange(Nn[2])[:, None, None] + 0 * np.zeros((1, Nn[1], Nn[0]), int)
    faces = [X == 0, X == Nn[0] - 1, Y == 0, Y == Nn[1] - 1, Z == 0, Z == Nn[2] - 1]
    mask = np.zeros((Nn[2], Nn[1], Nn[0]), bool)
    for f in range(6):
        for bid, cmask in spec["dirichlet"]:
            if spec["boundary_id"][f] == bid and (cmask >> comp) & 1:
                mask |= faces[f]
    return np.nonzero(mask.reshape(-1))[0]


def apply_constraints(K, spec, Nn, nc):
    n_nodes = Nn[0] * Nn[1] * Nn[2]
    cons = np.concatenate([c * n_nodes + constrained_nodes(spec, Nn, c) for c in range(nc)])
    K[cons, :] = 0.0
    K[:, cons] = 0.0
    K[cons, cons] = 1.0
    return K


def assembled_heat(spec, kdt):
    p, C, Nn, h = mesh_geometry(spec)
    phi, grad, w = element_basis(p, h)
    Ke = np.einsum("q,qa,qb->ab", w, phi, phi) + kdt * np.einsum("q,qad,qbd->ab", w, grad, grad)
    n = Nn[0] * Nn[1] * Nn[2]
    K = np.zeros((n, n))
    for cz in range(C[2]):
        for cy in range(C[1]):
            for cx in range(C[0]):
                g = cell_nodes(p, C, Nn, cx, cy, cz)
                K[np.ix_(g, g)] += Ke
    return apply_constraints(K, spec, Nn, 1)


def assembled_nh_tangent(spec, u, mu, nu, rho_alpha):
    """Consistent tangent of P = mu F - (mu - 2 lambda ln J) F^{-T} plus
    rho alpha_1 times the mass matrix."""
    lam = 2 * mu * nu / (1 - 2 * nu)
    p, C, Nn, h = mesh_geometry(spec)
    phi, grad, w = element_basis(p, h)
    n_nodes = Nn[0] * Nn[1] * Nn[2]
    nd = p + 1
    K = np.zeros((3 * n_nodes, 3 * n_nodes))
    U = u.reshape(3, n_nodes)
    M_e = np.einsum("q,qa,qb->ab", w, phi, phi)
    I3 = np.eye(3)
    for cz in range(C[2]):
        for cy in range(C[1]):
            for cx in range(C[0]):
                g = cell_nodes(p, C, Nn, cx, cy, cz)
                ue = U[:, g]                                   # (3, nd^3)
                F = I3[None] + np.einsum("ia,qaJ->qiJ", ue, grad)
                Finv = np.linalg.inv(F)
                FiT = np.transpose(Finv, (0, 2, 1))
                lnJ = np.log(np.linalg.det(F))
                c = 2 * lam * lnJ - mu
                A = (mu * np.einsum("ik,JL->iJkL", I3, I3)[None]
                     + 2 * lam * np.einsum("qkL,qiJ->qiJkL", FiT, FiT)
                     - c[:, None, None, None, None] * np.einsum("qiL,qkJ->qiJkL", FiT, FiT))
                # Ke[i,a,k,b] = sum_q w_q grad[q,a,J] A[q,i,J,k,L] grad[q,b,L],
                # contracted as two matrix products
                nq, nb = grad.shape[0], grad.shape[1]
                AG = np.matmul(A.reshape(nq, 27, 3), np.transpose(grad, (0, 2, 1)))   # (q, iJk, b)
                AG = AG.reshape(nq, 3, 3, 3, nb).transpose(0, 2, 1, 3, 4).reshape(nq * 3, 9 * nb)
                WG = (w[:, None, None] * grad).transpose(1, 0, 2).reshape(nb, nq * 3)
                Ke = (WG @ AG).reshape(nb, 3, 3, nb).transpose(1, 0, 2, 3).reshape(3 * nd ** 3, 3 * nd ** 3)
                Ke += rho_alpha * np.kron(I3, M_e)
                dofs = np.concatenate([ci * n_nodes + g for ci in range(3)])
                K[np.ix_(dofs, dofs)] += Ke
    return apply_constraints(K, spec, Nn, 3)


# --- the checks -------------------------------------------------------------

ANISO = dict(rep=(2, 1, 1), length=(3.0, 1.0, 0.7))


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
def test_heat_oracle_matches_assembled(degree):
    spec = W.unit_cube_heat(degree, 0, rep=(2, 1, 1))
    spec["hi"] = (1.0, 0.6, 0.45)
    om = W.to_oracle_mesh(O, spec)
    K = assembled_heat(spec, 0.1)
    x = W.uniform_vector(K.shape[0], 11)
    assert rel(O.heat_vmult(om, 0, 0.1, x), K @ x) < 1e-12


_ASSEMBLED = {}


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("caching", ["scalar_referential", "tensor2", "tensor4", "tensor4_ns"])
def test_nh_oracle_matches_assembled_tangent(degree, caching):
    spec = W.cantilever(degree, 0, **ANISO)
    u = W.smooth_displacement(degree, 0, spec["rep"], spec["lo"], spec["hi"], seed=3)
    om = W.to_oracle_mesh(O, spec)
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    if degree not in _ASSEMBLED:  # one assembly per degree, shared by the caching variants
        _ASSEMBLED[degree] = assembled_nh_tangent(spec, u, 0.5e6, 0.4, 1000.0 * mat.alpha_1)
    K = _ASSEMBLED[degree]
    x = W.uniform_vector(K.shape[0], 12)
    assert rel(O.nh_vmult(om, 0, mat, caching, u, x), K @ x) < 1e-12, caching


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("caching", ["scalar_referential", "tensor2", "tensor4", "tensor4_ns"])
def test_nh_tangent_is_derivative_of_residual(degree, caching):
    spec = W.cantilever(degree, 0, **ANISO)
    u = W.smooth_displacement(degree, 0, spec["rep"], spec["lo"], spec["hi"], seed=4)
    om = W.to_oracle_mesh(O, spec)
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    n = len(u)
    v = W.uniform_vector(n, 13)
    # zero the Dirichlet DoFs of the direction (the tangent's constrained rows
    # are the identity, the residual's are zero)
    probe = O.nh_residual(om, 0, mat, np.ones(n) * 0.0, np.ones(n))
    free = probe != 0.0
    v[~free] = 0.0
    eps = 1e-6
    rp = O.nh_residual(om, 0, mat, u + eps * v, mat.alpha_1 * (u + eps * v))
    rm = O.nh_residual(om, 0, mat, u - eps * v, mat.alpha_1 * (u - eps * v))
    fd = (rp - rm) / (2 * eps)
    Av = O.nh_vmult(om, 0, mat, caching, u, v)
    assert rel(-fd[free], Av[free]) < 1e-7, caching


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
def test_formulation0_tangent_is_derivative_of_residual(degree):
    """Formulation 0 (isochoric/volumetric split, tensor2 caching only,
    mf_nh_operator.h:701-840): its tangent is the derivative of its residual
    (mf_elasticity.h:1649-1908) within 1e-7 relative."""
    spec = W.cantilever(degree, 0, **ANISO)
    u = W.smooth_displacement(degree, 0, spec["rep"], spec["lo"], spec["hi"], seed=5)
    om = W.to_oracle_mesh(O, spec)
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01, formulation=0)
    n = len(u)
    v = W.uniform_vector(n, 14)
    probe = O.nh_residual(om, 0, mat, np.zeros(n), np.ones(n))
    free = probe != 0.0
    v[~free] = 0.0
    eps = 1e-6
    rp = O.nh_residual(om, 0, mat, u + eps * v, mat.alpha_1 * (u + eps * v))
    rm = O.nh_residual(om, 0, mat, u - eps * v, mat.alpha_1 * (u - eps * v))
    fd = (rp - rm) / (2 * eps)
    Av = O.nh_vmult(om, 0, mat, "tensor2", u, v)
    assert rel(-fd[free], Av[free]) < 1e-7
    # and it is a different operator from formulation 1 on the same state
    Av1 = O.nh_vmult(om, 0, O.material(0.5e6, 0.4, 1000.0, 0.01), "tensor2", u, v)
    assert rel(Av1, Av) > 1e-6


# --- two dimensions (the reference's own test cases are 2D) -----------------

def element_basis_2d(p, h):
    nodes = W.gauss_lobatto(p)
    xg, wg = np.polynomial.legendre.leggauss(p + 1)
    xg, wg = (xg + 1) / 2, wg / 2
    V, dV = lagrange_1d(nodes, xg)
    N = p + 1
    # index order: (qy, qx) slowest to fastest, (ay, ax) likewise
    phi = np.einsum("aq,br->rqba", V, V).reshape(N * N, N * N)
    gx = np.einsum("aq,br->rqba", dV, V).reshape(N * N, N * N) / h[0]
    gy = np.einsum("aq,br->rqba", V, dV).reshape(N * N, N * N) / h[1]
    w = np.einsum("i,j->ji", wg, wg).reshape(-1) * h[0] * h[1]
    return phi, np.stack([gx, gy], axis=2), w


SPEC2 = dict(rep=(2, 1), lo=(0.0, 0.0), hi=(1.5, 0.6), bid=(1, 0, 0, 0))


def mesh2d(degree, nc):
    C = SPEC2["rep"]
    Nn = [C[0] * degree + 1, C[1] * degree + 1]
    h = [(SPEC2["hi"][d] - SPEC2["lo"][d]) / C[d] for d in range(2)]
    om = O.make_mesh(2, degree, degree + 1, 0, SPEC2["rep"], SPEC2["lo"], SPEC2["hi"],
                     boundary_id=SPEC2["bid"], dirichlet=[(1, (1 << nc) - 1)])
    return om, C, Nn, h


def assemble_2d(degree, nc, Ke, C, Nn):
    n_nodes = Nn[0] * Nn[1]
    K = np.zeros((nc * n_nodes, nc * n_nodes))
    a = np.arange(degree + 1)
    for cy in range(C[1]):
        for cx in range(C[0]):
            g = ((cx * degree + a[None, :]) + Nn[0] * (cy * degree + a[:, None])).reshape(-1)
            dofs = np.concatenate([ci * n_nodes + g for ci in range(nc)])
            K[np.ix_(dofs, dofs)] += Ke(g)
    # boundary id 1 is the face x = 0, constrained in every component
    left = np.arange(Nn[1]) * Nn[0]
    cons = np.concatenate([ci * n_nodes + left for ci in range(nc)])
    K[cons, :] = 0.0
    K[:, cons] = 0.0
    K[cons, cons] = 1.0
    return K


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
def test_heat_oracle_matches_assembled_2d(degree):
    om, C, Nn, h = mesh2d(degree, 1)
    phi, grad, w = element_basis_2d(degree, h)
    Ke = np.einsum("q,qa,qb->ab", w, phi, phi) + 0.1 * np.einsum("q,qad,qbd->ab", w, grad, grad)
    K = assemble_2d(degree, 1, lambda g: Ke, C, Nn)
    x = W.uniform_vector(K.shape[0], 15)
    assert rel(O.heat_vmult(om, 0, 0.1, x), K @ x) < 1e-12


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("caching", ["scalar_referential", "tensor2", "tensor4", "tensor4_ns"])
def test_nh_oracle_matches_assembled_tangent_2d(degree, caching):
    """Plane (dim = 2) neo-Hookean tangent: F is 2 x 2, J = det F."""
    om, C, Nn, h = mesh2d(degree, 2)
    mu, nu = 0.5e6, 0.4
    lam = 2 * mu * nu / (1 - 2 * nu)
    mat = O.material(mu, nu, 1000.0, 0.01)
    phi, grad, w = element_basis_2d(degree, h)
    n_nodes = Nn[0] * Nn[1]
    xs = W.axis_coords(C[0], SPEC2["lo"][0], SPEC2["hi"][0], degree)
    ys = W.axis_coords(C[1], SPEC2["lo"][1], SPEC2["hi"][1], degree)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    u = np.concatenate([0.03 * np.sin(2.1 * X + 0.4) * np.cos(1.3 * Y),
                        0.02 * np.cos(1.7 * X - 0.2 * Y + 0.9)]).reshape(-1)
    U = u.reshape(2, n_nodes)
    M_e = np.einsum("q,qa,qb->ab", w, phi, phi)
    I2 = np.eye(2)
    nb = grad.shape[1]

    def Ke(g):
        F = I2[None] + np.einsum("ia,qaJ->qiJ", U[:, g], grad)
        FiT = np.transpose(np.linalg.inv(F), (0, 2, 1))
        c = 2 * lam * np.log(np.linalg.det(F)) - mu
        A = (mu * np.einsum("ik,JL->iJkL", I2, I2)[None]
             + 2 * lam * np.einsum("qkL,qiJ->qiJkL", FiT, FiT)
             - c[:, None, None, None, None] * np.einsum("qiL,qkJ->qiJkL", FiT, FiT))
        k = np.einsum("q,qaJ,qiJkL,qbL->iakb", w, grad, A, grad, optimize=True).reshape(2 * nb, 2 * nb)
        return k + 1000.0 * mat.alpha_1 * np.kron(I2, M_e)

    K = assemble_2d(degree, 2, Ke, C, Nn)
    x = W.uniform_vector(K.shape[0], 16)
    assert rel(O.nh_vmult(om, 0, mat, caching, u, x), K @ x) < 1e-12, caching


# --- diagonal and level transfer --------------------------------------------

@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
def test_inverse_diagonals_match_assembled(degree):
    """compute_diagonal (heat_transfer.h:205-230, mf_nh_operator.h:1025-1060):
    the oracle's inverse diagonal is 1 / diag of the assembled operator, with
    1 on the constrained rows."""
    spec = W.unit_cube_heat(degree, 0, rep=(2, 1, 1))
    spec["hi"] = (1.0, 0.6, 0.45)
    K = assembled_heat(spec, 0.1)
    got = O.heat_inv_diagonal(W.to_oracle_mesh(O, spec), 0, 0.1)
    assert rel(got, 1.0 / np.diag(K)) < 1e-13
    if degree <= 4:
        spec = W.cantilever(degree, 0, **ANISO)
        u = W.smooth_displacement(degree, 0, spec["rep"], spec["lo"], spec["hi"], seed=3)
        mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
        K = assembled_nh_tangent(spec, u, 0.5e6, 0.4, 1000.0 * mat.alpha_1)
        got = O.nh_inv_diagonal(W.to_oracle_mesh(O, spec), 0, mat, "tensor4", u)
        assert rel(got, 1.0 / np.diag(K)) < 1e-12


def _box(degree, dirichlet):
    return dict(degree=degree, n_ref=1, rep=(2, 1, 1), lo=(0.0, -0.5, 0.2), hi=(1.4, 0.5, 0.9),
                boundary_id=(1, 0, 0, 0, 0, 0), dirichlet=dirichlet)


def _qp_poly(degree, seed):
    """A random tensor-product polynomial of degree `degree` in each variable
    (an element of Q_p, so FE_Q on either level represents it exactly)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    cs = [rng.uniform(-1, 1, degree + 1) for _ in range(3)]
    return lambda X, Y, Z: (np.polyval(cs[0], X) * np.polyval(cs[1], Y) * np.polyval(cs[2], Z))


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
def test_transfer_reproduces_qp_and_restriction_is_transpose(degree):
    """MGTransferMatrixFree for continuous elements (used at
    mf_elasticity.h:865-929, heat_transfer.h:515-573): prolongation and
    interpolation to the coarse level are exact on Q_p; restriction is the
    transpose of prolongation on the unconstrained DoFs."""
    spec = _box(degree, [])
    om = W.to_oracle_mesh(O, spec)
    f = _qp_poly(degree, 21)
    Xc = W.node_coords(degree, 0, spec["rep"], spec["lo"], spec["hi"])
    Xf = W.node_coords(degree, 1, spec["rep"], spec["lo"], spec["hi"])
    coarse = f(*Xc)
    fine = np.zeros(len(Xf[0]))
    O.transfer(om, 0, 1, "prolongate", coarse, fine)
    assert rel(fine, f(*Xf)) < 1e-12
    back = np.zeros_like(coarse)
    O.transfer(om, 0, 1, "interpolate", back, f(*Xf))
    assert rel(back, coarse) < 1e-12

    # transpose, with a Dirichlet face and three components
    spec = _box(degree, [(1, 0b101)])
    om = W.to_oracle_mesh(O, spec)
    nc_, nf_ = 3 * len(Xc[0]), 3 * len(Xf[0])
    c = W.uniform_vector(nc_, 22)
    g = W.uniform_vector(nf_, 23)
    Pc = np.zeros(nf_)
    O.transfer(om, 0, 3, "prolongate", c, Pc)
    Rg = np.zeros(nc_)
    O.transfer(om, 0, 3, "restrict", Rg, g)
    # constrained entries: P reads them as zero and writes zero, R skips them
    free_c = Rg != 0.0
    lhs = float(Pc @ g)
    rhs = float(c[free_c] @ Rg[free_c])
    assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + np.linalg.norm(Pc) * np.linalg.norm(g))
    assert (~free_c).sum() == 2 * (spec["rep"][1] * degree + 1) * (spec["rep"][2] * degree + 1)
