"""The algebra behind the heat operator's tensor-product kernels
(csrc/mf_heat_tp.cu), checked in numpy on the CPU:

* the element operator of mass + dt k Laplace on an affine brick, assembled
  with the (p+1)-point Gauss rule through the Gauss points (what
  LaplaceOperator::do_operation_on_cell integrates, heat_transfer.h:236-250),
  equals vol [Mz(x)My(x)(Mx + c0 Kx) + c1 Mz(x)Ky(x)Mx + c2 Kz(x)My(x)Mx] with the
  1D mass and stiffness matrices of the Gauss-Lobatto basis, for degrees 1-6
  and anisotropic cells;
* the grouping the kernels apply (x-sweeps P, Q; y-sweeps; z-sweeps, 7 of
  them per cell) gives the same product on random cell vectors;
* the even-odd form of the 1D matrices (sums and differences of mirrored
  entries) reproduces their products, which needs the matrices to be
  centro-symmetric.
"""
import numpy as np
import pytest


def lobatto(p):
    if p == 1:
        return np.array([0.0, 1.0])
    c = np.zeros(p + 1)
    c[-1] = 1.0
    inner = np.sort(np.real(np.polynomial.legendre.legroots(np.polynomial.legendre.legder(c))))
    return np.concatenate([[0.0], (inner + 1) / 2, [1.0]])


def basis(p):
    """Values and derivatives of the Lagrange basis on the Gauss-Lobatto
    nodes at the (p+1) Gauss points of [0,1], and the weights."""
    nodes = lobatto(p)
    xg, wg = np.polynomial.legendre.leggauss(p + 1)
    xq, w = (xg + 1) / 2, wg / 2
    n = p + 1
    S = np.zeros((n, n))
    G = np.zeros((n, n))
    for i in range(n):
        others = [j for j in range(n) if j != i]
        for q, x in enumerate(xq):
            S[q, i] = np.prod([(x - nodes[j]) / (nodes[i] - nodes[j]) for j in others])
            d = 0.0
            for m in others:
                d += np.prod([(x - nodes[j]) / (nodes[i] - nodes[j]) for j in others if j != m]) / (
                    nodes[i] - nodes[m])
            G[q, i] = d
    return S, G, w


def kron3(Az, Ay, Ax):
    # lexicographic cell numbering, x fastest: index = a + n b + n^2 k
    return np.kron(Az, np.kron(Ay, Ax))


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_tensor_product_equals_quadrature_element_matrix(p):
    S, G, w = basis(p)
    h = np.array([0.7, 1.3, 0.45])
    kdt = 0.37
    vol = h.prod()
    # quadrature through the Gauss points: sum_q w_q (phi_i phi_j + kdt grad phi_i . grad phi_j) vol
    Sq = kron3(S, S, S)                        # [q][i] values
    Gx = kron3(S, S, G) / h[0]                 # x-derivative
    Gy = kron3(S, G, S) / h[1]
    Gz = kron3(G, S, S) / h[2]
    Wq = kron3(np.diag(w), np.diag(w), np.diag(w)).diagonal() * vol
    A_quad = Sq.T @ (Wq[:, None] * Sq) + kdt * sum(D.T @ (Wq[:, None] * D) for D in (Gx, Gy, Gz))
    # tensor-product form
    M = S.T @ (w[:, None] * S)
    K = G.T @ (w[:, None] * G)
    A_tp = vol * (kron3(M, M, M + kdt / h[0] ** 2 * K) + kdt / h[1] ** 2 * kron3(M, K, M) +
                  kdt / h[2] ** 2 * kron3(K, M, M))
    assert np.abs(A_tp - A_quad).max() <= 1e-12 * np.abs(A_quad).max()
    # the kernels' grouping: 2 x-sweeps, 3 y-sweeps, 2 z-sweeps
    n = p + 1
    rng = np.random.default_rng(p)
    x = rng.uniform(-1, 1, (n, n, n))          # [k][b][a]
    Mx, Ax = M, vol * M + vol * kdt / h[0] ** 2 * K
    My, Ky = M, vol * kdt / h[1] ** 2 * K
    Mz, Kz = M, vol * kdt / h[2] ** 2 * K
    P = np.einsum("ia,kba->kbi", Mx, x)
    Q = np.einsum("ia,kba->kbi", Ax, x)
    S1 = np.einsum("ib,kba->kia", My, Q) + np.einsum("ib,kba->kia", Ky, P)
    S2 = np.einsum("ib,kba->kia", My, P)
    y = np.einsum("ik,kba->iba", Mz, S1) + np.einsum("ik,kba->iba", Kz, S2)
    assert np.allclose(y.reshape(-1), A_quad @ x.reshape(-1), rtol=1e-12, atol=1e-12 * np.abs(y).max())


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_even_odd_form_of_the_1d_matrices(p):
    S, G, w = basis(p)
    n, H = p + 1, (p + 1) // 2
    for A in (S.T @ (w[:, None] * S), G.T @ (w[:, None] * G)):
        # symmetric and centro-symmetric
        assert np.allclose(A, A.T, atol=1e-13)
        assert np.allclose(A, A[::-1, ::-1], atol=1e-13)
        E = (A[:H, :H] + A[:H, ::-1][:, :H]) / 2
        O = (A[:H, :H] - A[:H, ::-1][:, :H]) / 2
        v = np.random.default_rng(7).uniform(-1, 1, n)
        e = v[:H] + v[::-1][:H]
        o = v[:H] - v[::-1][:H]
        y = np.zeros(n)
        se = E @ e + (A[:H, H] * v[H] if n % 2 else 0)
        so = O @ o
        y[:H] = se + so
        y[n - H:] = (se - so)[::-1]
        if n % 2:
            y[H] = A[H, :H] @ e + A[H, H] * v[H]
        assert np.allclose(y, A @ v, rtol=1e-12, atol=1e-13)
