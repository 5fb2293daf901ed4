"""The even-odd form of the 1D shape matrices used by the cell kernels'
sweeps (EO in csrc/mf_common.cuh, mat_apply / eo_apply_t in
csrc/mf_cell.cuh), restated in numpy: the same coefficient arrays and the
same recombination, checked against the full products M x and M^T x for
the interpolation matrix S (Gauss-Lobatto nodes -> Gauss points,
centro-symmetric) and the collocation derivative D on the Gauss points
(skew-centro-symmetric), degrees 1-6.  CPU only."""
import numpy as np
import pytest


def lobatto_nodes(p):
    """Gauss-Lobatto points on [0,1] for degree p (p+1 points)."""
    if p == 1:
        return np.array([0.0, 1.0])
    inner = np.real(np.polynomial.legendre.Legendre.basis(p).deriv().roots())
    return np.concatenate([[0.0], np.sort((inner + 1) / 2), [1.0]])


def lagrange_matrix(nodes, x):
    """L[q][i] = l_i(x_q) for the Lagrange basis on `nodes`."""
    n = len(nodes)
    L = np.ones((len(x), n))
    for i in range(n):
        for j in range(n):
            if j != i:
                L[:, i] *= (x - nodes[j]) / (nodes[i] - nodes[j])
    return L


def lagrange_derivative(nodes, x):
    n = len(nodes)
    G = np.zeros((len(x), n))
    for i in range(n):
        for m in range(n):
            if m == i:
                continue
            term = np.full(len(x), 1.0 / (nodes[i] - nodes[m]))
            for j in range(n):
                if j != i and j != m:
                    term *= (x - nodes[j]) / (nodes[i] - nodes[j])
            G[:, i] += term
    return G


def shape_matrices(p):
    n = p + 1
    xg, _ = np.polynomial.legendre.leggauss(n)
    xg = (xg + 1) / 2
    S = lagrange_matrix(lobatto_nodes(p), xg)
    D = lagrange_derivative(xg, xg)
    return S, D


def make_eo(M):
    """Coefficients as make_eo (csrc/mf_kernel_util.cuh)."""
    N = M.shape[0]
    H, HR = N // 2, (N + 1) // 2
    e = np.zeros((HR, HR))
    o = np.zeros((HR, H))
    for r in range(HR):
        for k in range(H):
            e[r, k] = 0.5 * (M[r, k] + M[r, N - 1 - k])
            o[r, k] = 0.5 * (M[r, k] - M[r, N - 1 - k])
        if N % 2:
            e[r, H] = M[r, H]
    return e, o


def eo_apply(e, o, sig, x):
    """out = M x (mat_apply on an EO matrix)."""
    N = len(x)
    H, odd = N // 2, N % 2 == 1
    p = [x[k] + x[N - 1 - k] for k in range(H)]
    m = [x[k] - x[N - 1 - k] for k in range(H)]
    out = np.zeros(N)
    for r in range(H):
        E = sum(e[r, k] * p[k] for k in range(H)) + (e[r, H] * x[H] if odd else 0.0)
        O = sum(o[r, k] * m[k] for k in range(H))
        out[r] = E + O
        out[N - 1 - r] = sig * (E - O)
    if odd:
        if sig > 0:
            out[H] = sum(e[H, k] * p[k] for k in range(H)) + e[H, H] * x[H]
        else:
            out[H] = sum(o[H, k] * m[k] for k in range(H))
    return out


def eo_apply_t(e, o, sig, x, out=None):
    """out = M^T x, or out += M^T x when `out` is given (eo_apply_t)."""
    N = len(x)
    H, odd = N // 2, N % 2 == 1
    p = [x[r] + sig * x[N - 1 - r] for r in range(H)]
    m = [x[r] - sig * x[N - 1 - r] for r in range(H)]
    res = np.zeros(N) if out is None else out.copy()
    for k in range(H):
        E = sum(e[r, k] * p[r] for r in range(H))
        O = sum(o[r, k] * m[r] for r in range(H))
        if odd and sig > 0:
            E += e[H, k] * x[H]
        if odd and sig < 0:
            O += o[H, k] * x[H]
        res[k] += E + O
        res[N - 1 - k] += E - O
    if odd:
        c = sum(e[r, H] * p[r] for r in range(H))
        if sig > 0:
            c += e[H, H] * x[H]
        res[H] += c
    return res


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
def test_matrix_symmetries(p):
    S, D = shape_matrices(p)
    assert np.allclose(S[::-1, ::-1], S, atol=1e-14)
    assert np.allclose(D[::-1, ::-1], -D, atol=1e-12)
    # S interpolates (rows sum to 1), D annihilates constants
    assert np.allclose(S.sum(axis=1), 1.0, atol=1e-14)
    assert np.allclose(D.sum(axis=1), 0.0, atol=1e-11)


@pytest.mark.parametrize("p", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("which", ["S", "D"])
def test_even_odd_products(p, which):
    S, D = shape_matrices(p)
    M, sig = (S, 1) if which == "S" else (D / 0.37, -1)
    e, o = make_eo(M)
    rng = np.random.Generator(np.random.PCG64(p))
    for _ in range(5):
        x = rng.uniform(-1, 1, p + 1)
        y = rng.uniform(-1, 1, p + 1)
        scale = np.abs(M).sum() * 1e-15
        assert np.max(np.abs(eo_apply(e, o, sig, x) - M @ x)) < scale
        assert np.max(np.abs(eo_apply_t(e, o, sig, x) - M.T @ x)) < scale
        assert np.max(np.abs(eo_apply_t(e, o, sig, x, y) - (y + M.T @ x))) < scale + 1e-15


@pytest.mark.parametrize("N", [2, 3, 4, 5, 6, 7])
def test_product_counts(N):
    """Products per line: N^2 for the full matrix, against the even-odd
    split's ~N^2/2 + N/2 (13 for N = 5, 25 for N = 7)."""
    H, odd = N // 2, N % 2
    n_eo = H * (H + odd + H) + (odd * (H + 1) if odd else 0)
    assert n_eo <= N * N
    if N == 5:
        assert n_eo == 13
    if N == 7:
        assert n_eo == 25
