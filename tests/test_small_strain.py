"""J and ln J at small strain, computed from the displacement gradient.

For a linear displacement u = H0 X the deformation gradient F = I + H0 is
constant, so the Newton residual (zero acceleration, body force and
traction) is r_{c,i} = -sum_d P_cd oint phi_i n_d dS with the constant first
Piola-Kirchhoff stress P = tau F^{-T}, tau = mu b - (mu - 2 lambda ln J) I
(material.h:116-161; Solid::assemble_residual, mf_elasticity.h:1766-1845).
The expected residual is evaluated in numpy long double, with J - 1 from
the invariants of H0 and ln J = log1p(J - 1).

At |H0| ~ 1e-9, det F - 1 and mu b - mu cancel nine digits: evaluating
std::log(determinant(F)) as the reference does (mf_nh_operator.h:448,457)
leaves ~1e-7 relative error in the residual.  The oracle and the device
compute J - 1 from the invariants of Grad u and ln J with log1p, and
tau = mu (H + H^T + H H^T) + 2 lambda ln J I; both must reach 1e-12.
"""
import numpy as np
import pytest

import oracle as O
import workloads as W

LD = np.longdouble
MU, NU = 0.5e6, 0.4


def _h0(dim, seed=11, scale=1e-9):
    rng = np.random.Generator(np.random.PCG64(seed))
    return rng.uniform(-1.0, 1.0, (dim, dim)) * scale


def _boundary_mass_1d(n_cells, p, h):
    """int phi_k dx along one axis for every node k of the Q_p line."""
    gl = W.gauss_lobatto(p)
    xg, wg = np.polynomial.legendre.leggauss(p + 1)
    xg, wg = (xg + 1) / 2, wg / 2
    w = np.zeros(p + 1)
    for i in range(p + 1):
        li = np.ones_like(xg)
        for j in range(p + 1):
            if j != i:
                li *= (xg - gl[j]) / (gl[i] - gl[j])
        w[i] = np.dot(wg, li)
    out = np.zeros(n_cells * p + 1)
    for c in range(n_cells):
        out[c * p:c * p + p + 1] += w * h
    return out


def expected_residual(dim, degree, n_ref, rep, lo, hi, H0):
    """-P : oint phi n dS for the constant P of F = I + H0 (long double)."""
    H = H0.astype(LD)
    lam = LD(2) * LD(MU) * LD(NU) / (LD(1) - LD(2) * LD(NU))
    if dim == 2:
        jm1 = (H[0, 0] + H[1, 1]) + (H[0, 0] * H[1, 1] - H[0, 1] * H[1, 0])
    else:
        i1 = H[0, 0] + H[1, 1] + H[2, 2]
        i2 = (H[0, 0] * H[1, 1] - H[0, 1] * H[1, 0]) + (H[0, 0] * H[2, 2] - H[0, 2] * H[2, 0]) + \
             (H[1, 1] * H[2, 2] - H[1, 2] * H[2, 1])
        i3 = H[0, 0] * (H[1, 1] * H[2, 2] - H[1, 2] * H[2, 1]) - \
            H[0, 1] * (H[1, 0] * H[2, 2] - H[1, 2] * H[2, 0]) + \
            H[0, 2] * (H[1, 0] * H[2, 1] - H[1, 1] * H[2, 0])
        jm1 = i1 + (i2 + i3)
    lnJ = np.log1p(jm1)
    tau = LD(MU) * (H + H.T + H @ H.T) + LD(2) * lam * lnJ * np.eye(dim, dtype=LD)
    F = np.eye(dim, dtype=LD) + H
    J = LD(1) + jm1
    if dim == 2:
        adj = np.array([[F[1, 1], -F[0, 1]], [-F[1, 0], F[0, 0]]], dtype=LD)
    else:
        adj = np.empty((3, 3), dtype=LD)
        for i in range(3):
            for j in range(3):
                r = [k for k in range(3) if k != j]
                c = [k for k in range(3) if k != i]
                m = F[np.ix_(r, c)]
                adj[i, j] = (-1) ** (i + j) * (m[0, 0] * m[1, 1] - m[0, 1] * m[1, 0])
    Fi = adj / J
    P = tau @ Fi.T
    nc = [rep[d] << n_ref for d in range(dim)]
    h = [(hi[d] - lo[d]) / nc[d] for d in range(dim)]
    m1 = [_boundary_mass_1d(nc[d], degree, h[d]) for d in range(dim)]
    nn = [nc[d] * degree + 1 for d in range(dim)]
    # B[d] = oint phi n_d dS on the lexicographic node grid (x fastest)
    B = []
    for d in range(dim):
        sign = np.zeros(nn[d])
        sign[0], sign[-1] = -1.0, 1.0
        fac = [m1[e] if e != d else sign for e in range(dim)]
        grid = fac[0]
        for e in range(1, dim):
            grid = np.multiply.outer(fac[e], grid)
        B.append(grid.ravel())
    r = np.zeros((dim, B[0].size), dtype=LD)
    for c in range(dim):
        for d in range(dim):
            r[c] -= P[c, d] * B[d].astype(LD)
    return r.ravel()


def _linear_u(dim, degree, n_ref, rep, lo, hi, H0):
    axes = [W.axis_coords(rep[d] << n_ref, lo[d], hi[d], degree) for d in range(dim)]
    grids = np.meshgrid(*axes[::-1], indexing="ij")[::-1]  # X, Y(, Z), x fastest
    X = [g.ravel() for g in grids]
    return np.concatenate([sum(H0[c, d] * X[d] for d in range(dim)) for c in range(dim)])


CASES = {
    3: dict(degree=2, n_ref=1, rep=(2, 1, 1), lo=(0.0, 0.0, 0.0), hi=(2.0, 1.0, 1.0)),
    2: dict(degree=3, n_ref=1, rep=(3, 2), lo=(0.0, 0.0), hi=(1.5, 1.0)),
}


def _rel(a, b):
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(np.asarray(a, dtype=np.float64) - b) / np.linalg.norm(b))


@pytest.mark.parametrize("dim", [3, 2])
def test_oracle_residual_at_small_strain(dim):
    c = CASES[dim]
    H0 = _h0(dim)
    u = _linear_u(dim, c["degree"], c["n_ref"], c["rep"], c["lo"], c["hi"], H0)
    om = O.make_mesh(dim, c["degree"], c["degree"] + 1, c["n_ref"], c["rep"], c["lo"], c["hi"])
    got = O.nh_residual(om, c["n_ref"], O.material(MU, NU, 1000.0, 0.01), u, np.zeros_like(u))
    ref = expected_residual(dim, c["degree"], c["n_ref"], c["rep"], c["lo"], c["hi"], H0)
    assert _rel(got, ref) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("dim", [3, 2])
def test_device_residual_at_small_strain(ctx, dim):
    import torch
    import mfgpu
    c = CASES[dim]
    H0 = _h0(dim)
    u = _linear_u(dim, c["degree"], c["n_ref"], c["rep"], c["lo"], c["hi"], H0)
    p = mfgpu.SolidParams()
    p.mesh = mfgpu.make_mesh(c["degree"], c["n_ref"], c["rep"], c["lo"], c["hi"])
    p.material = mfgpu.material(MU, NU, 1000.0, 0.01)
    p.caching = b"referential_qp"
    p.solver = mfgpu.solver_params("none")
    p.max_newton, p.dt, p.n_steps, p.traction_id = 10, 0.01, 1, -1
    s = mfgpu.Solid(ctx, p)
    du = torch.from_numpy(u).cuda()
    acc = torch.zeros_like(du)
    rhs = torch.zeros_like(du)
    s.residual(du, acc, rhs)
    torch.cuda.synchronize()
    got = rhs.cpu().numpy()
    s.close()
    ref = expected_residual(dim, c["degree"], c["n_ref"], c["rep"], c["lo"], c["hi"], H0)
    assert _rel(got, ref) < 1e-12, _rel(got, ref)
