"""The solver entries of the C-ABI on their own: a caller that keeps its
own CG loop, as the reference's SolverCG::solve(op, x, b, preconditioner)
(mf_elasticity.h:2015-2051, heat_transfer.h:729-737, 811), uses the
operator, PreconditionMG (mfgpu_mg_*), SolverCG (mfgpu_pcg_solve), the
condition-number estimate and the DoF-numbering map, and nothing else.
Solutions are checked against the oracle's operator: |A x - b| <= 1e-9 |b|
for a solve to 1e-10; the same system through the solid driver takes the
same number of CG iterations (+-1)."""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W
from test_dof_permutation import caller_numbering

pytestmark = pytest.mark.gpu


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def _constrained_mask(spec, nc):
    """True on the rows the Dirichlet faces constrain (x = 0 here)."""
    X, _, _ = W.node_coords(spec["degree"], spec["n_ref"], spec["rep"], spec["lo"], spec["hi"])
    return np.tile(X == spec["lo"][0], nc)


def _nh_system(ctx, degree=2, n_ref=2):
    spec = W.cantilever(degree, n_ref, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    mesh = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 3)
    u = W.smooth_displacement(degree, n_ref, spec["rep"], spec["lo"], spec["hi"], seed=2)
    mat = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
    op = mfgpu.NeoHookOperator(ctx, mesh, -1, 64, "referential_qp")
    op.set_material(mat)
    du = dev(u)
    op.initialize(du)
    op.cache()
    x_true = W.uniform_vector(n, 9)
    x_true[_constrained_mask(spec, 3)] = 0.0
    om = W.to_oracle_mesh(O, spec)
    omat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    b = O.nh_vmult(om, n_ref, omat, "scalar_referential", u, x_true)
    apply_oracle = lambda x: O.nh_vmult(om, n_ref, omat, "scalar_referential", u, x)  # noqa: E731
    return spec, mesh, mat, op, du, u, b, apply_oracle


def test_pcg_with_multigrid_through_the_c_abi(ctx):
    import torch
    spec, mesh, mat, op, du, u, b, apply_oracle = _nh_system(ctx)
    mg = mfgpu.Multigrid(ctx, mesh, "nh", caching="referential_qp", material=mat,
                         solver=mfgpu.solver_params("gmg"))
    assert mg.info() == (3, len(b))
    mg.setup(du)
    db = dev(b)
    x = torch.zeros_like(db)
    tol = 1e-10 * np.linalg.norm(b)
    its, res = mfgpu.pcg_solve(op, x, db, tol, 1000, mg=mg)
    assert res <= tol and 0 < its < 60
    xs = host(x)
    assert np.linalg.norm(apply_oracle(xs) - b) <= 1e-9 * np.linalg.norm(b)
    # the same system through the solid driver: same preconditioner, same CG
    p = mfgpu.SolidParams()
    p.mesh = mesh
    p.material = mat
    p.caching = b"referential_qp"
    p.solver = mfgpu.solver_params("gmg", tol=1e-10)
    p.max_newton, p.dt, p.n_steps, p.traction_id = 10, 0.01, 1, W.TRACTION_ID
    s = mfgpu.Solid(ctx, p)
    x2 = torch.zeros_like(db)
    its2, _ = s.linear_solve(du, db, x2)
    s.close()
    assert abs(its2 - its) <= 1, (its, its2)
    assert np.linalg.norm(host(x2) - xs) <= 1e-8 * np.linalg.norm(xs)
    # a second setup at the same linearisation gives the same iterations
    mg.setup(du)
    x.zero_()
    its3, _ = mfgpu.pcg_solve(op, x, db, tol, 1000, mg=mg)
    assert abs(its3 - its) <= 1
    mg.close()


def test_pcg_heat_multigrid(ctx):
    import torch
    spec = W.unit_cube_heat(3, 2)
    mesh = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 1)
    op = mfgpu.LaplaceOperator(ctx, mesh, -1, 64, True, delta_t=0.1)
    mg = mfgpu.Multigrid(ctx, mesh, "heat", delta_t=0.1,
                         solver=mfgpu.solver_params("gmg", coarse_fp64=True))
    mg.setup()
    om = W.to_oracle_mesh(O, spec)
    x_true = W.uniform_vector(n, 4)
    x_true[_constrained_mask(spec, 1)] = 0.0
    b = O.heat_vmult(om, 2, 0.1, x_true)
    db = dev(b)
    x = torch.zeros_like(db)
    tol = 1e-10 * np.linalg.norm(b)
    its, _ = mfgpu.pcg_solve(op, x, db, tol, 500, mg=mg)
    assert 0 < its < 20
    assert np.linalg.norm(O.heat_vmult(om, 2, 0.1, host(x)) - b) <= 1e-9 * np.linalg.norm(b)
    mg.close()


def test_pcg_jacobi_identity_and_limits(ctx):
    import torch
    spec, mesh, mat, op, du, u, b, apply_oracle = _nh_system(ctx, degree=2, n_ref=1)
    db = dev(b)
    tol = 1e-10 * np.linalg.norm(b)
    x = torch.zeros_like(db)
    with pytest.raises(mfgpu.MfgpuError) as e:  # no diagonal yet
        mfgpu.pcg_solve(op, x, db, tol, 5000, jacobi_omega=0.65)
    assert e.value.code == 6
    op.compute_diagonal()
    its_j, _ = mfgpu.pcg_solve(op, x, db, tol, 5000, jacobi_omega=0.65)
    assert np.linalg.norm(apply_oracle(host(x)) - b) <= 1e-9 * np.linalg.norm(b)
    x.zero_()
    its_i, _ = mfgpu.pcg_solve(op, x, db, tol, 5000)
    assert np.linalg.norm(apply_oracle(host(x)) - b) <= 1e-9 * np.linalg.norm(b)
    assert its_i > its_j > 0
    # an initial guess that already solves the system: zero iterations
    its0, _ = mfgpu.pcg_solve(op, x, db, 1e-6 * np.linalg.norm(b), 10)
    assert its0 == 0
    x.zero_()
    with pytest.raises(mfgpu.MfgpuError) as e:
        mfgpu.pcg_solve(op, x, db, tol, 3)
    assert e.value.code == 5  # MFGPU_ERR_NOT_CONVERGED


def test_condition_number_estimate(ctx):
    """On a 27-DoF heat system the Lanczos estimate converges to the
    condition number of the assembled matrix; after a few iterations it
    bounds it from below (Ritz values lie inside the spectrum)."""
    spec = W.unit_cube_heat(2, 0)
    mesh = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 1)
    om = W.to_oracle_mesh(O, spec)
    A = np.stack([O.heat_vmult(om, 0, 0.1, np.eye(n)[i]) for i in range(n)], axis=1)
    ev = np.linalg.eigvalsh(0.5 * (A + A.T))
    kappa = ev[-1] / ev[0]
    op = mfgpu.LaplaceOperator(ctx, mesh, -1, 64, True, delta_t=0.1)
    b = dev(W.uniform_vector(n, 2))
    full = mfgpu.estimate_condition_number(op, b, n, 1e-13 * float(b.norm()))
    assert abs(full - kappa) <= 1e-6 * kappa, (full, kappa)
    few = mfgpu.estimate_condition_number(op, b, 3)
    assert 1.0 <= few <= kappa * (1 + 1e-10)


def test_solid_condition_estimate_changes_no_result(ctx):
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))

    def run(estimate):
        p = mfgpu.SolidParams()
        p.mesh = W.to_lib_mesh(mfgpu, spec)
        p.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
        p.caching = b"referential_qp"
        p.solver = mfgpu.solver_params("gmg", estimate_condition=estimate, cond_cg_iterations=20)
        p.max_newton, p.tol_f, p.tol_u = 10, 1e-9, 1e-6
        p.dt, p.n_steps, p.traction_id = 0.01, 1, W.TRACTION_ID
        p.traction[:] = [0.0, -100.0, 0.0]
        p.watch[:] = [2.0, 0.5, 0.5]
        s = mfgpu.Solid(ctx, p)
        r = s.step()
        table = s.convergence_table()
        s.close()
        return r, table

    (n0, cg0, sol0, w0), t0 = run(False)
    (n1, cg1, sol1, w1), t1 = run(True)
    # equal up to the round-off of the atomic scatter
    assert (n0, sol0) == (n1, sol1) and abs(cg0 - cg1) <= sol0
    assert np.linalg.norm(np.array(w1) - np.array(w0)) <= 1e-9 * np.linalg.norm(w0)
    rows0 = [r for r in t0.splitlines() if "|" in r and "LIN_IT" not in r]
    rows1 = [r for r in t1.splitlines() if "|" in r and "LIN_IT" not in r]
    assert len(rows0) == len(rows1) == n0 and "CONVERGED" in t1
    cond0 = [float(r.split("|")[1].split()[2]) for r in rows0]
    cond1 = [float(r.split("|")[1].split()[2]) for r in rows1]
    assert all(c == 1.0 for c in cond0) and all(c > 10.0 for c in cond1)


def test_permutation_on_the_device(ctx):
    """A vector in a shuffled, component-interleaved numbering goes to the
    library's numbering and back exactly, and the operator applied through
    the map equals the library's operator on the permuted vector."""
    import torch
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    mesh = W.to_lib_mesh(mfgpu, spec)
    pts, comp, lib_index = caller_numbering(spec, 3)
    perm = mfgpu.Permutation(ctx, mesh, -1, pts, comp)
    n = len(lib_index)
    xc = W.uniform_vector(n, 12)
    d_xc = dev(xc)
    d_xl = torch.zeros_like(d_xc)
    perm.to_library(d_xc, d_xl)
    xl = host(d_xl)
    assert np.array_equal(xl[lib_index], xc)
    back = torch.zeros_like(d_xc)
    perm.from_library(d_xl, back)
    assert np.array_equal(host(back), xc)
    # FP32 too
    f_c = d_xc.float()
    f_l = torch.zeros_like(f_c)
    perm.to_library(f_c, f_l, precision=32)
    assert np.array_equal(host(f_l)[lib_index], xc.astype(np.float32))
    u = W.smooth_displacement(2, 1, spec["rep"], spec["lo"], spec["hi"], seed=2)
    nh = mfgpu.NeoHookOperator(ctx, mesh, -1, 64, "referential_qp")
    nh.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.01))
    du = dev(u)
    nh.initialize(du)
    nh.cache()
    yl = torch.zeros_like(d_xl)
    nh.vmult(yl, d_xl)
    yc = torch.zeros_like(d_xl)
    perm.from_library(yl, yc)
    assert np.array_equal(host(yc), host(yl)[lib_index])
    perm.close()


def test_inclusion_material_and_material_ids(ctx):
    """set_material(material, inclusion) as the reference calls it (the
    inclusion with mu x 100, mf_elasticity.h:470-493): with every cell of
    material id 0 the inclusion applies to no cell and the vmult is the
    one without it; a nonzero material id is refused with
    MFGPU_ERR_UNSUPPORTED, as is an inclusion of another formulation."""
    import torch
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    mesh = W.to_lib_mesh(mfgpu, spec)
    n = W.n_dofs(spec, 3)
    u = dev(W.smooth_displacement(2, 1, spec["rep"], spec["lo"], spec["hi"], seed=2))
    src = dev(W.uniform_vector(n, 3))
    n_cells = 4 * 2 * 2
    out = []
    for with_inclusion in (False, True):
        op = mfgpu.NeoHookOperator(ctx, mesh, -1, 64, "referential_qp")
        op.set_scatter("colored")
        mat = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
        op.set_material(mat, mfgpu.material(0.5e8, 0.4, 1000.0, 0.01) if with_inclusion else None)
        op.set_cell_material_ids(np.zeros(n_cells, dtype=np.uint8))
        op.initialize(u)
        op.cache()
        d = torch.zeros_like(src)
        op.vmult(d, src)
        out.append(host(d))
        ids = np.zeros(n_cells, dtype=np.uint8)
        ids[5] = 1
        with pytest.raises(mfgpu.MfgpuError) as e:
            op.set_cell_material_ids(ids)
        assert e.value.code == 8
        with pytest.raises(mfgpu.MfgpuError) as e:
            op.set_cell_material_ids(np.zeros(n_cells - 1, dtype=np.uint8))
        assert e.value.code == 1
        with pytest.raises(mfgpu.MfgpuError) as e:
            op.set_material(mat, mfgpu.material(0.5e8, 0.4, 1000.0, 0.01, formulation=0))
        assert e.value.code == 8
        op.close()
    assert np.array_equal(out[0], out[1])
