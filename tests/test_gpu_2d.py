"""Two-dimensional device path against the CPU oracle and the reference's
own 2D goldens (tests/solid/*/ *.output of the reference: the turek_hron
flap, Q1, 320 cells; tests/heat/*: the partitioned-heat analytic solution).

Tolerances as in 3D: FP64 operators 1e-12 relative l2, FP32 2e-5,
diagonals 1e-11; solver runs: Newton counts equal, watchpoint within the
goldens' 6 printed digits, average CG within +-1 (GMG) / 1 % (Jacobi)."""
import json
import os

import numpy as np
import pytest

import mfgpu
import oracle as O

pytestmark = pytest.mark.gpu

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))


def rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def dev(x):
    import torch
    return torch.from_numpy(np.ascontiguousarray(x)).cuda()


def host(t):
    import torch
    torch.cuda.synchronize()
    return t.cpu().numpy()


def meshes(degree, n_ref, rep, lo, hi, bid, dirichlet):
    lib = mfgpu.make_mesh(degree, n_ref, rep, lo, hi, boundary_id=bid, dirichlet=dirichlet)
    orc = O.make_mesh(2, degree, degree + 1, n_ref, rep, lo, hi, boundary_id=bid, dirichlet=dirichlet)
    return lib, orc


def heat2(degree):
    return meshes(degree, 1, (3, 2), (0.0, 0.0), (1.2, 0.5), (1, 0, 0, 0), [(1, 1)])


def beam2(degree, n_ref=1):
    return meshes(degree, n_ref, (5, 1), (0.24899, 0.19), (0.6, 0.21), (1, 11, 11, 11), [(1, 0b11)])


def smooth_u2(degree, n_ref, rep, lo, hi, seed=3):
    """2-component smooth displacement on the Q_p nodes of a 2D box, with
    |grad u| <= ~0.05 (det F stays near 1)."""
    import workloads as W
    xs = W.axis_coords(rep[0] << n_ref, lo[0], hi[0], degree)
    ys = W.axis_coords(rep[1] << n_ref, lo[1], hi[1], degree)
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    rng = np.random.Generator(np.random.PCG64(seed))
    L = np.array(hi) - np.array(lo)
    out = []
    for c in range(2):
        ph = rng.uniform(0, 6.28, 2)
        a = 0.05 / (2 * np.pi) * min(L)
        out.append(a * (np.sin(2 * np.pi * X / L[0] + ph[0]) + np.sin(2 * np.pi * Y / L[1] + ph[1])))
    return np.concatenate([o.ravel() for o in out])


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("precision", [64, 32])
def test_heat2d_vmult_and_diagonal(ctx, degree, precision):
    m, om = heat2(degree)
    n = O.n_nodes(om, 1)
    dt = np.float64 if precision == 64 else np.float32
    src = np.random.Generator(np.random.PCG64(1)).uniform(-1, 1, n).astype(dt)
    ref = O.heat_vmult(om, 1, 0.1, src, precision=precision)
    op = mfgpu.LaplaceOperator(ctx, m, -1, precision, True, delta_t=0.1)
    d = dev(np.zeros(n, dt))
    op.vmult(d, dev(src))
    assert rel(host(d).astype(np.float64), np.asarray(ref, np.float64)) < (1e-12 if precision == 64 else 2e-5)
    op.compute_diagonal()
    inv = dev(np.zeros(n, dt))
    op.precondition_Jacobi(inv, dev(np.ones(n, dt)), 1.0)
    ref_inv = O.heat_inv_diagonal(om, 1, 0.1)
    assert rel(host(inv).astype(np.float64), ref_inv) < (1e-11 if precision == 64 else 5e-5)


@pytest.mark.parametrize("degree", [1, 2, 3, 4])
@pytest.mark.parametrize("caching,form", [("scalar_referential", 1), ("tensor4", 1), ("tensor2", 0)])
@pytest.mark.parametrize("precision", [64, 32])
def test_nh2d_vmult_and_diagonal(ctx, degree, caching, form, precision):
    m, om = beam2(degree)
    u = smooth_u2(degree, 1, (5, 1), (0.24899, 0.19), (0.6, 0.21))
    n = len(u)
    dt = np.float64 if precision == 64 else np.float32
    src = np.random.Generator(np.random.PCG64(2)).uniform(-1, 1, n)
    mat_o = O.material(0.5e6, 0.4, 1000.0, 0.1, form)
    ref = O.nh_vmult(om, 1, mat_o, caching, u, src)
    op = mfgpu.NeoHookOperator(ctx, m, -1, precision, caching)
    op.set_material(mfgpu.material(0.5e6, 0.4, 1000.0, 0.1, form))
    d_u = dev(u.astype(dt))
    op.initialize(d_u)
    op.cache()
    d = dev(np.zeros(n, dt))
    op.vmult(d, dev(src.astype(dt)))
    assert rel(host(d).astype(np.float64), ref) < (1e-12 if precision == 64 else 5e-5)
    op.compute_diagonal()
    inv = dev(np.zeros(n, dt))
    op.precondition_Jacobi(inv, dev(np.ones(n, dt)), 1.0)
    ref_inv = O.nh_inv_diagonal(om, 1, mat_o, caching, u)
    assert rel(host(inv).astype(np.float64), ref_inv) < (1e-11 if precision == 64 else 5e-5)


@pytest.mark.parametrize("degree", [1, 2, 4])
@pytest.mark.parametrize("nc", [1, 2])
def test_transfer2d(ctx, degree, nc):
    m, om = beam2(degree, n_ref=2) if nc == 2 else heat2(degree)
    nco = O.n_nodes(om, 0) * nc
    nf = O.n_nodes(om, 1) * nc
    coarse = np.random.Generator(np.random.PCG64(4)).uniform(-1, 1, nco)
    fine = np.random.Generator(np.random.PCG64(5)).uniform(-1, 1, nf)
    ref_f = np.zeros(nf)
    O.transfer(om, 0, nc, "prolongate", coarse.copy(), ref_f)
    d_f = dev(np.zeros(nf))
    mfgpu.prolongate(ctx, m, 0, nc, dev(coarse), d_f)
    assert rel(host(d_f), ref_f) < 1e-13
    ref_c = np.zeros(nco)
    O.transfer(om, 0, nc, "restrict", ref_c, fine.copy())
    d_c = dev(np.zeros(nco))
    mfgpu.restrict_add(ctx, m, 0, nc, d_c, dev(fine))
    assert rel(host(d_c), ref_c) < 1e-13


CASES = {
    "turek_gmg_scalar_referential": ("scalar_referential", "gmg", 1),
    "turek_gmg_tensor2": ("tensor2", "gmg", 1),
    "turek_gmg_tensor4": ("tensor4", "gmg", 1),
    "turek_gmg_tensor4_ns": ("tensor4_ns", "gmg", 1),
    "turek_gmg_tensor2_form0": ("tensor2", "gmg", 0),
    "turek_jacobi_tensor2": ("tensor2", "jacobi", 1),
}


def turek_lib_params(caching, precond, form):
    p = mfgpu.SolidParams()
    p.mesh = mfgpu.make_mesh(1, 3, (5, 1), (0.24899, 0.19), (0.6, 0.21), boundary_id=(1, 11, 11, 11),
                             dirichlet=[(1, 0b11)])
    p.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.1, form)
    p.caching = caching.encode()
    p.solver = mfgpu.solver_params(precond, tol=1e-6, relaxation=0.65, cheb_degree=5, cheb_range=20.0,
                                   cheb_eig_its=30, coarse_accurate=True, mg_precision=32)
    p.max_newton = 10
    p.tol_f, p.tol_f_abs, p.tol_u, p.tol_u_abs = 1e-9, 2e-9, 1e-6, 5e-15
    p.dt, p.n_steps = 0.1, 2
    p.body_force[:] = [0.0, -0.5, 0.0]
    p.traction_id = 11
    p.traction[:] = [0.0, -4.0, 0.0]
    p.watch[:] = [0.6, 0.2, 0.0]
    return p


@pytest.mark.parametrize("case", sorted(CASES))
def test_turek2d_reference_goldens(ctx, case):
    """The reference's own test cases on the device: Newton iterations, the
    watchpoint displacement (6 printed digits) and the average CG count of
    tests/solid/<case>/<case>_serial.output; and the oracle's run."""
    caching, precond, form = CASES[case]
    g = GOLD["solid"][case]
    p = turek_lib_params(caching, precond, form)
    if precond == "jacobi":
        # ~700 Jacobi-CG iterations against a cap of n_dofs (738): the device
        # averages 700.9 (reference 701), but the atomic scatter's summation
        # order moves single solves by a few iterations around the cap
        p.solver.max_it_mult = 2
    r = mfgpu.Solid(ctx, p).run()
    n_steps = len(g["newton_its"])
    assert list(r.newton_its[:n_steps]) == g["newton_its"]
    for s in range(n_steps):
        for d in range(2):
            gold = g["watch_disp"][s][d]
            assert abs(r.watch_disp[s][d] - gold) <= 6e-6 * abs(gold), (s, d, r.watch_disp[s][d], gold)
    avg = r.total_cg // r.n_solves
    if precond == "gmg":
        assert abs(avg - g["avg_cg"]) <= 1, (avg, g["avg_cg"])
    else:
        assert abs(avg - g["avg_cg"]) <= 0.01 * g["avg_cg"], (avg, g["avg_cg"])
    ro = O.solid_run(O.turek_params(caching, precond, form))
    for s in range(n_steps):
        wo = np.array(ro.watch_disp[s][:2])
        wl = np.array(r.watch_disp[s][:2])
        assert np.linalg.norm(wl - wo) <= 1e-8 * np.linalg.norm(wo)


def test_heat2d_analytic_solution(ctx):
    """u = 1 + x^2 + 3 y^2 + 1.3 t reproduced to round-off on the unit square
    (the reference's partitioned-heat golden: L2 error ~1e-13)."""
    import torch
    p = mfgpu.HeatParams()
    p.mesh = mfgpu.make_mesh(2, 3, (1, 1), (0.0, 0.0), (1.0, 1.0), boundary_id=(1, 1, 1, 1),
                             dirichlet=[(1, 1)])
    p.dt, p.n_steps = 0.1, 10
    p.solver = mfgpu.solver_params("gmg", tol=1e-12, cheb_range=15.0, cheb_eig_its=10)
    p.analytic, p.alpha, p.beta = 1, 3.0, 1.3
    h = mfgpu.Heat(ctx, p)
    h.run()
    om = O.make_mesh(2, 2, 3, 3, (1, 1), (0.0, 0.0), (1.0, 1.0))
    n = O.n_nodes(om, 3)
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.copy(u, h.solution_ptr(), n * 8)
    nodes = np.array([0.0, 0.5, 1.0])
    xs = np.concatenate([[c * 0.125 + nodes[i] * 0.125 for i in range(2)] for c in range(8)] + [[1.0]])
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    exact = 1 + X.ravel() ** 2 + 3 * Y.ravel() ** 2 + 1.3 * 1.0
    assert np.max(np.abs(u.cpu().numpy() - exact)) < 1e-11
