"""Device solvers (GMG-preconditioned CG, Newton-Newmark, backward Euler)
through the C-ABI against the CPU oracle: Newton iteration counts equal,
watchpoint displacement within 1e-8 relative, average CG counts within +-1,
heat solutions within the solver tolerance."""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu


def solid_pair(spec, caching="scalar_referential", precond="gmg", formulation=1,
               dt=0.01, n_steps=2, traction=(0.0, -100.0, 0.0), mg_precision=32,
               watch=None):
    watch = watch or (spec["hi"][0], 0.5 * spec["hi"][1], 0.5 * spec["hi"][2])
    # oracle
    po = O.SolidParams()
    po.mesh = W.to_oracle_mesh(O, spec)
    po.mat = O.material(0.5e6, 0.4, 1000.0, dt, formulation)
    po.caching = O.CACHING["scalar_referential" if caching == "referential_qp" else caching]
    po.precond = {"none": 0, "jacobi": 1, "gmg": 2}[precond]
    po.relaxation, po.tol_lin, po.max_it_mult, po.max_newton = 0.65, 1e-6, 1, 10
    po.tol_f, po.tol_f_abs, po.tol_u, po.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    po.dt, po.n_steps = dt, n_steps
    po.body_force[:] = [0.0, 0.0, 0.0]
    po.traction_id = W.TRACTION_ID
    po.traction[:] = list(traction)
    po.watch[:] = list(watch)
    po.cheb_degree, po.cheb_range, po.cheb_eig_its, po.coarse_accurate = 5, 20.0, 30, 1
    po.mg_float = 1 if mg_precision == 32 else 0
    # library
    pl = mfgpu.SolidParams()
    pl.mesh = W.to_lib_mesh(mfgpu, spec)
    pl.material = mfgpu.material(0.5e6, 0.4, 1000.0, dt, formulation)
    pl.caching = caching.encode()
    pl.solver = mfgpu.solver_params(precond, tol=1e-6, mg_precision=mg_precision)
    pl.max_newton = 10
    pl.tol_f, pl.tol_f_abs, pl.tol_u, pl.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    pl.dt, pl.n_steps = dt, n_steps
    pl.body_force[:] = [0.0, 0.0, 0.0]
    pl.traction_id = W.TRACTION_ID
    pl.traction[:] = list(traction)
    pl.watch[:] = list(watch)
    return po, pl


@pytest.mark.parametrize("degree,caching,precond,form", [
    (1, "scalar_referential", "gmg", 1),
    (2, "scalar_referential", "gmg", 1),
    (2, "tensor4", "gmg", 1),
    (2, "referential_qp", "gmg", 1),
    (3, "tensor2", "jacobi", 1),
    (2, "tensor2", "gmg", 0),
])
def test_solid_newton_newmark(ctx, degree, caching, precond, form):
    spec = W.cantilever(degree, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    po, pl = solid_pair(spec, caching, precond, form)
    ro = O.solid_run(po)
    s = mfgpu.Solid(ctx, pl)
    rl = s.run()
    n = po.n_steps
    assert list(rl.newton_its[:n]) == list(ro.newton_its[:n])
    for st in range(n):
        wo = np.array(ro.watch_disp[st][:3])
        wl = np.array(rl.watch_disp[st][:3])
        assert np.linalg.norm(wl - wo) <= 1e-8 * np.linalg.norm(wo), (st, wl, wo)
    avg_o = ro.total_cg / ro.n_solves
    avg_l = rl.total_cg / rl.n_solves
    assert abs(avg_l - avg_o) <= 1.0, (avg_l, avg_o)


def test_solid_all_fp64_vcycle(ctx):
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    po, pl = solid_pair(spec, mg_precision=64)
    ro = O.solid_run(po)
    rl = mfgpu.Solid(ctx, pl).run()
    assert list(rl.newton_its[:2]) == list(ro.newton_its[:2])
    wo = np.array(ro.watch_disp[1][:3])
    wl = np.array(rl.watch_disp[1][:3])
    assert np.linalg.norm(wl - wo) <= 1e-8 * np.linalg.norm(wo)


def heat_pair(spec, analytic=False, n_steps=1, tol=1e-10, mg_precision=32):
    po = O.HeatParams()
    po.mesh = W.to_oracle_mesh(O, spec)
    po.dt, po.n_steps, po.tol_rel, po.precond = 0.1, n_steps, tol, 2
    po.analytic, po.alpha, po.beta = int(analytic), 3.0, 1.3
    po.mg_float = 1 if mg_precision == 32 else 0
    pl = mfgpu.HeatParams()
    pl.mesh = W.to_lib_mesh(mfgpu, spec)
    pl.dt, pl.n_steps = 0.1, n_steps
    pl.solver = mfgpu.solver_params("gmg", tol=tol, cheb_range=15.0, cheb_eig_its=10,
                                    mg_precision=mg_precision)
    pl.analytic, pl.alpha, pl.beta = int(analytic), 3.0, 1.3
    if not analytic:
        c, w, a = W.gaussian_source(0)
        po.n_gauss = pl.n_gauss = 8
        for i in range(8):
            for d in range(3):
                po.g_center[i][d] = pl.g_center[i][d] = c[i, d]
            po.g_width[i] = pl.g_width[i] = w[i]
            po.g_amp[i] = pl.g_amp[i] = a[i]
    return po, pl


def test_heat_analytic_solution(ctx):
    """u = 1 + x^2 + 3 y^2 + 1.3 t is reproduced to round-off (the
    reference's partitioned-heat golden, here on a single 3D domain with
    Dirichlet data on all faces)."""
    import torch
    spec = W.unit_cube_heat(2, 2)
    spec["boundary_id"] = (1, 1, 1, 1, 1, 1)
    po, pl = heat_pair(spec, analytic=True, n_steps=5, tol=1e-12)
    h = mfgpu.Heat(ctx, pl)
    r = h.run()
    n = W.n_dofs(spec, 1)
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.copy(u, h.solution_ptr(), n * 8)
    X, Y, Z = W.node_coords(2, 2, spec["rep"], spec["lo"], spec["hi"])
    exact = 1 + X ** 2 + 3 * Y ** 2 + 1.3 * 0.5
    assert np.max(np.abs(u.cpu().numpy() - exact)) < 1e-11
    ro = O.heat_run(po)
    assert all(abs(a - b) <= 1 for a, b in zip(r.cg_its[:5], ro.cg_its[:5]))


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_heat_gaussian_step(ctx, degree):
    import torch
    spec = W.unit_cube_heat(degree, 2)
    po, pl = heat_pair(spec, analytic=False, n_steps=1, tol=1e-10)
    ro, uo = O.heat_run(po, return_u=True)
    h = mfgpu.Heat(ctx, pl)
    r = h.run()
    n = W.n_dofs(spec, 1)
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.copy(u, h.solution_ptr(), n * 8)
    ul = u.cpu().numpy()
    assert np.linalg.norm(ul - uo) / np.linalg.norm(uo) < 1e-8
    assert abs(r.cg_its[0] - ro.cg_its[0]) <= 1


@pytest.mark.parametrize("mg_precision", [32, 64])
def test_vcycle_graph_replay_matches_eager(ctx, mg_precision):
    """The V-cycle replayed as a CUDA graph gives the same Newton and CG
    counts and the same displacement (to round-off of the atomic scatter) as
    the eagerly launched V-cycle."""
    spec = W.cantilever(2, 2, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    res = {}
    for graphs in (False, True):
        _, pl = solid_pair(spec, "referential_qp", mg_precision=mg_precision)
        pl.solver.cuda_graphs = int(graphs)
        res[graphs] = mfgpu.Solid(ctx, pl).run()
    e, g = res[False], res[True]
    assert list(e.newton_its[:2]) == list(g.newton_its[:2])
    assert abs(e.total_cg - g.total_cg) <= 1
    for st in range(2):
        we, wg = np.array(e.watch_disp[st][:3]), np.array(g.watch_disp[st][:3])
        assert np.linalg.norm(wg - we) <= 1e-10 * np.linalg.norm(we)


def test_heat_graph_replay_matches_eager(ctx):
    spec = W.unit_cube_heat(3, 3)
    its = {}
    for graphs in (False, True):
        _, pl = heat_pair(spec, n_steps=2, tol=1e-10)
        pl.solver.cuda_graphs = int(graphs)
        its[graphs] = list(mfgpu.Heat(ctx, pl).run().cg_its[:2])
    assert its[False] == its[True]


def test_driver_timing_sections(ctx):
    """The drivers' wall-clock sections (the reference's TimerOutput): every
    section of a Newton-Newmark run and of a heat step is reported with its
    call count, the results do not change with timing on, and the sections
    add up to no more than the elapsed time."""
    spec = W.cantilever(2, 1, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    _, pl = solid_pair(spec, "referential_qp")
    plain = mfgpu.Solid(ctx, pl).run()
    s = mfgpu.Solid(ctx, pl)
    s.set_timing(True)
    r = s.run()
    text = s.timing_summary()
    tab = mfgpu.timing_table(text)
    newton = sum(r.newton_its[:2])
    assert tab["Linear solver"][0] == r.n_solves == newton
    assert tab["Assemble residual"][0] == newton + 2  # one more residual per step: the converged one
    for name in ("Setup MF: cache()", "Setup MF: diagonal()", "Setup MF: interpolate_to_mg",
                 "Setup MF: GMG setup"):
        assert tab[name][0] >= r.n_solves and tab[name][1] > 0, (name, text)
    assert sum(v[1] for v in tab.values()) <= r.seconds * 1.05 + 1e-3, text
    assert list(r.newton_its[:2]) == list(plain.newton_its[:2]) and r.total_cg == plain.total_cg
    s.set_timing(False)
    assert mfgpu.timing_table(s.timing_summary()) == {}
    s.close()
    _, ph = heat_pair(W.unit_cube_heat(2, 2), n_steps=3, tol=1e-10)
    h = mfgpu.Heat(ctx, ph)
    h.set_timing(True)
    h.run()
    th = mfgpu.timing_table(h.timing_summary())
    assert th["assemble rhs"][0] == 3 and th["GMG setup"][0] == 3 and th["solve system"][0] == 3
    h.close()


@pytest.mark.parametrize("mg_precision", [32, 64])
def test_dense_coarse_operator_solver_equivalence(ctx, mg_precision):
    """The level-0 operator as a dense matrix (default) and matrix-free give
    the same Newton and CG counts and the same displacement to round-off
    (the dense copy changes only the summation order of the coarse
    Chebyshev steps)."""
    spec = W.cantilever(2, 2, rep=(2, 1, 1), length=(2.0, 1.0, 1.0))
    res = {}
    for dense in (False, True):
        _, pl = solid_pair(spec, "referential_qp", mg_precision=mg_precision)
        pl.solver.coarse_dense = int(dense)
        res[dense] = mfgpu.Solid(ctx, pl).run()
    a, b = res[False], res[True]
    assert list(a.newton_its[:2]) == list(b.newton_its[:2])
    assert abs(a.total_cg - b.total_cg) <= 1
    for st in range(2):
        wa, wb = np.array(a.watch_disp[st][:3]), np.array(b.watch_disp[st][:3])
        assert np.linalg.norm(wb - wa) <= 1e-9 * np.linalg.norm(wa)


def test_heat_steps_reuse_the_multigrid_setup(ctx):
    """Heat time steps after the first keep the multigrid setup (unchanged
    level operators): the "GMG setup" section of the later steps costs a
    small fraction of the first, and the CG counts equal the oracle's."""
    spec = W.unit_cube_heat(2, 3)
    po, pl = heat_pair(spec, n_steps=4, tol=1e-10)
    ro = O.heat_run(po)
    h = mfgpu.Heat(ctx, pl)
    h.set_timing(True)
    its = [h.step() for _ in range(4)]
    first = mfgpu.timing_table(h.timing_summary())["GMG setup"][1]
    h.set_timing(True)  # clears the table
    for _ in range(3):
        its.append(h.step())
    later = mfgpu.timing_table(h.timing_summary())["GMG setup"][1] / 3
    assert later < 0.2 * first, (first, later)
    assert all(abs(a - b) <= 1 for a, b in zip(its[:4], ro.cg_its[:4]))
    h.close()
