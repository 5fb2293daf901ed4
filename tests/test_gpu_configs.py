"""Device solvers at the benchmark workloads, against the CPU oracle.

The oracle runs its cell-batched form (`fast`), which equals its plain loops
to 1e-12 (tests/test_oracle_fast.py), so that these full-size solves finish
in seconds on the host cores.  Bars (the reference path is
mf_elasticity.h:1402-1491 for Newton-Newmark and 1983-2070 for the linear
solve; heat_transfer.h:715-812 for the heat step):

* heat step, unit cube 16^3 cells Q2 (35,937 DoFs), GMG-CG to 1e-10:
  solution within 1e-8 relative l2 of the oracle's, CG iterations +-1;
* Newton-Newmark, cantilever 64x8x8 cells Q4 (839,619 DoFs), 5 steps:
  Newton iterations equal per step, average CG per linear solve +-1,
  watchpoint displacement within 1e-8 relative per step;
* one Newton system of the cantilever 128x16x16 cells Q3 (2,773,155 DoFs)
  to a 1e-8 relative residual, FP64 CG with an FP32 V-cycle and with an
  all-FP64 V-cycle: l2 and max error against the oracle's FP64-everywhere
  solve to 1e-12 below 1e-8, CG iterations +-1 of the oracle's;
* heat step on the unit cube 64^3 cells at Q2 (2.1M DoFs) and Q5 (33M
  DoFs), GMG-CG to 1e-8 with an FP32 and an FP64 V-cycle: error against
  the oracle's FP64-everywhere solve to 1e-12 below 1e-7, CG iterations +-1.
"""
import numpy as np
import pytest

import mfgpu
import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _heat_params(spec, tol, mg_float, fast):
    c, w, a = W.gaussian_source(0)
    po = O.HeatParams()
    po.mesh = W.to_oracle_mesh(O, spec)
    po.dt, po.n_steps, po.tol_rel, po.precond = 0.1, 1, tol, 2
    po.mg_float, po.fast = int(mg_float), int(fast)
    pl = mfgpu.HeatParams()
    pl.mesh = W.to_lib_mesh(mfgpu, spec)
    pl.dt, pl.n_steps = 0.1, 1
    pl.solver = mfgpu.solver_params("gmg", tol=tol, cheb_range=15.0, cheb_eig_its=10,
                                    mg_precision=32 if mg_float else 64,
                                    coarse_fp64=bool(mg_float))
    po.n_gauss = pl.n_gauss = 8
    for i in range(8):
        for d in range(3):
            po.g_center[i][d] = pl.g_center[i][d] = c[i, d]
        po.g_width[i] = pl.g_width[i] = w[i]
        po.g_amp[i] = pl.g_amp[i] = a[i]
    return po, pl


def _device_heat(ctx, pl, n):
    import torch
    h = mfgpu.Heat(ctx, pl)
    r = h.run()
    u = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    ctx.copy(u, h.solution_ptr(), n * 8)
    out = u.cpu().numpy()
    h.close()
    return r, out


def test_heat_step_16cube_q2(ctx):
    spec = W.unit_cube_heat(2, 4)
    n = W.n_dofs(spec, 1)
    po, pl = _heat_params(spec, 1e-10, mg_float=True, fast=False)
    ro, uo = O.heat_run(po, return_u=True)
    rl, ul = _device_heat(ctx, pl, n)
    assert _rel(ul, uo) < 1e-8
    assert abs(rl.cg_its[0] - ro.cg_its[0]) <= 1, (rl.cg_its[0], ro.cg_its[0])


def _solid_params(spec, n_steps, tol_lin, mg_float, fast=True):
    po = O.SolidParams()
    po.mesh = W.to_oracle_mesh(O, spec)
    po.mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    po.caching = O.CACHING["tensor2"]
    po.precond = 2
    po.relaxation, po.tol_lin, po.max_it_mult, po.max_newton = 0.65, tol_lin, 1, 10
    po.tol_f, po.tol_f_abs, po.tol_u, po.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    po.dt, po.n_steps = 0.01, n_steps
    po.traction_id = W.TRACTION_ID
    po.traction[:] = [0.0, -100.0, 0.0]
    po.watch[:] = [spec["hi"][0], 0.5 * spec["hi"][1], 0.5 * spec["hi"][2]]
    po.cheb_degree, po.cheb_range, po.cheb_eig_its, po.coarse_accurate = 5, 20.0, 30, 1
    po.mg_float, po.fast = int(mg_float), int(fast)
    pl = mfgpu.SolidParams()
    pl.mesh = W.to_lib_mesh(mfgpu, spec)
    pl.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
    pl.caching = b"referential_qp"
    pl.solver = mfgpu.solver_params("gmg", tol=tol_lin, mg_precision=32 if mg_float else 64,
                                    coarse_fp64=False)
    pl.max_newton = 10
    pl.tol_f, pl.tol_f_abs, pl.tol_u, pl.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    pl.dt, pl.n_steps = 0.01, n_steps
    pl.traction_id = W.TRACTION_ID
    pl.traction[:] = [0.0, -100.0, 0.0]
    pl.watch[:] = list(po.watch[:])
    return po, pl


def test_solid_newton_newmark_64x8x8_q4_five_steps(ctx):
    spec = W.cantilever(4, 3)
    po, pl = _solid_params(spec, 5, 1e-6, mg_float=True)
    ro = O.solid_run(po)
    s = mfgpu.Solid(ctx, pl)
    rl = s.run()
    s.close()
    assert list(rl.newton_its[:5]) == list(ro.newton_its[:5])
    for st in range(5):
        wo = np.array(ro.watch_disp[st][:3])
        wl = np.array(rl.watch_disp[st][:3])
        assert np.linalg.norm(wl - wo) <= 1e-8 * np.linalg.norm(wo), (st, wl, wo)
    avg_o = ro.total_cg / ro.n_solves
    avg_l = rl.total_cg / rl.n_solves
    assert abs(avg_l - avg_o) <= 1.0, (avg_l, avg_o)


@pytest.fixture(scope="module")
def q3_oracle_solution():
    """The oracle's FP64-everywhere solve (FP64 V-cycle) of the first Newton
    system of the 128x16x16-cell Q3 cantilever to 1e-12."""
    spec = W.cantilever(3, 4)
    po, _ = _solid_params(spec, 1, 1e-12, mg_float=False)
    _, _, _, du = O.solid_first_solve(po, 1e-12)
    return spec, du


@pytest.mark.parametrize("mg_float", [True, False], ids=["fp32_vcycle", "fp64_vcycle"])
def test_newton_system_128x16x16_q3_against_fp64_oracle(ctx, q3_oracle_solution, mg_float):
    import torch
    spec, du_ref = q3_oracle_solution
    po, pl = _solid_params(spec, 1, 1e-8, mg_float=mg_float)
    pl.solver.coarse_fp64 = int(mg_float)
    its_o, _, _, _ = O.solid_first_solve(po, 1e-8)
    n = W.n_dofs(spec, 3)
    zero = torch.zeros(n, dtype=torch.float64, device="cuda")
    rhs = torch.zeros_like(zero)
    du = torch.zeros_like(zero)
    s = mfgpu.Solid(ctx, pl)
    s.residual(zero, zero, rhs)
    its, _ = s.linear_solve(zero, rhs, du)
    s.close()
    got = du.cpu().numpy()
    l2 = _rel(got, du_ref)
    mx = float(np.max(np.abs(got - du_ref)) / np.max(np.abs(du_ref)))
    assert l2 < 1e-8 and mx < 1e-8, (l2, mx)
    assert abs(its - its_o) <= 1, (its, its_o)


@pytest.mark.parametrize("degree", [2, 5])
def test_heat_step_64cube_against_fp64_oracle(ctx, degree):
    spec = W.unit_cube_heat(degree, 6)
    n = W.n_dofs(spec, 1)
    po_ref, _ = _heat_params(spec, 1e-12, mg_float=False, fast=True)
    _, u_ref = O.heat_run(po_ref, return_u=True)
    for mg_float in (True, False):
        po, pl = _heat_params(spec, 1e-8, mg_float=mg_float, fast=True)
        ro = O.heat_run(po)
        rl, ul = _device_heat(ctx, pl, n)
        assert _rel(ul, u_ref) < 1e-7, (mg_float, _rel(ul, u_ref))
        assert abs(rl.cg_its[0] - ro.cg_its[0]) <= 1, (mg_float, rl.cg_its[0], ro.cg_its[0])
