"""The CPU oracle against the reference's own blessed outputs.

The reference pins its path only end to end (tests/solid/*/ *_serial.output,
tests/heat/*/ *_serial.output): Newton iterations per step, the watchpoint
displacement at (0.6, 0.2) of the 2D turek_hron beam after each step, the
average CG iteration count, and the heat L2 error against the analytic
solution.  These tests run the oracle's restatement of the same cases and
compare against the committed golden numbers (tests/golden/).
"""
import json
import os

import numpy as np
import pytest

import oracle as O

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden",
                                   "reference_goldens.json")))

CASES = {
    "turek_gmg_scalar_referential": ("scalar_referential", "gmg", 1),
    "turek_gmg_tensor2": ("tensor2", "gmg", 1),
    "turek_gmg_tensor4": ("tensor4", "gmg", 1),
    "turek_gmg_tensor4_ns": ("tensor4_ns", "gmg", 1),
    "turek_gmg_tensor2_form0": ("tensor2", "gmg", 0),
    "turek_jacobi_tensor2": ("tensor2", "jacobi", 1),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_turek_golden(case):
    caching, precond, form = CASES[case]
    g = GOLD["solid"][case]
    p = O.turek_params(caching, precond, form)
    r = O.solid_run(p)
    n_steps = len(g["newton_its"])
    assert r.n_steps == n_steps
    # Newton iteration counts must match exactly
    assert list(r.newton_its[:n_steps]) == g["newton_its"]
    # watchpoint displacement: the goldens print 6 significant digits
    for s in range(n_steps):
        for d in range(2):
            gold = g["watch_disp"][s][d]
            got = r.watch_disp[s][d]
            assert abs(got - gold) <= 6e-6 * abs(gold), (s, d, got, gold)
    avg = r.total_cg // r.n_solves
    if precond == "gmg":
        # CG counts within +-1 of the reference (deal.II's GMG details:
        # Chebyshev eigenvalue start vector and DoF numbering differ)
        assert abs(avg - g["avg_cg"]) <= 1, (avg, g["avg_cg"])
    else:
        # ~700 Jacobi-CG iterations: finite-precision CG, within 1 %
        assert abs(avg - g["avg_cg"]) <= 0.01 * g["avg_cg"], (avg, g["avg_cg"])


def test_turek_mesh_size():
    g = GOLD["solid"]["turek_gmg_tensor4"]
    p = O.turek_params()
    nn = O.n_nodes(p.mesh, p.mesh.n_ref)
    assert 2 * nn == g["n_dofs"] == 738
    assert 40 * 8 == g["n_cells"]
    vol = (0.6 - 0.24899) * (0.21 - 0.19)
    assert abs(vol - g["ref_volume"]) < 1e-6


@pytest.mark.parametrize("dim", [2, 3])
def test_heat_analytic_roundoff(dim):
    """partitioned_heat: u = 1 + x^2 + 3 y^2 + 1.3 t with f = beta - 2 - 2 alpha
    is reproduced by Q2 + backward Euler to round-off (golden max L2 error
    1.3e-13 for the coupled run, 10 steps of dt = 0.1)."""
    p = O.HeatParams()
    p.mesh = O.make_mesh(dim, 2, 3, 3 if dim == 2 else 2, (1,) * dim,
                         (0.0,) * dim, (1.0,) * dim, boundary_id=(1,) * 6,
                         dirichlet=[(1, 1)])
    p.dt, p.n_steps, p.tol_rel, p.precond = 0.1, 10, 1e-12, 2
    p.analytic, p.alpha, p.beta, p.mg_float = 1, 3.0, 1.3, 1
    r = O.heat_run(p)
    errs = np.array(r.l2_error[:10])
    gold = GOLD["heat"]["partitioned-heat"]["max_l2_error"]
    assert errs.max() < 10 * gold, errs


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("degree", [3, 4, 5, 6])
def test_heat_analytic_roundoff_higher_degree(dim, degree):
    """The same analytic solution lies in Q_p for every p >= 2, so the heat
    step reproduces it to round-off at every degree the path supports (CG to
    1e-12 relative; the errors seen are 5e-14 .. 1.6e-12)."""
    p = O.HeatParams()
    p.mesh = O.make_mesh(dim, degree, degree + 1, 2 if dim == 2 else 1, (1,) * dim,
                         (0.0,) * dim, (1.0,) * dim, boundary_id=(1,) * 6,
                         dirichlet=[(1, 1)])
    p.dt, p.n_steps, p.tol_rel, p.precond = 0.1, 10, 1e-12, 2
    p.analytic, p.alpha, p.beta, p.mg_float = 1, 3.0, 1.3, 1
    r = O.heat_run(p)
    errs = np.array(r.l2_error[:10])
    assert errs.max() < 1e-11, errs
