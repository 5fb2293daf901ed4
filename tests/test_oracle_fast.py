"""The throughput form of the oracle's tangent and heat vmults (oracle/oracle_fast.hpp,
timed as the CPU baseline) gives the oracle's vmult (mf_nh_operator.h:545-625)
to round-off: every degree 1-6, every caching variant, every lane count,
on meshes whose colours leave partly filled cell batches and with a clamped
face (constrained DoFs read as zero, identity rows)."""
import numpy as np
import pytest

import oracle as O
import workloads as W

ANISO = dict(rep=(3, 1, 1), length=(3.0, 1.0, 0.7))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("caching", ["scalar_referential", "tensor2", "tensor4", "tensor4_ns"])
@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_fast_form_matches_oracle(degree, caching, lanes):
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    for n_ref in (0, 1):
        spec = W.cantilever(degree, n_ref, **ANISO)
        u = W.smooth_displacement(degree, n_ref, spec["rep"], spec["lo"], spec["hi"], seed=3)
        om = W.to_oracle_mesh(O, spec)
        x = W.uniform_vector(len(u), 12)
        ref = O.nh_vmult(om, n_ref, mat, caching, u, x)
        got, secs = O.nh_vmult_fast_timed(om, n_ref, mat, caching, u, x, 2, lanes=lanes)
        assert rel(got, ref) < 1e-13, (n_ref, rel(got, ref))
        assert secs > 0.0


def test_fast_form_rejects_what_it_does_not_cover():
    spec = W.cantilever(2, 0, **ANISO)
    u = W.smooth_displacement(2, 0, spec["rep"], spec["lo"], spec["hi"], seed=3)
    om = W.to_oracle_mesh(O, spec)
    x = W.uniform_vector(len(u), 12)
    with pytest.raises(RuntimeError):
        O.nh_vmult_fast_timed(om, 0, O.material(0.5e6, 0.4, 1000.0, 0.01, formulation=0),
                              "tensor4_ns", u, x, 1)
    with pytest.raises(RuntimeError):
        O.nh_vmult_fast_timed(om, 0, O.material(0.5e6, 0.4, 1000.0, 0.01), "tensor4_ns", u, x, 1,
                              lanes=3)


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_fast_heat_matches_oracle(degree, lanes):
    """The heat operator M + k dt K (heat_transfer.h:236-250) in the same
    form, with a Dirichlet face, to round-off."""
    for n_ref in (0, 1):
        spec = W.unit_cube_heat(degree, n_ref, rep=(3, 1, 1))
        spec["hi"] = (1.0, 0.6, 0.45)
        om = W.to_oracle_mesh(O, spec)
        x = W.uniform_vector(W.n_dofs(spec, 1), 13)
        ref = O.heat_vmult(om, n_ref, 0.1, x)
        got, secs = O.heat_vmult_fast_timed(om, n_ref, 0.1, x, 2, lanes=lanes)
        assert rel(got, ref) < 1e-13, (n_ref, rel(got, ref))
        assert secs > 0.0


def _solid_params(spec, caching, mg_float, fast):
    p = O.SolidParams()
    p.mesh = W.to_oracle_mesh(O, spec)
    p.mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    p.caching = O.CACHING[caching]
    p.precond, p.dt, p.n_steps, p.max_newton, p.max_it_mult = 2, 0.01, 1, 10, 1
    p.relaxation, p.tol_lin = 0.65, 1e-8
    p.traction_id = W.TRACTION_ID
    p.traction[:] = [0.0, -100.0, 0.0]
    p.cheb_degree, p.cheb_range, p.cheb_eig_its, p.coarse_accurate = 5, 20.0, 30, 1
    p.mg_float, p.fast = mg_float, fast
    return p


@pytest.mark.parametrize("degree,n_ref", [(1, 2), (2, 1), (3, 1)])
@pytest.mark.parametrize("caching", ["scalar_referential", "tensor2", "tensor4", "tensor4_ns"])
@pytest.mark.parametrize("mg_float", [1, 0])
def test_fast_first_solve_matches_plain(degree, n_ref, caching, mg_float):
    """The GMG-CG solve of the first Newton system (mf_elasticity.h:1983-2070)
    with every operator, level operator and diagonal in the throughput form
    takes the same CG iterations as with the oracle's loops and gives the
    same update (FP64 levels to round-off, FP32 levels to FP32 round-off
    amplified by the solve)."""
    spec = W.cantilever(degree, n_ref)
    a = O.solid_first_solve(_solid_params(spec, caching, mg_float, 0), 1e-8)
    b = O.solid_first_solve(_solid_params(spec, caching, mg_float, 1), 1e-8)
    # CG within +-1 (round-off in the FP32 V-cycle can move the step that
    # crosses the tolerance); equal counts here give round-off-level updates
    assert abs(a[0] - b[0]) <= 1
    if a[0] == b[0]:
        assert rel(b[3], a[3]) < (1e-12 if mg_float == 0 else 1e-10)
    else:
        assert rel(b[3], a[3]) < 1e-6


@pytest.mark.parametrize("degree", [1, 2, 3])
def test_fast_heat_step_matches_plain(degree):
    c, w, a = W.gaussian_source(0)
    res = []
    for fast in (0, 1):
        p = O.HeatParams()
        p.mesh = W.to_oracle_mesh(O, W.unit_cube_heat(degree, 2))
        p.dt, p.n_steps, p.tol_rel, p.precond, p.mg_float, p.fast = 0.1, 2, 1e-10, 2, 1, fast
        p.n_gauss = 8
        for i in range(8):
            for d in range(3):
                p.g_center[i][d] = c[i, d]
            p.g_width[i] = w[i]
            p.g_amp[i] = a[i]
        res.append(O.heat_run(p, return_u=True))
    (ra, ua), (rb, ub) = res
    assert all(abs(x - y) <= 1 for x, y in zip(ra.cg_its[:2], rb.cg_its[:2]))
    same = list(ra.cg_its[:2]) == list(rb.cg_its[:2])
    assert rel(ub, ua) < (1e-10 if same else 1e-8)
