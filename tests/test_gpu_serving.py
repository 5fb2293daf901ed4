"""The request server: independent heat and neo-Hookean solves submitted
together run concurrently (their kernels overlap on separate streams, and
heat requests of one shape are solved as one batch), and every result
equals the same request solved alone: same CG and Newton iteration counts
(+-1 CG for round-off in the scatter), solution norms within 1e-9 relative,
watchpoints within 1e-8 relative."""
import numpy as np
import pytest

import mfgpu
import workloads as W

pytestmark = pytest.mark.gpu


def run_all(reqs, workers, max_batch=None):
    """All requests submitted at once; max_batch 1 solves each alone."""
    srv = mfgpu.Server(0, workers, 0.5)
    if max_batch is not None:
        srv.set_max_batch(max_batch)
    ids = [srv.submit(r) for r in reqs]
    res = [srv.wait(i) for i in ids]
    max_running, _ = srv.stats()
    srv.close()
    return res, max_running


@pytest.mark.parametrize("emulation", [True, False], ids=["df64_operators", "native_fp64_operators"])
def test_results_alone_equal_results_in_the_mix(ctx, emulation):
    """The FP64 operators of the mixed-precision solver in native FP64 (the
    serving default) and in double-float."""
    reqs = W.serving_requests(mfgpu, 12, seed=3, max_heat_ref=4, solid_k=(2, 4),
                              degrees=(1, 2, 3), fp64_emulation=emulation)
    alone, mr1 = run_all(reqs, 1, max_batch=1)
    mix, mr4 = run_all(reqs, 4)
    assert mr1 == 1
    assert mr4 > 1, "requests did not overlap"
    for a, b, r in zip(alone, mix, reqs):
        assert a.status == 0, a.message
        assert b.status == 0, b.message
        assert abs(a.cg_iterations - b.cg_iterations) <= 1
        assert a.newton_iterations == b.newton_iterations
        assert abs(a.solution_norm - b.solution_norm) <= 1e-9 * abs(a.solution_norm)
        if r.kind == 1:
            wa, wb = np.array(a.watch[:3]), np.array(b.watch[:3])
            assert np.linalg.norm(wa - wb) <= 1e-8 * np.linalg.norm(wa)


def test_request_errors_are_reported_per_request(ctx):
    reqs = W.serving_requests(mfgpu, 2, seed=5, max_heat_ref=3, solid_k=(2,), degrees=(1,))
    bad = W.serving_requests(mfgpu, 1, seed=9, max_heat_ref=3, solid_k=(2,), degrees=(1,))[0]
    bad.kind = 1
    bad.solid.caching = b"no_such_caching"
    srv = mfgpu.Server(0, 2, 0.5)
    ids = [srv.submit(r) for r in reqs] + [srv.submit(bad)]
    res = [srv.wait(i) for i in ids]
    srv.close()
    assert res[0].status == 0 and res[1].status == 0
    assert res[2].status == 1 and b"caching" in res[2].message


def test_resident_problems_are_reused_with_the_same_results(ctx):
    """A worker keeps the problems it solved: a second request of the same
    shape (another source or traction) reuses the driver, and the result
    equals that of a fresh server solving the request alone."""
    reqs = W.serving_requests(mfgpu, 6, seed=11, max_heat_ref=4, solid_k=(2,), degrees=(2,))
    # two rounds of the same shapes: the second round's loads differ
    again = W.serving_requests(mfgpu, 6, seed=12, max_heat_ref=4, solid_k=(2,), degrees=(2,))
    srv = mfgpu.Server(0, 1, 0.5)
    first = [srv.wait(srv.submit(r)) for r in reqs]
    assert srv.pool_stats()[0] >= 0
    built_before = srv.pool_stats()[1]
    # the same requests once more: every shape is resident now
    second = [srv.wait(srv.submit(r)) for r in reqs]
    reused, built = srv.pool_stats()
    assert built == built_before and reused >= len(reqs)
    srv.close()
    for a, b in zip(first, second):
        assert a.status == 0 and b.status == 0
        assert abs(a.cg_iterations - b.cg_iterations) <= 1
        assert a.newton_iterations == b.newton_iterations
        assert abs(a.solution_norm - b.solution_norm) <= 1e-9 * abs(a.solution_norm)
    # other loads on resident shapes equal a fresh server's results
    srv = mfgpu.Server(0, 1, 0.5)
    for r in reqs:
        srv.wait(srv.submit(r))
    pooled = [srv.wait(srv.submit(r)) for r in again]
    srv.close()
    fresh, _ = run_all(again, 1, max_batch=1)
    for a, b in zip(pooled, fresh):
        assert a.status == 0 and b.status == 0
        assert abs(a.cg_iterations - b.cg_iterations) <= 1
        assert a.newton_iterations == b.newton_iterations
        assert abs(a.solution_norm - b.solution_norm) <= 1e-9 * abs(a.solution_norm)


def _heat_request(degree, n_ref, seed, n_steps=1):
    r = mfgpu.Request()
    r.kind = 0
    hp = r.heat
    hp.mesh = W.to_lib_mesh(mfgpu, W.unit_cube_heat(degree, n_ref))
    hp.dt, hp.n_steps = 0.1, n_steps
    hp.solver = mfgpu.solver_params("gmg", tol=1e-8, cheb_range=15.0, cheb_eig_its=10, mg_precision=32,
                                    coarse_fp64=True)
    c, w, a = W.gaussian_source(seed)
    hp.n_gauss = 8
    for j in range(8):
        for d in range(3):
            hp.g_center[j][d] = c[j, d]
        hp.g_width[j] = w[j]
        hp.g_amp[j] = a[j]
    return r


@pytest.mark.parametrize("degree,n_ref", [(2, 3), (3, 4), (1, 5)])
def test_batched_heat_requests_equal_their_solo_solves(ctx, degree, n_ref):
    """Continuous batching: heat requests of one shape queued behind a busy
    worker are solved together (one operator, V-cycle and CG over all of
    them); each result equals the request solved alone.  The 32^3-cell Q1
    case runs its finest FP32 level through the register form of the
    tensor-product heat kernel, the others through the block form."""
    heat = [_heat_request(degree, n_ref, seed) for seed in (31, 32, 33, 34)]
    # a solid request keeps the single worker busy while the heat requests queue
    blocker = next(r for r in W.serving_requests(mfgpu, 30, seed=5, max_heat_ref=3, solid_k=(8,), degrees=(3,))
                   if r.kind == 1)
    srv = mfgpu.Server(0, 1, 0.5)
    ids = [srv.submit(blocker)] + [srv.submit(r) for r in heat]
    batched = [srv.wait(i) for i in ids][1:]
    n_batched, largest = srv.batch_stats()
    srv.close()
    assert n_batched >= 2 and largest >= 2, (n_batched, largest)
    solo_srv = mfgpu.Server(0, 1, 0.5)
    solo_srv.set_max_batch(1)
    solo = [solo_srv.wait(solo_srv.submit(r)) for r in heat]
    assert solo_srv.batch_stats() == (0, 1)
    solo_srv.close()
    for a, b in zip(solo, batched):
        assert a.status == 0, a.message
        assert b.status == 0, b.message
        assert abs(a.cg_iterations - b.cg_iterations) <= 1, (a.cg_iterations, b.cg_iterations)
        assert abs(a.solution_norm - b.solution_norm) <= 1e-9 * abs(a.solution_norm)
        assert a.n_dofs == b.n_dofs
    # the problems differ: the batch did not hand one result to all
    norms = [b.solution_norm for b in batched]
    assert len(set(norms)) == len(norms)


def _oracle_heat(spec, seed, tol):
    import oracle as O
    po = O.HeatParams()
    po.mesh = W.to_oracle_mesh(O, spec)
    po.dt, po.n_steps, po.tol_rel, po.precond = 0.1, 1, tol, 2
    po.mg_float = 0
    c, w, a = W.gaussian_source(seed)
    po.n_gauss = 8
    for j in range(8):
        for d in range(3):
            po.g_center[j][d] = c[j, d]
        po.g_width[j] = w[j]
        po.g_amp[j] = a[j]
    return O.heat_run(po, return_u=True)


def _oracle_solid(spec, traction, tol):
    import oracle as O
    po = O.SolidParams()
    po.mesh = W.to_oracle_mesh(O, spec)
    po.mat = O.material(0.5e6, 0.4, 1000.0, 0.01, 1)
    po.caching = O.CACHING["scalar_referential"]
    po.precond, po.relaxation, po.tol_lin, po.max_it_mult, po.max_newton = 2, 0.65, tol, 1, 10
    po.tol_f, po.tol_f_abs, po.tol_u, po.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
    po.dt, po.n_steps = 0.01, 1
    po.body_force[:] = [0.0, 0.0, 0.0]
    po.traction_id = W.TRACTION_ID
    po.traction[:] = list(traction)
    po.watch[:] = [8.0, 0.5, 0.5]
    po.cheb_degree, po.cheb_range, po.cheb_eig_its, po.coarse_accurate = 5, 20.0, 30, 1
    po.mg_float = 0
    return O.solid_run(po)


def test_served_results_match_the_oracle(ctx):
    """Requests served concurrently against the oracle's FP64 solves of the
    same problems: heat steps (solution norm within 1e-7 relative, CG within
    +-1) and Newton-Newmark steps (Newton iterations equal, watchpoint within
    1e-6 relative), FP32-GMG preconditioned FP64 CG to 1e-8 on the server,
    all-FP64 GMG-CG in the oracle (heat_transfer.h:715-754,
    mf_elasticity.h:1402-1491)."""
    import oracle as O
    tol = 1e-8
    heat = [(W.unit_cube_heat(1, 4), 41), (W.unit_cube_heat(2, 3), 42)]
    solid = [(W.cantilever(1, 1), (0.0, -80.0, 0.0)), (W.cantilever(2, 1), (0.0, -120.0, 0.0))]
    reqs = []
    for spec, seed in heat:
        r = mfgpu.Request()
        r.kind = 0
        hp = r.heat
        hp.mesh = W.to_lib_mesh(mfgpu, spec)
        hp.dt, hp.n_steps = 0.1, 1
        hp.solver = mfgpu.solver_params("gmg", tol=tol, cheb_range=15.0, cheb_eig_its=10, mg_precision=32,
                                        coarse_fp64=True)
        c, w, a = W.gaussian_source(seed)
        hp.n_gauss = 8
        for j in range(8):
            for d in range(3):
                hp.g_center[j][d] = c[j, d]
            hp.g_width[j] = w[j]
            hp.g_amp[j] = a[j]
        reqs.append(r)
    for spec, traction in solid:
        r = mfgpu.Request()
        r.kind = 1
        sp = r.solid
        sp.mesh = W.to_lib_mesh(mfgpu, spec)
        sp.material = mfgpu.material(0.5e6, 0.4, 1000.0, 0.01)
        sp.caching = b"referential_qp"
        sp.solver = mfgpu.solver_params("gmg", tol=tol, mg_precision=32, coarse_fp64=True)
        sp.max_newton = 10
        sp.tol_f, sp.tol_f_abs, sp.tol_u, sp.tol_u_abs = 1e-9, 0.0, 1e-6, 0.0
        sp.dt, sp.n_steps = 0.01, 1
        sp.traction_id = W.TRACTION_ID
        sp.traction[:] = list(traction)
        sp.watch[:] = [8.0, 0.5, 0.5]
        reqs.append(r)
    res, max_running = run_all(reqs, 4)
    assert max_running > 1
    for (spec, seed), r in zip(heat, res[:2]):
        assert r.status == 0, r.message
        ro, uo = _oracle_heat(spec, seed, tol)
        assert abs(r.solution_norm - np.linalg.norm(uo)) <= 1e-7 * np.linalg.norm(uo)
        assert abs(r.cg_iterations - ro.cg_its[0]) <= 1, (r.cg_iterations, ro.cg_its[0])
    for (spec, traction), r in zip(solid, res[2:]):
        assert r.status == 0, r.message
        ro = _oracle_solid(spec, traction, tol)
        assert r.newton_iterations == ro.newton_its[0]
        wo = np.array(ro.watch_disp[0][:3])
        assert np.linalg.norm(np.array(r.watch[:3]) - wo) <= 1e-6 * np.linalg.norm(wo)
