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
