"""The request server: independent heat and neo-Hookean solves submitted
together run concurrently (their kernels overlap on separate streams), and
every result equals the same request solved alone: same CG and Newton
iteration counts (+-1 CG for round-off in the scatter), solution norms
within 1e-9 relative, watchpoints within 1e-8 relative."""
import numpy as np
import pytest

import mfgpu
import workloads as W

pytestmark = pytest.mark.gpu


def run_all(reqs, workers):
    srv = mfgpu.Server(0, workers, 0.5)
    ids = [srv.submit(r) for r in reqs]
    res = [srv.wait(i) for i in ids]
    max_running, _ = srv.stats()
    srv.close()
    return res, max_running


def test_results_alone_equal_results_in_the_mix(ctx):
    reqs = W.serving_requests(mfgpu, 12, seed=3, max_heat_ref=4, solid_k=(2, 4),
                              degrees=(1, 2, 3))
    alone, mr1 = run_all(reqs, 1)
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
