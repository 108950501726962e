"""Serving loop (continuous batching): every request's result equals the same
solve run alone, within the FP64 parity tolerance, although requests share
pools and streams, join running pools as slots free up, and are admitted as
memory frees up."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _solo(ctx, r):
    from theses_code_gb300.solvers import HSolverBatch, TGSolver
    if r.kind == "1d":
        s = HSolverBatch(ctx, [r.params], r.steps + 1)
        s.set_u([r.U0])
        s.calc_step(r.steps)
        ref = s.get_u()[0]
    else:
        s = TGSolver(ctx, r.params, r.steps, r.mode)
        s.set_state(r.V2, r.C0)
        s.calc_step(r.steps)
        ref = s.get_c()
    s.close()
    return ref


def _check(reqs, done):
    from theses_code_gb300._lib import Context
    by_id = {d.rid: d for d in done}
    ctx = Context(0)
    for r in reqs:
        ref = _solo(ctx, r)
        got = by_id[r.rid].result
        err = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300)
        assert err <= 1e-12, (r.rid, r.kind, err)
    ctx.close()


@pytest.mark.parametrize("mode_2d", ["FH_TG_FP64", "FH_TG_BLOCKED"])
def test_serving_results_match_solo_runs(mode_2d):
    from theses_code_gb300 import _lib, serve
    reqs = serve.make_mix(16, rate=2000.0, seed=9, max_2d=48, steps=(40, 160), nrange=(40, 300),
                          mode_2d=getattr(_lib, mode_2d))
    # a budget far below the total forces queueing and staggered admission
    total = sum(r.device_bytes() for r in reqs)
    budget = max(max(r.device_bytes() for r in reqs) * 4.0, total / 3.0)
    srv = serve.Server(budget, chunk=37, max_pool=4, max_active=4, min_slots=4)
    done, stats = srv.run(reqs, realtime=True)
    assert stats["requests"] == len(reqs)
    assert stats["p99_s"] >= stats["p50_s"] > 0
    assert stats["peak_device_bytes"] <= budget
    _check(reqs, done)


def test_requests_join_running_pools():
    """1D requests arriving while a pool runs take its free slots (spares and
    slots of finished requests) instead of waiting for the pool to end."""
    from theses_code_gb300 import serve
    reqs = serve.make_mix(24, rate=400.0, seed=4, steps=(30, 90), nrange=(40, 200), frac_2d=0.0)
    srv = serve.Server(1e12, chunk=15, max_pool=3, max_active=2, min_slots=6, step_factor=4.0)
    done, stats = srv.run(reqs, realtime=False)
    assert stats["requests"] == len(reqs)
    assert stats["joined_running_pools"] > 0
    _check(reqs, done)


SLACK = 2 << 20  # the estimates' allowance for allocation granularity


def test_byte_estimates_bound_the_allocations():
    from theses_code_gb300 import _lib, serve, workloads
    from theses_code_gb300._lib import Context
    from theses_code_gb300.solvers import HSolverBatch, TGSolver
    ctx = Context(0)
    for caps, steps in (([64, 128, 2048], 500), ([40] * 10, 70), ([1024], 5000)):
        s = HSolverBatch(ctx, [dict(workloads.caputo_1d(c - 1)[0]) for c in caps], steps)
        got, est = s.device_bytes(), serve.pool_bytes(caps, steps)
        assert 0.7 * (est - SLACK) <= got <= est, (caps, steps, got, est)
        s.close()
    for g, steps, mode in ((64, 500, _lib.FH_TG_FP64), (200, 300, _lib.FH_TG_BLOCKED), (96, 60, _lib.FH_TG_BLOCKED),
                           (128, 5000, _lib.FH_TG_FP64)):
        p, V2, C0 = workloads.convection_2d(g, g, alpha=0.7, tau=5e-4, d=0.1, seed=1)
        s = TGSolver(ctx, p, steps, mode)
        got, est = s.device_bytes(), serve.tg_bytes(g, g, steps, mode)
        assert 0.7 * (est - SLACK) <= got <= est, (g, steps, mode, got, est)
        s.close()
    ctx.close()


def test_request_over_budget_is_rejected():
    from theses_code_gb300 import serve
    reqs = serve.make_mix(2, seed=1, max_2d=64, steps=(50, 60), nrange=(40, 60))
    srv = serve.Server(budget_bytes=1000.0)
    with pytest.raises(ValueError):
        srv.run(reqs)
