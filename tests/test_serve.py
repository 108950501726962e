"""Serving loop (continuous batching): every request's result equals the same
solve run alone, within the FP64 parity tolerance, although requests share
cohorts and streams and are admitted as memory frees up."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_serving_results_match_solo_runs():
    from theses_code_gb300 import serve
    from theses_code_gb300._lib import Context
    from theses_code_gb300.solvers import HSolverBatch, TGSolver
    reqs = serve.make_mix(14, rate=2000.0, seed=9, max_2d=48, steps=(40, 160), nrange=(40, 300))
    # a budget far below the total forces queueing, cohorts and staggered admission
    total = sum(r.history_bytes() for r in reqs)
    budget = max(max(r.history_bytes() for r in reqs) * 2.0, total / 4.0)
    srv = serve.Server(budget, chunk=37, max_cohort=4, max_active=4)
    done, stats = srv.run(reqs, realtime=True)
    assert stats["requests"] == len(reqs)
    assert stats["p99_s"] >= stats["p50_s"] > 0
    by_id = {d.rid: d for d in done}
    ctx = Context(0)
    for r in reqs:
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
        got = by_id[r.rid].result
        err = np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300)
        assert err <= 1e-12, (r.rid, r.kind, err)
    ctx.close()


def test_request_over_budget_is_rejected():
    from theses_code_gb300 import serve
    reqs = serve.make_mix(2, seed=1, max_2d=64, steps=(50, 60), nrange=(40, 60))
    srv = serve.Server(budget_bytes=1000.0)
    with pytest.raises(ValueError):
        srv.run(reqs)
