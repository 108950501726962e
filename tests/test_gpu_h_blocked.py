"""Blocked history mode of the 1D batch (FH_H_BLOCKED): the history slots
older than the current 64-step block contracted on the tensor cores (exact
bf16 slices, one 128-point tile of an instance against its 64 weight rows),
the block's own slots in double-float; against the CPU oracle at the
mixed-precision bound (1e-9 relative max-norm)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O

TOL_MIXED = 1e-9


def relmax(a, b):
    a, b = np.asarray(a), np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def ctx():
    from conftest import torch_ordered_context
    c = torch_ordered_context(0)
    yield c
    c.close()


def test_blocked_psi_batch_vs_oracle(ctx):
    """Ragged psi batch with D(u) = D0 exp(gamma u) over several blocks, as one
    captured solve and as uneven calls."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_H_BLOCKED
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=6, seed=3, Nmin=17, Nmax=300, tau=2e-3)
    steps = 300
    refs = [O.h_solve(p, u, steps)[0] for p, u in zip(params, U0s)]
    a = HSolverBatch(ctx, params, steps + 1, FH_H_BLOCKED)
    a.set_u(U0s)
    a.calc_step(steps)
    b = HSolverBatch(ctx, params, steps + 1, FH_H_BLOCKED)
    b.set_u(U0s)
    for n in (1, 64, 100, 135):
        b.calc_step(n)
    for k, (ga, gb, r) in enumerate(zip(a.get_u(), b.get_u(), refs)):
        assert relmax(ga, r) <= TOL_MIXED, (k, relmax(ga, r))
        assert relmax(gb, ga) <= 1e-13, k
    a.close()
    b.close()


def test_blocked_mixed_weight_kinds(ctx):
    """L1, psi = t and psi = t^beta instances (constant and variable
    coefficients) in one blocked batch, long enough (300 steps) that the
    oldest chunk group of the psi instances is interpolated across the block
    at 256 slots while the L1 instance's is evaluated per step."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_H_BLOCKED
    from theses_code_gb300.solvers import HSolverBatch
    p1, u1 = workloads.caputo_1d(150, 0.8, 1.0, 1e-3)
    params, U0s = workloads.psi_batch(n=3, seed=5, Nmin=40, Nmax=200, tau=2e-3)
    pt = dict(params[0], beta=1.0)
    allp = [p1, pt] + params
    allu = [u1, U0s[0]] + U0s
    steps = 300
    s = HSolverBatch(ctx, allp, steps + 1, FH_H_BLOCKED)
    s.set_u(allu)
    s.calc_step(steps)
    for k, (p, u, g) in enumerate(zip(allp, allu, s.get_u())):
        ref, _ = O.h_solve(p, u, steps)
        assert relmax(g, ref) <= TOL_MIXED, (k, relmax(g, ref))
    s.close()


def test_blocked_mode_limits(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_H_BLOCKED, FH_H_FP64, FhError, check
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=2, seed=3, Nmin=17, Nmax=40, tau=2e-3)
    s = HSolverBatch(ctx, params, 70, FH_H_BLOCKED)
    with pytest.raises(FhError):
        s.autotune()
    s.set_u(U0s)
    s.calc_step(66)
    assert ctx.L.fh_h_batch_set_mode(s.h, FH_H_FP64) != 0  # only before the first step
    # back to FP64 before stepping: the full history is allocated again
    t = HSolverBatch(ctx, params, 70, FH_H_BLOCKED)
    check(ctx.L.fh_h_batch_set_mode(t.h, FH_H_FP64), ctx.h)
    t.set_u(U0s)
    t.calc_step(69)
    ref, _ = O.h_solve(params[1], U0s[1], 69)
    assert relmax(t.get_u()[1], ref) <= 1e-12
    s.close()
    t.close()
