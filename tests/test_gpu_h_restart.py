"""Continuous batching of the 1D batch (fh_h_batch_restart): an instance takes
a new solve between two batch steps while the others go on.  The new
occupant's result after n batch steps equals a fresh n-step solve (oracle)
within the FP64 tolerance, and the other instances are unaffected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O

TOL_SOLVER = 1e-12


def relmax(a, b):
    a, b = np.asarray(a), np.asarray(b)
    den = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (den if den > 0 else 1.0))


@pytest.fixture(scope="module")
def ctx():
    from conftest import torch_ordered_context
    c = torch_ordered_context(0)
    c.set_graphs(False)
    yield c
    c.close()


def _mix():
    from theses_code_gb300 import workloads
    params, U0s = workloads.psi_batch(n=5, seed=9, Nmin=40, Nmax=160, tau=2e-3)
    p1, u1 = workloads.caputo_1d(120, 0.8, 1.0, 1e-3)
    return [p1] + params, [u1] + U0s


@pytest.mark.parametrize("mode_name", ["FH_H_FP64", "FH_H_DF64"])
def test_restart_matches_fresh_solves(ctx, mode_name):
    from theses_code_gb300 import _lib, workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = _mix()
    s = HSolverBatch(ctx, params, 200, getattr(_lib, mode_name))
    s.set_u(U0s)
    s.calc_step(37)
    # instance 2 (psi, N <= 160) becomes an L1 solve with a smaller N;
    # instance 0 (L1, N = 120) becomes a psi solve with D(u) = D0 exp(gamma u)
    pa, ua = workloads.caputo_1d(90, 0.65, 0.5, 1e-3)
    pq, uq = workloads.psi_batch(n=1, seed=21, Nmin=100, Nmax=120, tau=2e-3)
    s.restart(2, pa, ua)
    s.calc_step(11)
    s.restart(0, pq[0], uq[0])
    s.calc_step(52)
    got = s.get_u()
    assert relmax(got[2], O.h_solve(pa, ua, 63)[0]) <= TOL_SOLVER
    assert relmax(got[0], O.h_solve(pq[0], uq[0], 52)[0]) <= TOL_SOLVER
    for k in (1, 3, 4, 5):
        assert relmax(got[k], O.h_solve(params[k], U0s[k], 100)[0]) <= TOL_SOLVER, k
    # a whole-batch state reset puts every instance back on the batch clock
    s.set_u(s.get_u())
    s.close()


def test_restart_twice_and_limits(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_H_BLOCKED, FhError
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = _mix()
    s = HSolverBatch(ctx, params, 120)
    s.set_u(U0s)
    s.calc_step(5)
    pa, ua = workloads.caputo_1d(60, 0.7, 1.0, 1e-3)
    s.restart(4, pa, ua)
    s.calc_step(20)
    pb, ub = workloads.caputo_1d(50, 0.9, 2.0, 1e-3)
    s.restart(4, pb, ub)  # the same slot again
    s.calc_step(30)
    assert relmax(s.get_u()[4], O.h_solve(pb, ub, 30)[0]) <= TOL_SOLVER
    big, ubig = workloads.caputo_1d(params[4]["N"] + 10, 0.7, 1.0, 1e-3)
    with pytest.raises(FhError):
        s.restart(4, big, ubig)  # more nodes than the slot holds
    s.close()
    b = HSolverBatch(ctx, params, 120, FH_H_BLOCKED)
    b.set_u(U0s)
    with pytest.raises(FhError):
        b.restart(1, pa, ua)
    b.close()


def test_persistent_path_matches_kernel_by_kernel(ctx):
    """Small FP64 batches run each call as one launch of clustered CTAs
    (k_h_persistent); the kernel-by-kernel path and the oracle agree with it
    over uneven calls and a restart (mixed L1 / psi = t / psi = t^beta, constant
    and variable coefficients)."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = _mix()
    pt = dict(params[1], beta=1.0)
    params = params + [pt]
    U0s = U0s + [U0s[1]]
    res = []
    for persistent in (True, False):
        s = HSolverBatch(ctx, params, 300)
        s.set_persistent(persistent)
        s.set_u(U0s)
        for n in (1, 40, 7):
            s.calc_step(n)
        pa, ua = workloads.caputo_1d(90, 0.65, 0.5, 1e-3)
        s.restart(3, pa, ua)
        s.calc_step(60)
        res.append(s.get_u())
        s.close()
    for k in range(len(params)):
        if k == 3:
            ref = O.h_solve(pa, ua, 60)[0]
        else:
            ref = O.h_solve(params[k], U0s[k], 108)[0]
        assert relmax(res[0][k], ref) <= TOL_SOLVER, k
        assert relmax(res[0][k], res[1][k]) <= TOL_SOLVER, k
