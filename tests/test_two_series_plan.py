"""The host bookkeeping of the two-series approximation (dt_alg 4), CPU only:
the library's planned item tables (fh_tg_two_series_plan), executed here in
numpy the way the device kernel executes them, reproduce the oracle's per-node
calc_va sums (a restatement checked bit for bit against the reference)."""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O

MAXAK = 20


def plan(alpha, max_steps):
    from theses_code_gb300._lib import load
    L = load()
    ns = (C.c_int * 2)()
    dt = (C.c_double * 2)()
    ni, nc = C.c_int(0), C.c_int(0)
    assert L.fh_tg_two_series_plan(alpha, max_steps, ns, dt, C.byref(ni), None, C.byref(nc), None, None) == 0
    items = np.zeros((ni.value, 4), dtype=np.int32)
    coef = np.zeros(max(nc.value, 1))
    spans = np.zeros((2 * (max_steps + 1), 4), dtype=np.int32)
    assert L.fh_tg_two_series_plan(alpha, max_steps, ns, dt, C.byref(ni), items.ctypes.data_as(C.c_void_p),
                                   C.byref(nc), coef.ctypes.data_as(C.c_void_p),
                                   spans.ctypes.data_as(C.c_void_p)) == 0
    return list(ns), list(dt), items, coef, spans


def run_plan(alpha, steps, F):
    """F[r][p], r = 0..steps: the sums V[j][p] of steps j = 1..steps - 1."""
    ns, dterm, items, coef, spans = plan(alpha, steps)
    P = F.shape[1]
    out = np.zeros((2, steps, P))
    for d in range(2):
        c = np.full((ns[d] + 1, MAXAK, P), np.nan)  # unset coefficients poison the sums
        for j in range(1, steps):
            b, e, z, _ = spans[2 * j + d]
            Fj = F[j]
            V = np.zeros(P)
            for k, s_, src, off in items[b:e]:
                nt = k >> 8
                r = np.zeros(P)
                for i in range(nt):
                    r = r + c[s_, i] * coef[off + i]
                V = V + r
            out[d, j] = V + dterm[d] * Fj
            for k, s_, src, off in items[e:z]:
                kind, nt = k & 0xff, k >> 8
                if kind == 1:
                    c[s_] = c[src]
                    continue
                i0 = 1 if kind in (2, 4) else 0
                if kind >= 4:
                    c[s_, :] = 0.0
                for i in range(i0, nt):
                    v = coef[off + i] * (Fj * coef[off + nt + i])
                    c[s_, i] = c[s_, i] + v if kind in (2, 3) else v
    return out


@pytest.mark.parametrize("alpha,steps", [(0.7, 160), (0.3, 90), (0.95, 120)])
def test_plan_reproduces_oracle_sums(alpha, steps):
    rng = np.random.default_rng(5)
    P = 3
    F = rng.normal(size=(steps + 1, P))
    F[0] = 0.0
    got = run_plan(alpha, steps, F)
    Vx = np.zeros((steps + 1) * P)
    Vy = np.zeros((steps + 1) * P)
    Fc = np.ascontiguousarray(F)
    assert O.lib().fho_two_series_sums(C.c_double(alpha), steps, P, Fc.ctypes.data_as(C.c_void_p),
                                       Vx.ctypes.data_as(C.c_void_p), Vy.ctypes.data_as(C.c_void_p)) == 0
    Vx = Vx.reshape(steps + 1, P)
    Vy = Vy.reshape(steps + 1, P)
    for d, V in ((0, Vx), (1, Vy)):
        assert np.all(np.isfinite(got[d, 1:]))
        # the same operations in the same order: equal bit for bit
        assert np.array_equal(got[d, 1:], V[1:steps]), d


def test_plan_limits():
    from theses_code_gb300._lib import load
    L = load()
    ns = (C.c_int * 2)()
    dt = (C.c_double * 2)()
    ni, nc = C.c_int(0), C.c_int(0)
    assert L.fh_tg_two_series_plan(1.0, 10, ns, dt, C.byref(ni), None, C.byref(nc), None, None) != 0
    assert L.fh_tg_two_series_plan(0.5, 0, ns, dt, C.byref(ni), None, C.byref(nc), None, None) != 0
    ns2, _, items, _, _ = plan(0.6, 400)
    assert 10 < ns2[0] < 120 and 10 < ns2[1] < 120
