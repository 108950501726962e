"""GPU parity: every libfhist entry point against the CPU oracle and the
reference golden vectors.  FP64 tolerance (the plain path's contract):
relative max-norm <= 1e-12 for solver states, tighter for primitives."""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O

G = os.path.join(os.path.dirname(__file__), "golden")
TOL_SOLVER = 1e-12


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


@pytest.fixture(scope="module")
def torch_mod():
    import torch
    return torch


def dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device="cuda")


# ------------------------------------------------------------------ weights
@pytest.mark.parametrize("alpha,beta", [(0.7, 1.0), (0.3, 1.0), (0.95, 1.0), (0.6, 0.5), (0.8, 2.0),
                                        (0.55, 1.37), (0.9, 0.75)])
def test_weights_psi(ctx, torch_mod, alpha, beta):
    torch = torch_mod
    for X, tau in [(7.0, 1e-3), (500.5, 5e-4), (4001.0, 1e-2)]:
        K = int(X - 1.0)
        w = torch.zeros(K, dtype=torch.float64, device="cuda")
        ctx.call("fh_weights_psi", K, 0.0, 1.0, X, tau, alpha, beta, 2.5, w.data_ptr())
        ctx.sync()
        got = w.cpu().numpy()
        ref = np.array([2.5 * O.psi_int(k, k + 1.0, X, tau, alpha, beta) for k in range(K)])
        # psi = t: the reference's closed form subtracts nearly equal powers, so
        # a 1-ulp pow difference (CUDA vs glibc) grows to ~eps * X / (1 - alpha)
        # relative; beta != 1: the divided-difference form holds a few ulps
        tol = max(1e-13, 4e-16 * X / (1 - alpha)) if beta == 1.0 else 1e-14
        assert np.all(np.abs(got - ref) <= tol * np.abs(ref)), (X, np.max(np.abs(got - ref) / np.abs(ref)))


def test_weights_l1(ctx, torch_mod):
    torch = torch_mod
    for os_ in (0, 1, 2, 3, 1000):
        w = torch.zeros(max(os_, 1), dtype=torch.float64, device="cuda")
        ctx.call("fh_weights_l1", os_, 0.8, w.data_ptr())
        ctx.sync()
        got = w.cpu().numpy()[:max(os_ - 1, 0)]
        ref = np.array([O.l1_b(os_ - t - 1, 0.8) for t in range(os_ - 1)])
        # (k+1)^0.2 - k^0.2 cancels: 1-ulp pow differences grow like eps * k / (1 - alpha)
        lag = np.arange(os_ - 1, 0, -1, dtype=float)
        assert np.all(np.abs(got - ref) <= 4e-16 * np.maximum(lag, 1.0) / 0.2 * np.abs(ref))


def test_weights_ab(ctx, torch_mod):
    torch = torch_mod
    for alpha, tau, n in [(0.6, 1e-4, 3000), (0.5, 0.01, 50), (0.3, 1e-3, 800)]:
        w = torch.zeros(n + 1, dtype=torch.float64, device="cuda")
        ctx.call("fh_weights_ab", n, tau, alpha, w.data_ptr())
        ctx.sync()
        got = w.cpu().numpy()
        lags = [1, 2, 3, 10, n // 2, n - 1, n]
        for lag in lags:
            ref = O.ab_int(lag, tau, alpha)
            assert abs(got[lag] - ref) <= 1e-12 * abs(ref), (alpha, lag, got[lag], ref)
        assert got[0] == got[1]


def test_weights_ab_reference_golden(ctx, torch_mod):
    """Lag weights against the reference MF_int_choice series (lags the history uses)."""
    torch = torch_mod
    g = json.load(open(os.path.join(G, "ab.json")))["abw"]
    n = g["n"]
    w = torch.zeros(n + 1, dtype=torch.float64, device="cuda")
    ctx.call("fh_weights_ab", n, g["tau"], g["alpha"], w.data_ptr())
    ctx.sync()
    got = w.cpu().numpy()
    for lag, val in g["w"]:
        if lag >= 2:
            assert abs(got[lag] - val) <= 1e-12 * abs(val)


def test_mittag_leffler(ctx, torch_mod):
    torch = torch_mod
    g = json.load(open(os.path.join(G, "ab.json")))["ml"]
    for a, b, z, val in g:
        zz = dev(torch, [z])
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        ctx.call("fh_mittag_leffler", 1, a, b, zz.data_ptr(), out.data_ptr())
        ctx.sync()
        assert abs(out.item() - val) <= 2e-14 * abs(val)
    zs = np.linspace(-3, 1, 41)
    zz = dev(torch, zs)
    out = torch.zeros(41, dtype=torch.float64, device="cuda")
    ctx.call("fh_mittag_leffler", 41, 1.0, 1.0, zz.data_ptr(), out.data_ptr())
    ctx.sync()
    assert relmax(out.cpu().numpy(), np.exp(zs)) < 1e-14


# ------------------------------------------------------------------ history
@pytest.mark.parametrize("M", [1, 2])
@pytest.mark.parametrize("K,P", [(0, 64), (1, 2), (5, 130), (137, 1000), (2049, 4096), (40001, 64)])
def test_history_sum(ctx, torch_mod, M, K, P):
    """(40001, 64): 16 splits of 2504 layers, each walked in two weight stages."""
    torch = torch_mod
    rng = np.random.default_rng(K * 7 + P + M)
    D = rng.normal(size=(max(K, 1), P))
    W = rng.uniform(0.1, 1.0, size=(M, max(K, 1)))
    Dd, Wd = dev(torch, D), dev(torch, W)
    S = torch.full((M, P), 7.0, dtype=torch.float64, device="cuda")
    ctx.call("fh_history_sum", M, K, P, Wd.data_ptr(), W.shape[1], Dd.data_ptr(), P, S.data_ptr(), P)
    ctx.sync()
    ref = W[:, :K] @ D[:K] if K > 0 else np.zeros((M, P))
    scale = np.abs(W[:, :K]) @ np.abs(D[:K]) if K > 0 else np.ones((M, P))
    assert np.all(np.abs(S.cpu().numpy() - ref) <= 1e-14 * np.maximum(scale, 1e-300) * max(K, 1) ** 0.5 + 0.0)


def test_history_sum_rejects_odd_and_misaligned(ctx, torch_mod):
    torch = torch_mod
    from theses_code_gb300._lib import FhError
    D = torch.zeros(10, dtype=torch.float64, device="cuda")
    W = torch.ones(2, dtype=torch.float64, device="cuda")
    S = torch.zeros(10, dtype=torch.float64, device="cuda")
    with pytest.raises(FhError):
        ctx.call("fh_history_sum", 1, 2, 3, W.data_ptr(), 2, D.data_ptr(), 4, S.data_ptr(), 4)
    with pytest.raises(FhError):
        ctx.call("fh_history_sum", 3, 2, 4, W.data_ptr(), 2, D.data_ptr(), 4, S.data_ptr(), 4)


@pytest.mark.parametrize("K,P,ldh", [(41, 333, 333), (0, 17, 17), (5000, 700, 704), (129, 100000, 100000)])
def test_history_sum_layers(ctx, torch_mod, K, P, ldh):
    """One split (few layers or many points) and K splits added in split
    order (few points, long history), strided layers."""
    torch = torch_mod
    rng = np.random.default_rng(3)
    H = rng.normal(size=(K + 1, ldh))
    w = rng.uniform(size=max(K, 1))
    S = torch.full((P,), 7.0, dtype=torch.float64, device="cuda")
    wd, Hd = dev(torch, w), dev(torch, H)  # keep the device buffers alive until the kernel ran
    ctx.call("fh_history_sum_layers", K, P, wd.data_ptr(), Hd.data_ptr(), ldh, S.data_ptr())
    ctx.sync()
    ref = O.history_sum_layers(H[:, :P], w[:K]) if K > 0 else np.zeros(P)
    got = S.cpu().numpy()
    assert (np.max(np.abs(got)) == 0.0) if K == 0 else relmax(got, ref) < 1e-13


# ------------------------------------------------------------- tridiagonal
@pytest.mark.parametrize("N,right_mode", [(1, 0), (2, 1), (37, 0), (513, 1)])
def test_tridiag_batched(ctx, torch_mod, N, right_mode):
    torch = torch_mod
    rng = np.random.default_rng(N)
    nsys = 5
    A = rng.uniform(0.2, 1.0, (nsys, N + 1))
    B = rng.uniform(0.2, 1.0, (nsys, N + 1))
    B[:, 3 % (N + 1)] = 0.0  # exercise the zero-B branch
    R = A + B + rng.uniform(0.1, 1.0, (nsys, N + 1))
    Om = rng.normal(size=(nsys, N + 1))
    al1 = rng.uniform(0, 1, nsys)
    bt1 = rng.normal(size=nsys)
    ur = rng.normal(size=nsys)
    u = torch.zeros((nsys, N + 2), dtype=torch.float64, device="cuda")
    t = [dev(torch, x) for x in (A, R, B, Om, al1, bt1, ur)]
    ctx.call("fh_tridiag_batched", nsys, N, t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(),
             N + 1, t[4].data_ptr(), t[5].data_ptr(), right_mode, t[6].data_ptr(), u.data_ptr(), N + 2)
    ctx.sync()
    got = u.cpu().numpy()
    for s in range(nsys):
        ref = O.thomas(A[s], R[s], B[s], Om[s], al1[s], bt1[s], right_mode, ur[s], np.zeros(N + 2))
        assert relmax(got[s], ref) < 1e-13


@pytest.mark.parametrize("n", [1, 2, 5, 64, 513, 2048])
def test_pcr(ctx, torch_mod, n):
    torch = torch_mod
    rng = np.random.default_rng(n)
    nsys = 3
    a = rng.uniform(-1, 1, (nsys, n))
    c = rng.uniform(-1, 1, (nsys, n))
    b = np.abs(a) + np.abs(c) + rng.uniform(0.5, 1.5, (nsys, n))
    d = rng.normal(size=(nsys, n))
    x = torch.zeros((nsys, n), dtype=torch.float64, device="cuda")
    t = [dev(torch, v) for v in (a, b, c, d)]
    ctx.call("fh_pcr_solver", *[v.data_ptr() for v in t], x.data_ptr(), n, nsys)
    ctx.sync()
    got = x.cpu().numpy()
    for s in range(nsys):
        Mx = np.diag(b[s]) + np.diag(a[s, 1:], -1) + np.diag(c[s, :-1], 1)
        assert relmax(got[s], np.linalg.solve(Mx, d[s])) < 1e-12


# ---------------------------------------------------------------- 1D solver
@pytest.mark.parametrize("name,weights,beta", [("h_minimal_l1.json", 0, 1.0), ("h_psi_t.json", 1, 1.0),
                                               ("h_psi_t07.json", 1, 0.7), ("h_psi_t15.json", 1, 1.5)])
def test_h_solver_reference_golden(ctx, name, weights, beta):
    from theses_code_gb300.solvers import HSolverBatch
    g = json.load(open(os.path.join(G, name)))
    N = g["N"]
    p = dict(N=N, L=g["L"], tau=g["tau"], alpha=g["alpha"], weights=weights, beta=beta, kmodel=0,
             kc=g["k"], kgam=0.0, cinv=20.0, gravity=1, al_left=1.0, bt_left=-g["uc"], u_right=g["Hbottom"])
    U0 = np.zeros(N + 2)
    U0[:N + 1] = g["U0"]
    s = HSolverBatch(ctx, [p, p], g["steps"] + 1)
    s.set_u([U0, U0])
    s.calc_step(g["steps"])
    u = s.get_u()
    assert relmax(u[0], g["U"]) <= TOL_SOLVER
    assert np.array_equal(u[0], u[1])


@pytest.mark.parametrize("name,weights,beta", [("h_minimal_space.json", 0, 1.0), ("h_psi_space.json", 1, 1.0),
                                               ("h_psi_t07_space.json", 1, 0.7)])
def test_h_solver_space_fractional_reference_golden(ctx, name, weights, beta):
    """gamma < 1 (the calc_v term) against the reference runs; the second
    instance of the batch stays classical (gamma = 1)."""
    from theses_code_gb300.solvers import HSolverBatch
    g = json.load(open(os.path.join(G, name)))
    N = g["N"]
    p = dict(N=N, L=g["L"], tau=g["tau"], alpha=g["alpha"], weights=weights, beta=beta, kmodel=0,
             kc=g["k"], kgam=0.0, cinv=20.0, gravity=1, al_left=1.0, bt_left=-g["uc"], u_right=g["Hbottom"])
    U0 = np.zeros(N + 2)
    U0[:N + 1] = g["U0"]
    s = HSolverBatch(ctx, [p, p], g["steps"] + 1)
    s.set_space_order([g["extra"][3], 1.0])
    s.set_u([U0, U0])
    s.calc_step(g["steps"])
    u = s.get_u()
    assert relmax(u[0], g["U"]) <= TOL_SOLVER
    ref1, _ = O.h_solve(p, U0, g["steps"])
    assert relmax(u[1], ref1) <= TOL_SOLVER


@pytest.mark.parametrize("mode", [0, 1])  # FH_H_FP64, FH_H_DF64
def test_h_solver_space_fractional_batch_vs_oracle(ctx, mode):
    """Ragged psi batch (D(u) = D0 exp(gamma u)) with mixed space orders."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=6, seed=3, Nmin=17, Nmax=300, tau=2e-3)
    gam = [0.55, 1.0, 0.8, 0.95, 1.0, 0.65]
    steps = 60
    s = HSolverBatch(ctx, params, steps + 1, mode)
    s.set_space_order(gam)
    s.set_u(U0s)
    s.calc_step(steps)
    for p, U0, gm, got in zip(params, U0s, gam, s.get_u()):
        ref, _ = O.h_solve(dict(p, gamma=gm), U0, steps)
        assert relmax(got, ref) <= TOL_SOLVER, (p["alpha"], p["beta"], gm)


def test_h_solver_space_order_limits(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FhError
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=2, seed=3, Nmin=17, Nmax=40, tau=2e-3)
    s = HSolverBatch(ctx, params, 5)
    for bad in ([0.0, 1.0], [1.2, 1.0], [float("nan"), 1.0]):
        with pytest.raises(FhError):
            s.set_space_order(bad)
    big = dict(params[0], N=3000)
    with pytest.raises(FhError):
        HSolverBatch(ctx, [big], 5).set_space_order([0.7])
    s.set_space_order([0.7, 1.0])
    s.set_u(U0s)
    s.calc_step(1)
    with pytest.raises(FhError):  # only before the first step
        s.set_space_order([1.0, 1.0])


def test_h_solver_caputo_1d_vs_oracle(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    p, U0 = workloads.caputo_1d(200, 0.8, 1.0, 1e-3)
    steps = 300
    s = HSolverBatch(ctx, [p], steps + 1)
    s.set_u([U0])
    s.calc_step(steps)
    ref, _ = O.h_solve(p, U0, steps)
    assert relmax(s.get_u()[0], ref) <= TOL_SOLVER


def test_h_solver_psi_batch_vs_oracle(ctx):
    """Ragged batch of psi-Caputo instances with D(u) = D0 exp(gamma u): each
    instance matches the oracle run alone."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=6, seed=3, Nmin=17, Nmax=90, tau=2e-3)
    steps = 60
    s = HSolverBatch(ctx, params, steps + 1)
    s.set_u(U0s)
    s.calc_step(steps)
    got = s.get_u()
    for p, U0, g in zip(params, U0s, got):
        ref, _ = O.h_solve(p, U0, steps)
        assert relmax(g, ref) <= TOL_SOLVER, (p["alpha"], p["beta"])


def test_h_solver_psi_long_run_vs_oracle(ctx):
    """600 steps of two psi instances (the weights' cancellation grows with the
    step number): one call (captured graph, next-step weights on the side
    stream) and uneven calls (no graph, the first step of each call computes
    its own weights) both match the oracle to the plain-path bound."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=2, seed=3, Nmin=17, Nmax=40, tau=2e-3)
    steps = 600
    a = HSolverBatch(ctx, params, steps + 1)
    a.set_u(U0s)
    a.calc_step(steps)
    b = HSolverBatch(ctx, params, steps + 1)
    b.set_u(U0s)
    for n in (1, 250, 349):
        b.calc_step(n)
    for p, U0, ga, gb in zip(params, U0s, a.get_u(), b.get_u()):
        ref, _ = O.h_solve(p, U0, steps)
        assert relmax(ga, ref) <= TOL_SOLVER, (p["alpha"], p["beta"])
        assert relmax(gb, ga) <= 1e-14


def test_h_solver_warp_and_cta_line_paths(ctx):
    """Batches of 152 instances or more solve one instance per warp, smaller
    ones one instance per CTA: both match the oracle, and each other."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=160, seed=11, Nmin=17, Nmax=60, tau=2e-3)
    steps = 40
    big = HSolverBatch(ctx, params, steps + 1)   # warp per instance
    big.set_u(U0s)
    big.calc_step(steps)
    small = HSolverBatch(ctx, params[:8], steps + 1)  # CTA per instance
    small.set_u(U0s[:8])
    small.calc_step(steps)
    gb, gs = big.get_u(), small.get_u()
    for k in (0, 3, 7, 159):
        ref, _ = O.h_solve(params[k], U0s[k], steps)
        assert relmax(gb[k], ref) <= TOL_SOLVER, k
    for k in range(8):
        assert relmax(gs[k], gb[k]) <= 1e-13, k


def test_h_solver_df64_history_vs_oracle(ctx):
    """History stored as (hi, lo) FP32 pairs and summed in double-float: the
    plain-path bound still holds for the L1 and the psi batch."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_H_DF64
    from theses_code_gb300.solvers import HSolverBatch
    p, U0 = workloads.caputo_1d(200, 0.8, 1.0, 1e-3)
    s = HSolverBatch(ctx, [p], 301, FH_H_DF64)
    s.set_u([U0])
    s.calc_step(300)
    ref, _ = O.h_solve(p, U0, 300)
    assert relmax(s.get_u()[0], ref) <= TOL_SOLVER
    params, U0s = workloads.psi_batch(n=6, seed=3, Nmin=17, Nmax=90, tau=2e-3)
    s = HSolverBatch(ctx, params, 61, FH_H_DF64)
    s.set_u(U0s)
    s.calc_step(60)
    for q, u0, g in zip(params, U0s, s.get_u()):
        ref, _ = O.h_solve(q, u0, 60)
        assert relmax(g, ref) <= TOL_SOLVER, (q["alpha"], q["beta"])


def test_h_batch_autotune_keeps_results(ctx):
    """The launch-shape autotuner changes only how the history sum is tiled:
    the batch still matches the oracle afterwards."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import HSolverBatch
    params, U0s = workloads.psi_batch(n=40, seed=5, Nmin=17, Nmax=300, tau=2e-3)
    s = HSolverBatch(ctx, params, 81)
    shape = s.autotune()
    assert shape["tile_threads"] in (128, 256, 512) and shape["split_cap"] in (1, 8, 64)
    s.set_u(U0s)
    s.calc_step(80)
    for q, u0, g in list(zip(params, U0s, s.get_u()))[:5]:
        ref, _ = O.h_solve(q, u0, 80)
        assert relmax(g, ref) <= TOL_SOLVER


def test_h_solver_history_full_is_reported(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FhError
    from theses_code_gb300.solvers import HSolverBatch
    p, U0 = workloads.caputo_1d(10)
    s = HSolverBatch(ctx, [p], 3)
    s.set_u([U0])
    s.calc_step(3)
    with pytest.raises(FhError):
        s.calc_step(1)


# ---------------------------------------------------------------- 2D solver
def test_tg_reference_golden(ctx):
    from theses_code_gb300.solvers import TGSolver
    g = json.load(open(os.path.join(G, "tg_adi.json")))
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"], d=g["d"],
             C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"])
    s = TGSolver(ctx, p, g["steps"])
    s.set_state(np.array(g["V2"]), np.array(g["C0"]))
    s.calc_step(g["steps"])
    assert relmax(s.get_c(), g["C"]) <= TOL_SOLVER


@pytest.mark.parametrize("mode", [0, 2])  # FH_TG_FP64, FH_TG_DF64 (double-float history)
@pytest.mark.parametrize("sN,M,steps", [(64, 48, 40), (130, 97, 25), (40, 40, 150)])
def test_tg_vs_oracle(ctx, sN, M, steps, mode):
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(sN, M, alpha=0.7, tau=5e-4, d=0.1, seed=sN, C1=0.2, S=0.01)
    s = TGSolver(ctx, p, steps, mode)
    s.set_state(V2, C0)
    s.calc_step(steps)
    ref, _ = O.tg_solve(p, V2, C0, steps)
    assert relmax(s.get_c(), ref) <= TOL_SOLVER


@pytest.mark.parametrize("mode", [0, 2])  # FH_TG_FP64, FH_TG_DF64
def test_tg_restricted_reference_golden(ctx, mode):
    """Restricted summing (dt_alg 2, dt_eps 0.012) against the reference run."""
    from theses_code_gb300.solvers import TGSolver
    g = json.load(open(os.path.join(G, "tg_adi_restricted.json")))
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"], d=g["d"],
             C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"])
    s = TGSolver(ctx, p, g["steps"], mode)
    s.set_state(np.array(g["V2"]), np.array(g["C0"]))
    s.set_restricted(g["dt_eps"])
    s.calc_step(g["steps"])
    assert relmax(s.get_c(), g["C"]) <= TOL_SOLVER


@pytest.mark.parametrize("mode,tol", [(0, TOL_SOLVER), (2, TOL_SOLVER), (1, 1e-9)])  # FP64, DF64, blocked
def test_tg_restricted_vs_oracle(ctx, mode, tol):
    """150 steps with the sums cut about 32 layer pairs back (psi = t: the
    sums read only those layers); the blocked mode also zeroes the cut
    weights of its tensor-core rows.  A second solve with dt_eps = 0 is the
    full history again."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(40, 40, alpha=0.7, tau=5e-4, d=0.1, seed=9, C1=0.2, S=0.01)
    steps, eps = 150, 0.003
    s = TGSolver(ctx, p, steps, mode)
    s.set_state(V2, C0)
    s.set_restricted(eps)
    s.calc_step(steps)
    ref, _ = O.tg_solve(dict(p, dt_alg=2, dt_eps=eps), V2, C0, steps)
    full, _ = O.tg_solve(p, V2, C0, steps)
    assert relmax(full, ref) > 1e-4
    assert relmax(s.get_c(), ref) <= tol
    s.set_state(V2, C0)
    s.set_restricted(0.0)
    s.calc_step(steps)
    assert relmax(s.get_c(), full) <= tol


def test_tg_restricted_blocked_skips_old_groups(ctx):
    """Blocked mode, 400 steps, cut ~100 layer pairs back: from step 256 on the
    tensor-core contraction starts at the first 128-layer group with a
    non-zero weight."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(40, 40, alpha=0.7, tau=5e-4, d=0.1, seed=9, C1=0.2, S=0.01)
    steps, eps = 400, 1.4e-3
    s = TGSolver(ctx, p, steps, FH_TG_BLOCKED)
    s.set_state(V2, C0)
    s.set_restricted(eps)
    s.calc_step(steps)
    ref, _ = O.tg_solve(dict(p, dt_alg=2, dt_eps=eps), V2, C0, steps)
    assert relmax(s.get_c(), ref) <= 1e-9


def test_tg_restricted_psi_beta_vs_oracle(ctx):
    """psi = t^1.3 (weights not Toeplitz: every stored layer pair is visited,
    the cut ones with weight 0)."""
    import math
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(40, 33, alpha=0.6, tau=1e-3, seed=4, C1=0.1)
    p["beta"] = 1.3
    steps = 60
    Da = 1.0 / math.gamma(1.0 - p["alpha"])
    w = [Da * O.psi_int(k, k + 1.0, steps - 0.5, p["tau"], p["alpha"], 1.3) for k in (39, 40)]
    eps = 0.5 * (w[0] + w[1])  # between the weights 20 and 19 layer pairs back at the last step
    s = TGSolver(ctx, p, steps)
    s.set_state(V2, C0)
    s.set_restricted(eps)
    s.calc_step(steps)
    ref, _ = O.tg_solve(dict(p, dt_alg=2, dt_eps=eps), V2, C0, steps)
    full, _ = O.tg_solve(p, V2, C0, steps)
    assert relmax(full, ref) > 1e-6
    assert relmax(s.get_c(), ref) <= TOL_SOLVER


@pytest.mark.parametrize("mode", [0, 2])  # FH_TG_FP64, FH_TG_DF64
def test_tg_series_reference_golden(ctx, mode):
    """Series expansion (dt_alg 3, 12 terms) against the reference run."""
    from theses_code_gb300.solvers import TGSolver
    g = json.load(open(os.path.join(G, "tg_adi_restricted.json")))
    sr = json.load(open(os.path.join(G, "tg_adi_series.json")))
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"], d=g["d"],
             C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"])
    s = TGSolver(ctx, p, sr["steps"], mode)
    s.set_series(sr["dt_eps"])
    s.set_state(np.array(g["V2"]), np.array(g["C0"]))
    s.calc_step(sr["steps"])
    assert relmax(s.get_c(), sr["C"]) <= TOL_SOLVER


@pytest.mark.parametrize("mode", [0, 2])
def test_tg_series_vs_oracle(ctx, mode):
    """40 x 40, 150 steps, 20 terms: captured-graph solve, a second solve from
    the same state (the accumulators restart), uneven calls, and back to the
    full history with 0 terms."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(40, 40, alpha=0.7, tau=5e-4, d=0.1, seed=9, C1=0.2, S=0.01)
    steps, J = 150, 20
    ref, _ = O.tg_solve(dict(p, dt_alg=3, dt_eps=J), V2, C0, steps)
    full, _ = O.tg_solve(p, V2, C0, steps)
    assert relmax(full, ref) > 1e-4
    s = TGSolver(ctx, p, steps, mode)
    s.set_series(J)
    for calls in ((steps,), (steps,), (1, 60, 89)):
        s.set_state(V2, C0)
        for n in calls:
            s.calc_step(n)
        assert relmax(s.get_c(), ref) <= TOL_SOLVER, calls
    s.set_state(V2, C0)
    s.set_series(0)
    s.calc_step(steps)
    assert relmax(s.get_c(), full) <= TOL_SOLVER


def test_tg_series_limits(ctx):
    """The series needs psi = t and a plain mode; bad term counts are refused."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED, FhError
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(40, 40, alpha=0.7, tau=5e-4, d=0.1, seed=9)
    with pytest.raises(FhError):
        TGSolver(ctx, p, 100, FH_TG_BLOCKED).set_series(10)
    s = TGSolver(ctx, dict(p, beta=1.3), 10)
    with pytest.raises(FhError):
        s.set_series(10)
    s = TGSolver(ctx, p, 10)
    for bad in (-1, 257):
        with pytest.raises(FhError):
            s.set_series(bad)
    s.set_state(V2, C0)
    s.calc_step(1)
    with pytest.raises(FhError):  # only before the first step
        s.set_series(5)


def test_tg_solvers_of_different_sizes_coexist(ctx):
    """A smaller solver created after a larger one must not break the larger
    one's sweeps (their shared-memory needs differ)."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    pb, V2b, C0b = workloads.convection_2d(320, 300, alpha=0.7, tau=5e-4, d=0.1, seed=2)
    big = TGSolver(ctx, pb, 3)
    big.set_state(V2b, C0b)
    ps, V2s, C0s = workloads.convection_2d(40, 40, alpha=0.7, tau=5e-4, d=0.1, seed=3)
    small = TGSolver(ctx, ps, 3)
    small.set_state(V2s, C0s)
    big.calc_step(3)
    small.calc_step(3)
    ref, _ = O.tg_solve(pb, V2b, C0b, 3)
    assert relmax(big.get_c(), ref) <= TOL_SOLVER
    ref, _ = O.tg_solve(ps, V2s, C0s, 3)
    assert relmax(small.get_c(), ref) <= TOL_SOLVER
    big.close()
    small.close()


def test_size_limits_are_reported(ctx):
    """Sizes beyond what the staged sweeps and lines hold are refused with
    FH_EINVAL instead of being launched."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FhError
    from theses_code_gb300.solvers import ABSolver, TGSolver
    p, _, _ = workloads.convection_2d(40, 40)
    p["M"] = 2000
    with pytest.raises(FhError):
        TGSolver(ctx, p, 10)
    with pytest.raises(FhError):
        ABSolver(ctx, 4000, 10, 1e-3, 0.5)


def test_tg_psi_beta_vs_oracle(ctx):
    """psi(t) = t^1.3: the factorization is rebuilt every step."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(40, 33, alpha=0.6, tau=1e-3, seed=4, C1=0.1)
    p["beta"] = 1.3
    s = TGSolver(ctx, p, 20)
    s.set_state(V2, C0)
    s.calc_step(20)
    ref, _ = O.tg_solve(p, V2, C0, 20)
    assert relmax(s.get_c(), ref) <= TOL_SOLVER


# ------------------------------------------------------------------ AB solve
@pytest.mark.parametrize("key", ["solve", "solve2"])
def test_ab_reference_golden(ctx, key):
    """solve_and_check of the reference (full history, its own current-step
    coefficient and lag-weight cache): the field of the last step, and the
    mean-squared error."""
    from theses_code_gb300.solvers import ABSolver
    s_ = json.load(open(os.path.join(G, "ab.json")))[key]
    m, n, a = s_["m"], s_["n"], s_["alpha"]
    tau = s_["T"] / n
    lam = -a / (1 - a)
    src = np.array([[(24.0 / (1 - a)) * (i * tau) ** 4 * O.mittag_leffler(a, 5.0, lam * (i * tau) ** a)
                     for _ in range(m + 1)] for i in range(1, n + 1)])
    ex = np.array([[(i * tau) ** 4 for _ in range(m + 1)] for i in range(1, n + 1)])
    s = ABSolver(ctx, m, n, tau, a)
    s.set_source(src, ex[:, 0].copy(), ex[:, -1].copy())
    s.set_c(np.zeros(m + 1))
    s.set_current_coef(s_["ii"])
    s.set_lag_weights(s_["lagw"])
    err = 0.0
    for i in range(n):
        s.calc_step(1)
        err += float(np.sum((s.get_c() - ex[i]) ** 2))
    err /= (m + 1.0) * n
    assert relmax(s.get_c(), s_["C"]) <= TOL_SOLVER
    assert abs(err - s_["err"]) <= 1e-10 * s_["err"]
    s.close()


def test_ab_vs_oracle(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import ABSolver
    cfg, src, bl, br, C0 = workloads.ab_1d(m=256, alpha=0.6, tau=1e-3, seed=2)
    n = 400
    s = ABSolver(ctx, cfg["m"], n, cfg["tau"], cfg["alpha"])
    s.set_source(src, bl, br)
    s.set_c(C0)
    s.calc_step(n)
    w = O.ab_weights(n, cfg["tau"], cfg["alpha"])
    srcs = np.repeat(src, n, axis=0)
    ref, _ = O.ab_solve(cfg["m"], n, cfg["tau"], cfg["alpha"], w, srcs, np.zeros(n), np.zeros(n), C0)
    assert relmax(s.get_c(), ref) <= TOL_SOLVER


@pytest.mark.parametrize("mode_name", ["FH_TG_FP64", "FH_TG_DF64"])
def test_tg_two_series_vs_reference_and_oracle(ctx, mode_name):
    """dt_alg 4 (two-series approximation, psi = t) through the library:
    against the reference's own run (golden) and the oracle, and ~1e-7 away
    from the full-history solve (the approximation is the reference's)."""
    from theses_code_gb300 import _lib
    from theses_code_gb300.solvers import TGSolver
    g = json.load(open(os.path.join(G, "tg_adi_restricted.json")))
    for key in ("0.7_150", "0.9_300"):
        r = json.load(open(os.path.join(G, "tg_adi_two_series.json")))[key]
        p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=r["alpha"], beta=1.0, sigma=g["sigma"], d=g["d"],
                 C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"])
        s = TGSolver(ctx, p, r["steps"] + 1, getattr(_lib, mode_name))
        s.set_two_series(True)
        s.set_state(np.array(g["V2"]), np.array(g["C0"]))
        s.calc_step(r["steps"])
        got = s.get_c()
        assert relmax(got, r["C"]) <= TOL_SOLVER, (key, relmax(got, r["C"]))
        ref, _ = O.tg_solve(dict(p, dt_alg=4, dt_eps=1e-8), np.array(g["V2"]), np.array(g["C0"]), r["steps"])
        assert relmax(got, ref) <= TOL_SOLVER
        s.close()


def test_tg_two_series_larger_grid(ctx):
    """dt_alg 4 on a 48 x 40 grid over 300 steps (tens of approximations per
    node) against the oracle, in uneven step calls after a captured solve."""
    from theses_code_gb300 import workloads
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(48, 40, alpha=0.6, tau=1e-3, d=0.1, seed=4, C1=0.2)
    steps = 300
    ref, _ = O.tg_solve(dict(p, dt_alg=4, dt_eps=1e-8), V2, C0, steps)
    full, _ = O.tg_solve(p, V2, C0, steps)
    assert 1e-10 < relmax(ref, full) < 1e-4  # the approximation is in play
    s = TGSolver(ctx, p, steps + 1)
    s.set_two_series(True)
    s.set_state(V2, C0)
    s.calc_step(steps)
    assert relmax(s.get_c(), ref) <= TOL_SOLVER
    s.set_state(V2, C0)
    for n in (1, 150, 149):
        s.calc_step(n)
    assert relmax(s.get_c(), ref) <= TOL_SOLVER
    s.close()


def test_tg_two_series_limits(ctx):
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED, FhError
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(24, 20, alpha=0.6, tau=1e-3, d=0.1, seed=4)
    s = TGSolver(ctx, p, 20)
    s.set_series(8)
    with pytest.raises(FhError):
        s.set_two_series(True)  # not with the single-series expansion
    s.set_series(0)
    s.set_two_series(True)
    with pytest.raises(FhError):
        s.set_series(8)
    s.set_state(V2, C0)
    s.calc_step(3)
    with pytest.raises(FhError):
        s.set_two_series(False)  # only before the first step
    s.close()
    b = TGSolver(ctx, p, 20, FH_TG_BLOCKED)
    with pytest.raises(FhError):
        b.set_two_series(True)
    b.close()
    q = TGSolver(ctx, dict(p, beta=1.3), 20)
    with pytest.raises(FhError):
        q.set_two_series(True)
    q.close()


@pytest.mark.parametrize("mode_name", ["FH_TG_FP64", "FH_TG_DF64"])
@pytest.mark.parametrize("key", ["massN", "variable_d", "variable_d_massN"])
def test_tg_variants_vs_reference(ctx, mode_name, key):
    """TG_solver_ with the mass-exchange stage and/or the velocity-dependent
    diffusion coefficient (TG_solver_<0,0,0>) against the reference's own
    runs of the 12 x 10 problem (40 steps)."""
    from theses_code_gb300 import _lib
    from theses_code_gb300.solvers import TGSolver
    g = json.load(open(os.path.join(G, "tg_adi_restricted.json")))
    r = json.load(open(os.path.join(G, "tg_adi_variants.json")))[key]
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"], d=g["d"],
             C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"])
    s = TGSolver(ctx, p, r["steps"] + 1, getattr(_lib, mode_name))
    if r["massN"]:
        s.set_mass_exchange(True, r["massN_a"], r["massN_b"])
    if not r["fixed_d"]:
        s.set_diffusion(False, *r["dcoef"])
    s.set_state(np.array(g["V2"]), np.array(g["C0"]))
    s.calc_step(r["steps"])
    assert relmax(s.get_c(), r["C"]) <= TOL_SOLVER
    # a second solve from the same state (N back to 0)
    s.set_state(np.array(g["V2"]), np.array(g["C0"]))
    for n in (7, 33):
        s.calc_step(n)
    assert relmax(s.get_c(), r["C"]) <= TOL_SOLVER
    s.close()


def test_tg_variants_larger_grid_and_blocked(ctx):
    """Both variants together on a 64 x 48 grid (150 steps) against the
    oracle; the velocity-dependent coefficient in the blocked mode at the
    mixed-precision bound; the mass exchange refused there."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED, FhError
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(64, 48, alpha=0.7, tau=5e-4, d=0.1, seed=6, C1=0.2, S=0.05)
    lam, ka0, kk = 5.0, 1.005e-3, 2.0 * math.sqrt(5.0) / (math.pi * 2.5)
    q = dict(p, massN=1, massN_a=0.4, massN_b=1.5, fixed_d=0, ka0=ka0, kk=kk)
    q["lambda"] = lam
    steps = 150
    ref, _ = O.tg_solve(q, V2, C0, steps)
    base, _ = O.tg_solve(p, V2, C0, steps)
    assert relmax(ref, base) > 1e-3
    s = TGSolver(ctx, p, steps)
    s.set_mass_exchange(True, 0.4, 1.5)
    s.set_diffusion(False, lam, ka0, kk)
    s.set_state(V2, C0)
    s.calc_step(steps)
    assert relmax(s.get_c(), ref) <= TOL_SOLVER
    s.close()
    qd = dict(p, fixed_d=0, ka0=ka0, kk=kk)
    qd["lambda"] = lam
    ref_d, _ = O.tg_solve(qd, V2, C0, steps)
    b = TGSolver(ctx, p, steps, FH_TG_BLOCKED)
    with pytest.raises(FhError):
        b.set_mass_exchange(True, 0.4, 1.5)
    b.set_diffusion(False, lam, ka0, kk)
    b.set_state(V2, C0)
    b.calc_step(steps)
    assert relmax(b.get_c(), ref_d) <= 1e-9
    b.close()


@pytest.mark.parametrize("J,P,ldh", [(16, 1000, 1000), (1, 7, 8), (256, 3001, 3072)])
def test_series_sum(ctx, torch_mod, J, P, ldh):
    """Series accumulators of the irrigation model (sum_alg 2): the update and
    the evaluation in the reference's operation order, bit for bit against
    the same sequence in numpy, over three steps."""
    torch = torch_mod
    import ctypes as C
    from theses_code_gb300._lib import FhError
    rng = np.random.default_rng(J)
    H = rng.normal(size=(J, ldh))
    Hd = dev(torch, H)
    S = torch.zeros(P, dtype=torch.float64, device="cuda")
    Href = H.copy()
    for step in range(3):
        c = rng.normal(size=J) * 0.1
        e = rng.normal(size=J)
        tau = 1e-3 * (1 + step)
        d = rng.normal(size=P)
        dd = dev(torch, d)
        ctx.call("fh_series_sum", J, P, c.ctypes.data_as(C.c_void_p), e.ctypes.data_as(C.c_void_p), tau,
                 dd.data_ptr(), Hd.data_ptr(), ldh, S.data_ptr())
        ctx.sync()
        s = np.zeros(P)
        for n in range(J):
            Href[n, :P] = Href[n, :P] + c[n] * d
            s = s + e[n] * Href[n, :P]
        s = s / tau
        assert np.array_equal(S.cpu().numpy(), s)
        assert np.array_equal(Hd.cpu().numpy()[:, :P], Href[:, :P])
    with pytest.raises(FhError):
        ctx.call("fh_series_sum", 0, P, c.ctypes.data_as(C.c_void_p), e.ctypes.data_as(C.c_void_p), 1e-3,
                 dd.data_ptr(), Hd.data_ptr(), ldh, S.data_ptr())
