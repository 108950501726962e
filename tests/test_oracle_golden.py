"""Pins the CPU oracle against golden vectors produced by the reference itself
(tests/golden/make_golden.py runs the reference solvers compiled from their own
sources).  CPU only."""
import json
import math
import os

import numpy as np
import pytest

from oracle import oracle as O

G = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    with open(os.path.join(G, name)) as f:
        return json.load(f)


def relmax(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("name,weights,beta", [
    ("h_minimal_space.json", O.W_L1, 1.0),   # gamma 0.7: space-fractional derivative in z
    ("h_psi_space.json", O.W_PSI, 1.0),      # gamma 0.75
    ("h_psi_t07_space.json", O.W_PSI, 0.7),  # gamma 0.6, psi = t^0.7
])
def test_h_solver_space_fractional_matches_reference(name, weights, beta):
    g = load(name)
    N = g["N"]
    p = dict(N=N, L=g["L"], tau=g["tau"], alpha=g["alpha"], weights=weights, beta=beta,
             kmodel=O.K_CONST, kc=g["k"], kgam=0.0, cinv=20.0, gravity=1, al_left=1.0,
             bt_left=-g["uc"], u_right=g["Hbottom"], gamma=g["extra"][3])
    U0 = np.zeros(N + 2)
    U0[:N + 1] = g["U0"]
    U, _ = O.h_solve(p, U0, g["steps"])
    assert relmax(U, g["U"]) <= 1e-13
    # the nonlocal term matters: the classical run is far from the reference's
    U1, _ = O.h_solve(dict(p, gamma=1.0), U0, g["steps"])
    assert relmax(U1, g["U"]) > 1e-4


@pytest.mark.parametrize("name,weights,beta", [
    ("h_minimal_l1.json", O.W_L1, 1.0),   # mt_minimal.cpp H_solver
    ("h_psi_t.json", O.W_PSI, 1.0),       # mt_psi_caputo.cpp H_solver, psi = t
    ("h_psi_t07.json", O.W_PSI, 0.7),     # psi = t^0.7, reference series at eps 1e-15
    ("h_psi_t15.json", O.W_PSI, 1.5),     # psi = t^1.5
])
def test_h_solver_matches_reference(name, weights, beta):
    g = load(name)
    N = g["N"]
    p = dict(N=N, L=g["L"], tau=g["tau"], alpha=g["alpha"], weights=weights, beta=beta,
             kmodel=O.K_CONST, kc=g["k"], kgam=0.0, cinv=20.0, gravity=1, al_left=1.0,
             bt_left=-g["uc"], u_right=g["Hbottom"])
    U0 = np.zeros(N + 2)
    U0[:N + 1] = g["U0"]
    U, _ = O.h_solve(p, U0, g["steps"])
    # the solution moved by O(1): the comparison is not trivially satisfied
    assert np.max(np.abs(np.array(g["U"])[:N + 1] - np.array(g["U0"]))) > 0.5
    assert relmax(U, g["U"]) <= 1e-12


def test_tg_adi_matches_reference():
    g = load("tg_adi.json")
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"],
             d=g["d"], C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"])
    C, _ = O.tg_solve(p, np.array(g["V2"]), np.array(g["C0"]), g["steps"])
    assert np.max(np.abs(np.array(g["C"]) - np.array(g["C0"]))) > 0.1
    assert relmax(C, g["C"]) <= 1e-13


def test_tg_adi_restricted_matches_reference():
    """dt_alg 2 (restricted summing, dt_eps 0.012): the sums stop about 12
    layer pairs back; the result moves far from the full-history run."""
    g = load("tg_adi_restricted.json")
    full = load("tg_adi_40.json")
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"],
             d=g["d"], C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"], dt_alg=2, dt_eps=g["dt_eps"])
    C, _ = O.tg_solve(p, np.array(g["V2"]), np.array(g["C0"]), g["steps"])
    assert relmax(C, g["C"]) <= 1e-13
    assert relmax(np.array(full["C"]), g["C"]) > 0.05
    p["dt_alg"] = 0
    C, _ = O.tg_solve(p, np.array(g["V2"]), np.array(g["C0"]), g["steps"])
    assert relmax(C, full["C"]) <= 1e-13


def test_tg_adi_series_matches_reference():
    """dt_alg 3 (series expansion, 12 terms, psi = t) against the reference run."""
    g = load("tg_adi_restricted.json")  # the same problem
    sr = load("tg_adi_series.json")
    full = load("tg_adi_40.json")
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"],
             d=g["d"], C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"], dt_alg=3, dt_eps=sr["dt_eps"])
    C, _ = O.tg_solve(p, np.array(g["V2"]), np.array(g["C0"]), sr["steps"])
    assert relmax(C, sr["C"]) <= 1e-13
    assert relmax(np.array(full["C"]), sr["C"]) > 0.01


@pytest.mark.parametrize("key", ["0.7_150", "0.9_300"])
def test_tg_adi_two_series_matches_reference(key):
    """dt_alg 4 (two-series approximation of the history sums, psi = t):
    the per-point long and short approximations are rebuilt from the same
    F-independent ranges, so the oracle meets the reference run bit for bit,
    while the approximation itself stays ~1e-7 from the full-history run."""
    g = load("tg_adi_restricted.json")  # the same problem
    r = load("tg_adi_two_series.json")[key]
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=r["alpha"], beta=1.0, sigma=g["sigma"],
             d=g["d"], C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"], dt_alg=4, dt_eps=1e-8)
    C, _ = O.tg_solve(p, np.array(g["V2"]), np.array(g["C0"]), r["steps"])
    assert relmax(C, r["C"]) <= 1e-14
    full, _ = O.tg_solve(dict(p, dt_alg=0), np.array(g["V2"]), np.array(g["C0"]), r["steps"])
    assert 1e-9 < relmax(full, r["C"]) < 1e-5


@pytest.mark.parametrize("key", ["massN", "variable_d", "variable_d_massN"])
def test_tg_adi_variants_match_reference(key):
    """TG_solver_ with the mass-exchange stage N1 (fr_d_t_g_2d.cpp:2503-2521,
    3330-3332) and/or the velocity-dependent diffusion coefficient of
    TG_solver_<0,0,0> (2787-2800), bit for bit against the reference runs."""
    g = load("tg_adi_restricted.json")  # the same problem
    r = load("tg_adi_variants.json")[key]
    lam, ka0, kk = r["dcoef"]
    p = dict(sN=g["sN"], M=g["M"], tau=g["tau"], alpha=g["alpha"], beta=1.0, sigma=g["sigma"], d=g["d"],
             C1=g["C1"], S=g["S"], dL=g["dL"], dLx=g["dLx"], dt_alg=0, dt_eps=0.0, massN=r["massN"],
             massN_a=r["massN_a"], massN_b=r["massN_b"], fixed_d=r["fixed_d"], ka0=ka0, kk=kk)
    p["lambda"] = lam
    C, _ = O.tg_solve(p, np.array(g["V2"]), np.array(g["C0"]), r["steps"])
    assert relmax(C, r["C"]) <= 1e-15
    full = load("tg_adi_40.json")["C"]
    assert relmax(full, r["C"]) > 0.01  # the variant matters


def test_two_series_bookkeeping_counts():
    """The approximation sets stay small: after 2000 layers tens of long and
    short approximations per point and direction, growing slower than the
    layer count."""
    import ctypes as C
    n = 2000
    for a, b in ((1.5, 0.5), (2.0, 1.0)):
        nia = np.zeros(n, dtype=np.int32)
        nibk = np.zeros(n, dtype=np.int32)
        assert O.lib().fho_tg_two_series_counts(C.c_double(0.7), n, C.c_double(a), C.c_double(b),
                                                nia.ctypes.data_as(C.c_void_p), nibk.ctypes.data_as(C.c_void_p)) == 0
        assert 10 <= nia[-1] <= 40 and 10 <= nibk[-1] <= 100
        assert nia[999] <= nia[-1] < 2 * nia[999] and nibk.max() < 100


def test_psi_weights_match_reference_series():
    """calc_int (mt_psi_caputo.cpp:720-741) at eps 1e-15 against the converged
    incomplete-beta value.  The reference series does not converge on the very
    first interval [0, tau] of step 1 (both endpoints singular, ratio 1 in
    _kb_row); that entry is pinned against the closed Beta-function value."""
    for key, v in load("psi_weights.json").items():
        a_, b_ = v["alpha"], v["beta"]
        for a, t0, val in v["w"]:
            o = O.psi_int(t0, t0 + 1, a, v["tau"], a_, b_)
            if a == 1 and t0 == 0:
                exact = (v["tau"] ** (1 - a_ * b_) / b_) * math.exp(
                    math.lgamma(1 / b_) + math.lgamma(1 - a_) - math.lgamma(1 / b_ + 1 - a_))
                assert abs(o - exact) <= 1e-13 * abs(exact), (key, a, t0)
            else:
                assert abs(o - val) <= 1e-9 * abs(val), (key, a, t0, o, val)


def test_psi_weights_match_incomplete_beta():
    """The oracle's psi = t^beta weights against mpmath's incomplete beta
    function at 40 digits, T^(1-a b)/b * betainc(1/b, 1-a, y0, y1), over early,
    middle and late intervals of long solves (where the difference of the two
    incomplete-beta values loses log10(X) digits if it is formed directly)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    rng = np.random.default_rng(3)
    for alpha, beta in [(0.6, 0.5), (0.8, 2.0), (0.55, 1.37), (0.9, 0.75), (0.5, 2.0), (0.7, 1.3)]:
        for X, tau in [(2.0, 1e-3), (7.0, 1e-3), (60.5, 1e-3), (500.5, 5e-4), (5001.0, 1e-3)]:
            ks = {0, 1, int(X) - 2, int(X) - 1} | {int(k) for k in rng.integers(0, int(X - 1), 6)}
            for k in sorted(ks):
                x0, x1 = float(k), min(k + 1.0, X)
                if not 0.0 <= x0 < X:
                    continue
                Xm, b = mp.mpf(X), mp.mpf(beta)
                ref = (Xm * tau) ** (1 - mp.mpf(alpha) * b) / b * mp.betainc(
                    1 / b, 1 - mp.mpf(alpha), (mp.mpf(x0) / Xm) ** b, (mp.mpf(x1) / Xm) ** b)
                got = O.psi_int(x0, x1, X, tau, alpha, beta)
                assert abs(got - float(ref)) <= 4e-16 * abs(float(ref)), (alpha, beta, X, k)


def test_psi_t_is_l1():
    """For psi = t the psi-Caputo weight is the L1 coefficient times tau^(1-a)/(1-a)."""
    for alpha in (0.3, 0.7, 0.95):
        for n in (1, 5, 200, 4000):
            for k in (0, n // 2, n):
                w = O.psi_int(k, k + 1, n + 1, 1e-3, alpha, 1.0)
                b = O.l1_b(n - k, alpha) * (1e-3) ** (1 - alpha) / (1 - alpha)
                assert abs(w - b) <= 1e-11 * abs(b)


def test_mittag_leffler_matches_reference_and_identities():
    for a, b, z, v in load("ab.json")["ml"]:
        assert abs(O.mittag_leffler(a, b, z) - v) <= 1e-14 * abs(v)
    for z in (-3.0, -0.5, 0.0, 0.7, 2.0):
        assert abs(O.mittag_leffler(1.0, 1.0, z) - math.exp(z)) <= 1e-14 * math.exp(z)
    for x in (0.3, 1.0, 2.5):
        assert abs(O.mittag_leffler(2.0, 1.0, -x * x) - math.cos(x)) <= 1e-13


def test_ab_lag_weights_match_reference():
    """MF_int_choice series (MF_int_series.cpp:436-455) at the lags the history
    sum uses (lag >= 2; MF_intF_simple sums tt <= n-2)."""
    v = load("ab.json")["abw"]
    for lag, val in v["w"]:
        if lag >= 2:
            assert abs(O.ab_int(lag, v["tau"], v["alpha"]) - val) <= 1e-12 * abs(val)


@pytest.mark.parametrize("key", ["solve", "solve2"])
def test_ab_solve_matches_reference(key):
    """solve_and_check (full history) with the reference's own current-step
    coefficient and lag-weight cache (MF_intF_simple's I_cache: the converged
    series while (a/(1-a)) (lag tau)^a < 1, the MF_intFv quadrature beyond, up
    to 1e-5 from the series): the field of the last step and the mean-squared
    error."""
    s = load("ab.json")[key]
    m, n, a = s["m"], s["n"], s["alpha"]
    tau = s["T"] / n
    w = np.zeros(n + 1)
    w[1:] = s["lagw"]
    w[0] = s["ii"]
    conv = O.ab_weights(n, tau, a)  # the converged series: equal where the reference sums the series
    for L in range(2, n + 1):
        if (a / (1 - a)) * (L * tau) ** a < 1.0:
            assert abs(conv[L] - w[L]) <= 1e-13 * abs(w[L]), L
    lam = -a / (1 - a)
    src = np.array([[(24.0 / (1 - a)) * (i * tau) ** 4 * O.mittag_leffler(a, 5.0, lam * (i * tau) ** a)
                     for _ in range(m + 1)] for i in range(1, n + 1)])
    ex = np.array([[(i * tau) ** 4 for _ in range(m + 1)] for i in range(1, n + 1)])
    c, err = O.ab_solve(m, n, tau, a, w, src, ex[:, 0].copy(), ex[:, -1].copy(), np.zeros(m + 1), ex)
    ref = np.array(s["C"])
    assert np.max(np.abs(c - ref)) <= 1e-13 * np.max(np.abs(ref))
    assert abs(err - s["err"]) <= 1e-12 * s["err"]


def test_thomas_solves_system():
    rng = np.random.default_rng(0)
    N = 37
    A = rng.uniform(0.5, 1.0, N + 1)
    B = rng.uniform(0.5, 1.0, N + 1)
    R = A + B + rng.uniform(0.1, 1.0, N + 1)
    Om = rng.normal(size=N + 1)
    u = O.thomas(A, R, B, Om, 0.0, 0.25, 0, -0.5, np.zeros(N + 2))
    res = A[1:N] * u[0:N - 1] - R[1:N] * u[1:N] + B[1:N] * u[2:N + 1] - Om[1:N]
    assert np.max(np.abs(res)) < 1e-12
    assert u[0] == 0.25 and u[N] == -0.5 and u[N + 1] == u[N]
