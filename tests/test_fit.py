"""Steepest-descent fitting (mt_psi_caputo.cpp:1892-1953) over the batched 1D
solver: the GPU driver follows the oracle driver's iterates."""
import numpy as np
import pytest

from theses_code_gb300 import fit, workloads


def oracle_runner(metric: int = 0):
    """fit.gpu_runner's scoring with every candidate solved by the CPU oracle."""
    from oracle import oracle as O

    @fit._only_valid
    def run(params_list, U0, tau, t_end, values):
        tts = fit._schedule(tau, t_end)
        steps = len(tts)
        out = []
        for p in params_list:
            U, hist = O.h_solve(p, U0, steps)
            before = [U0] + [hist[s] for s in range(steps - 1)]
            after = [hist[s] for s in range(steps)]
            N, dL = p["N"], p["L"] / p["N"]
            sc = fit._score(before, after, tts, tau, dL, N, values, metric)
            out.append(fit.BIG if not np.all(np.isfinite(U)) else sc)
        return out

    return run


def _problem():
    from oracle import oracle as O
    params, U0s = workloads.psi_batch(n=1, seed=3, Nmin=40, Nmax=40, tau=2e-3)
    base = dict(params[0], u_right=0.0)
    U0 = -np.asarray(U0s[0])  # pressure heads <= 0 (solve_and_test clamps v to <= 0)
    truth = dict(base, alpha=0.7, kc=0.4)
    tau, t_end = base["tau"], 0.1
    tts = fit._schedule(tau, t_end)
    _, hist = O.h_solve(truth, U0, len(tts))
    dL = base["L"] / base["N"]
    values = []
    for T in (0.021, 0.05, 0.0731, 0.099):
        s = int(T / tau)
        before = U0 if s == 0 else hist[s - 1]
        k1 = (T - tts[s]) / tau
        for Z in (0.13, 0.42, 0.77):
            v = (1 - k1) * fit._interp_z(before, dL, Z, base["N"] - 1) + k1 * fit._interp_z(hist[s], dL, Z, base["N"])
            values.append((T, Z, min(0.0, v)))
    return base, truth, U0, t_end, values


def test_oracle_driver_reduces_misfit():
    base, truth, U0, t_end, values = _problem()
    run = oracle_runner()
    assert run([truth], U0, base["tau"], t_end, values)[0] < 1e-20
    v_base = run([base], U0, base["tau"], t_end, values)[0]
    p, v, it, ns = fit.steepest_descent(run, base, ["alpha", "kc"], U0, t_end, values, vmax=[0.01, 0.01],
                                        eps=1e-9, max_iter=6)
    assert v < 0.01 * v_base and it >= 1 and ns >= 1 + 3 * it and (ns - 1) % 3 == 0


@pytest.mark.gpu
def test_gpu_driver_matches_oracle_driver():
    from theses_code_gb300._lib import Context
    ctx = Context(0)
    base, truth, U0, t_end, values = _problem()
    kw = dict(vmax=[0.01, 0.01], eps=1e-9, max_iter=6)
    pc, vc, itc, nc = fit.steepest_descent(oracle_runner(), base, ["alpha", "kc"], U0, t_end, values, **kw)
    pg, vg, itg, ng = fit.steepest_descent(fit.gpu_runner(ctx), base, ["alpha", "kc"], U0, t_end, values, **kw)
    assert (itg, ng) == (itc, nc)
    for k in ("alpha", "kc"):
        assert abs(pg[k] - pc[k]) <= 1e-9 * abs(pc[k]), k
    assert abs(vg - vc) <= 1e-8 * vc + 1e-20
    ctx.close()


def test_oracle_pso_reduces_misfit():
    base, truth, U0, t_end, values = _problem()
    run = oracle_runner()
    v_base = run([base], U0, base["tau"], t_end, values)[0]
    p, v, it, ns = fit.pso(run, base, ["alpha", "kc"], [(0.55, 0.9), (0.2, 0.9)], U0, t_end, values, n=8,
                           max_iter=4, seed=1)
    assert v < 0.2 * v_base and ns == 8 * (it + 1)
    # an out-of-range candidate scores 1e300 instead of failing the batch
    assert run([dict(base, alpha=1.2), base], U0, base["tau"], t_end, values)[0] == fit.BIG


@pytest.mark.gpu
def test_gpu_pso_matches_oracle_pso():
    from theses_code_gb300._lib import Context
    ctx = Context(0)
    base, truth, U0, t_end, values = _problem()
    kw = dict(n=8, max_iter=4, seed=1)
    b = [(0.55, 0.9), (0.2, 0.9)]
    pc, vc, itc, nc = fit.pso(oracle_runner(), base, ["alpha", "kc"], b, U0, t_end, values, **kw)
    pg, vg, itg, ng = fit.pso(fit.gpu_runner(ctx), base, ["alpha", "kc"], b, U0, t_end, values, **kw)
    assert (itg, ng) == (itc, nc)
    for k in ("alpha", "kc"):
        assert abs(pg[k] - pc[k]) <= 1e-9 * abs(pc[k]), k
    assert abs(vg - vc) <= 1e-8 * vc + 1e-20
    ctx.close()


def test_fit_input_file_round_trip(tmp_path):
    """The reference's fit_input.txt layout (mt_minimal.cpp:1955-2043): heads
    scaled by Hmult, the initial profile interpolated and extrapolated as in
    mt_psi_caputo.cpp:1700-1733, and a fit driven from the file."""
    from theses_code_gb300 import fit_input as FI
    base, truth, U0, t_end, values = _problem()
    lines = ["1 %d 3 1 0 0 0 0 1.0" % len(values), "8 0.7 1.4 1.4 1e-8 4"]
    lines += ["%r %r %r" % (float(T), float(Z), float(F) / FI.HMULT) for (T, Z, F) in values]
    lines += ["0.2 -0.03", "0.5 -0.01", "0.9 -0.02"]  # initial heads / Hmult
    lines += ["0.05 0.5 -0.01"]  # one check value
    lines += ["0.7 0.4"]  # fixed parameter values
    path = tmp_path / "fit_input.txt"
    path.write_text("\n".join(lines) + "\n")
    inp = FI.read_fit_input(str(path))
    assert inp["pso"]["n"] == 8 and inp["pso"]["max_iter"] == 4 and inp["param_values"] == [0.7, 0.4]
    assert np.allclose([v[2] for v in inp["values"]], [v[2] for v in values], rtol=1e-15)
    assert inp["check"][0][2] == pytest.approx(-0.1)
    U = FI.initial_profile(inp["init_Z"], inp["init_F"], 10, 0.1)
    assert U[0] == pytest.approx(-0.3 - 0.2 * (-0.1 - -0.3) / 0.3)      # extrapolated above the first depth
    assert U[3] == pytest.approx(-0.3 + (0.1 / 0.3) * 0.2)              # between 0.2 and 0.5
    assert U[10] == pytest.approx(-0.2 + 0.1 * (-0.2 - -0.1) / 0.4)     # extrapolated below the last
    U0f, t_endf, vals = FI.fit_problem(inp, base)
    run = oracle_runner()
    v0 = run([base], U0f, base["tau"], t_endf, vals)[0]
    p, v, it, ns = fit.steepest_descent(run, base, ["alpha", "kc"], U0f, t_endf, vals, vmax=[0.01, 0.01],
                                        eps=1e-9, max_iter=3)
    assert v < v0
    lines[0] = "1 %d 3 1 1 0 0 0 1.0" % len(values)  # one precipitation record: not modelled
    lines.insert(2 + len(values) + 3, "0.01 1e-7")
    path.write_text("\n".join(lines) + "\n")
    with pytest.raises(NotImplementedError):
        FI.fit_problem(FI.read_fit_input(str(path)), base)


def test_misfit_metrics():
    """solve_and_test's metrics 0, 1 and 2 (mt_psi_caputo.cpp:1790-1803) on
    hand-made states: one step, two measurements."""
    before = [np.array([-1.0, -2.0, -3.0])]
    after = [np.array([-1.0, -2.0, -4.0])]
    tts, tau, dL, N = [0.0], 1.0, 1.0, 2
    values = [(0.5, 0.5, -1.0), (0.25, 1.5, -3.0)]
    # point 1: z 0.5 -> (-1.5 before, -1.5 after) -> -1.5; point 2: z 1.5 ->
    # before (j < N-1: none) 0, after -3.0; k1 0.25 -> -0.75
    v1, v2 = -1.5, 0.75 * 0.0 + 0.25 * -3.0
    e0 = fit._score(before, after, tts, tau, dL, N, values, 0)
    assert e0 == pytest.approx((-1.0 - v1) ** 2 + (-3.0 - v2) ** 2)
    r1, r2 = abs((-1.0 - v1) / -1.0), abs((-3.0 - v2) / -3.0)
    assert fit._score(before, after, tts, tau, dL, N, values, 1) == pytest.approx(max(r1, r2))
    assert fit._score(before, after, tts, tau, dL, N, values, 2) == pytest.approx(r1 + r2 if r2 > r1 else r1)


def test_oracle_adaptive_pso_runs():
    """The adaptive schedule (omega and per-coordinate fi) on the oracle."""
    base, truth, U0, t_end, values = _problem()
    run = oracle_runner()
    v_base = run([base], U0, base["tau"], t_end, values)[0]
    p, v, it, ns = fit.pso(run, base, ["alpha", "kc"], [(0.55, 0.9), (0.2, 0.9)], U0, t_end, values, n=8,
                           max_iter=4, seed=1, adaptive=True)
    assert v < v_base and ns == 8 * (it + 1) and 0.0 < p["alpha"] < 1.0


def test_oracle_pso_restarts():
    """With restart_prox = 1 and omega 0.5 about half the moves restart: the
    swarm takes another path than without restarts (same random stream)."""
    base, truth, U0, t_end, values = _problem()
    run = oracle_runner()
    kw = dict(n=8, omega=0.5, max_iter=2, seed=3)
    b = [(0.55, 0.9), (0.2, 0.9)]
    p1, v1, _, _ = fit.pso(run, base, ["alpha", "kc"], b, U0, t_end, values, restart_prox=1.0, **kw)
    p0, v0, _, _ = fit.pso(run, base, ["alpha", "kc"], b, U0, t_end, values, restart_prox=0.0, **kw)
    assert v1 < fit.BIG and v0 < fit.BIG
    assert (p1["alpha"], p1["kc"]) != (p0["alpha"], p0["kc"])


def test_pso_log_lines():
    """The reference's PSO log layout (mt_psi_caputo.cpp:2056-2244)."""
    import io
    base, truth, U0, t_end, values = _problem()
    buf = io.StringIO()
    p, v, it, ns = fit.pso(oracle_runner(), base, ["alpha", "kc"], [(0.55, 0.9), (0.2, 0.9)], U0, t_end,
                           values, n=4, max_iter=2, seed=2, log=buf)
    lines = buf.getvalue().splitlines()
    assert [l.split(" - ")[0] for l in lines[:4]] == ["#initial %d" % i for i in range(4)]
    assert lines[4].startswith("#initial best: ") and len(lines[4].split()) == 2 + 3
    assert len(lines) == 5 + it and lines[5].startswith("0 avg ")
    last = lines[-1].split("best: ")[1].split()
    assert float(last[0]) == pytest.approx(v, rel=1e-5) and float(last[1]) == pytest.approx(p["alpha"], rel=1e-5)
