"""The reference's 2D time loop with its result files (theses_code_gb300.tg_solve,
fr_d_t_g_2d.cpp solve()): log1 / log2 lines at the reference's output and save
times, values against the oracle's fields at those steps."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import oracle as O


def test_solve_writes_reference_logs(tmp_path):
    from theses_code_gb300 import tg_solve, workloads
    from theses_code_gb300._lib import Context
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(24, 20, alpha=0.7, tau=5e-3, d=0.1, seed=2, C1=0.3, S=0.05)
    p8 = dict(p, alpha=0.8)
    t, save_tau, out_tau = 0.2, 0.05, 0.04
    tts, outs, saves = tg_solve.event_steps(t, save_tau, out_tau, p["tau"])
    steps = len(tts)
    ctx = Context(0)
    a = TGSolver(ctx, p, steps)
    b = TGSolver(ctx, p8, steps)
    for s in (a, b):
        s.set_mass_exchange(True, 0.3, 0.7)  # the reference's massN applies to every solver
        s.set_state(V2, C0)
    l1, l2 = tmp_path / "log1.txt", tmp_path / "log2.txt"
    n = tg_solve.solve([a, b], t, save_tau, out_tau, p["tau"], str(l1), str(l2), mass=True)
    assert n == steps and a.get_c().size == V2.size
    _, wa = O.tg_solve(dict(p, massN=1, massN_a=0.3, massN_b=0.7), V2, C0, steps)
    _, wb = O.tg_solve(dict(p8, massN=1, massN_a=0.3, massN_b=0.7), V2, C0, steps)
    sN, M, ld = p["sN"], p["M"], p["sN"] + 2
    # log2: one line per output time, V of both solvers after that step
    lines2 = l2.read_text().splitlines()
    ks = [k for k, o in enumerate(outs) if o]
    assert len(lines2) == len(ks) > 0
    for k, line in zip(ks, lines2):
        f = line.split()
        assert f[0] == "T" and float(f[1]) == pytest.approx(tts[k], rel=1e-5)
        va, vb = float(f[3]), float(f[7])
        assert va == pytest.approx(wa[k + 1][sN // 4 + (M // 2) * ld], rel=1e-5, abs=1e-12)
        assert vb == pytest.approx(wb[k + 1][sN // 4 + (M // 2) * ld], rel=1e-5, abs=1e-12)
        assert "diffs(avgsq,maxabs,global" in line and len(f) == 16
    # log1: sN + 1 lines per save time; C at M/4, M/2, 3M/4 of each solver (+ N of each)
    lines1 = l1.read_text().splitlines()
    kss = [k for k, s_ in enumerate(saves) if s_]
    assert len(lines1) == (sN + 1) * len(kss) > 0
    for q, k in enumerate(kss):
        for i in range(sN + 1):
            f = [float(x) for x in lines1[q * (sN + 1) + i].split()]
            assert len(f) == 2 + 3 + 3 + 3 + 3
            assert f[0] == pytest.approx(tts[k], rel=1e-5) and f[1] == pytest.approx(i * p["dL"], rel=1e-5, abs=1e-12)
            for c, w in ((f[2:5], wa[k + 1]), (f[8:11], wb[k + 1])):
                ref = [w[i + (M * r // 4) * ld] for r in (1, 2, 3)]
                assert c == pytest.approx(ref, rel=1e-5, abs=1e-12)
    a.close()
    b.close()
    ctx.close()
