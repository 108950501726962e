"""Parameter fitting over the batched 1D solver.

The reference fits its H_solver parameters to measured pressure heads by
steepest descent and PSO (mt_psi_caputo.cpp:1750-2240): every candidate
parameter set is one full solve scored by ``solve_and_test``.  Here the
candidates of one round (the forward-difference perturbations of a gradient,
or a whole swarm) run as instances of one ``HSolverBatch`` (``gpu_runner``),
so a round costs one batched solve instead of one solve per candidate.

``_score`` restates ``solve_and_test`` with metric 0
(mt_psi_caputo.cpp:1762-1812): at each measurement (T, Z, F) the solution is
interpolated linearly in depth before and after the step whose interval
[tt, tt + tau) holds T, then linearly in time, clamped to <= 0, and
(F - v)^2 is summed; a non-finite solution scores 1e300.  ``steepest_descent``
restates mt_psi_caputo.cpp:1892-1953 (step halving on failure, stop below
``eps`` or after ``max_iter`` rounds); ``pso`` the swarm update of 2183-2223
in synchronous form.

A runner is any callable that scores a list of candidate parameter sets;
the tests also score the same candidates on the CPU oracle and check that
both drivers take the same rounds on either runner.
"""
from __future__ import annotations

import numpy as np

BIG = 1e300


def _schedule(tau: float, t_end: float):
    """Start times tt of the reference's loop ``for (tt = 0; tt <= t; tt += tau)``."""
    tts, tt = [], 0.0
    while tt <= t_end:
        tts.append(tt)
        tt += tau
    return tts


def _interp_z(U: np.ndarray, dL: float, z: float, jmax: int):
    for j in range(jmax):
        if dL * j < z <= dL * (j + 1):
            k2 = (z - dL * j) / dL
            return (1 - k2) * U[j] + k2 * U[j + 1]
    return None


def _score(before: list, after: list, tts, tau, dL, N, values, metric: int = 0) -> float:
    """Misfit from the states before/after each step (lists indexed by step).
    metric 0: sum of squared differences; 1: largest relative difference;
    2: relative differences added when one exceeds the running value (the
    reference's rule, mt_psi_caputo.cpp:1790-1803); F = 0 points are skipped
    by metrics 1 and 2."""
    err = 0.0
    for s, tt in enumerate(tts):
        for (T, Z, F) in values:
            if not (T >= tt and T < tt + tau):
                continue
            vb = _interp_z(before[s], dL, Z, N - 1)
            va = _interp_z(after[s], dL, Z, N)
            if va is None:
                continue
            k1 = (T - tt) / tau
            v = (1 - k1) * (vb if vb is not None else 0.0) + k1 * va
            if v > 0.0:
                v = 0.0
            if metric == 0:
                err += (F - v) * (F - v)
            elif F != 0:
                rel = abs((F - v) / F)
                if rel > err:
                    err = rel if metric == 1 else err + rel
        if not np.isfinite(after[s][0]):
            return BIG
    return err


def _valid(p: dict) -> bool:
    """The parameter checks of fh_h_batch_create (a candidate outside them,
    e.g. alpha >= 1 after a PSO move, scores 1e300 instead of failing the
    batch)."""
    return (p["N"] >= 2 and p["L"] > 0 and p["tau"] > 0 and 0 < p["alpha"] < 1
            and (p["weights"] == 0 or p["beta"] > 0) and np.isfinite(p["kc"]) and np.isfinite(p["kgam"]))


def _only_valid(run):
    def wrapped(params_list, U0, tau, t_end, values):
        ok = [k for k, p in enumerate(params_list) if _valid(p)]
        out = [BIG] * len(params_list)
        if ok:
            for k, v in zip(ok, run([params_list[k] for k in ok], U0, tau, t_end, values)):
                out[k] = v
        return out
    return wrapped


def gpu_runner(ctx, mode: int | None = None, metric: int = 0):
    """Scores a list of parameter sets as one batch on the GPU."""
    from .solvers import HSolverBatch
    from . import _lib

    @_only_valid
    def run(params_list, U0, tau, t_end, values):
        tts = _schedule(tau, t_end)
        steps = len(tts)
        b = HSolverBatch(ctx, params_list, steps + 1, _lib.FH_H_FP64 if mode is None else mode)
        b.set_u([U0] * len(params_list))
        # steps whose interval holds a measurement: states before and after them
        need = {s for s, tt in enumerate(tts) for (T, _, _) in values if T >= tt and T < tt + tau}
        before = [[None] * steps for _ in params_list]
        after = [[None] * steps for _ in params_list]
        done = 0
        for s in sorted(need):
            if s > done:
                b.calc_step(s - done)
                done = s
            cur = b.get_u()
            b.calc_step(1)
            done += 1
            nxt = b.get_u()
            for k in range(len(params_list)):
                before[k][s], after[k][s] = cur[k], nxt[k]
        if done < steps:
            b.calc_step(steps - done)
        last = b.get_u()
        b.close()
        out = []
        for k, p in enumerate(params_list):
            N, dL = p["N"], p["L"] / p["N"]
            for s in range(steps):  # steps without measurements only need finiteness
                if after[k][s] is None:
                    after[k][s] = last[k] if s == steps - 1 else np.zeros(1)
            out.append(_score(before[k], after[k], tts, tau, dL, N, values, metric))
            if not np.all(np.isfinite(last[k])):
                out[-1] = BIG
        return out

    return run


def steepest_descent(run, base: dict, keys: list[str], U0: np.ndarray, t_end: float, values,
                     vmax: list[float] | None = None, eps: float = 1e-6, max_iter: int = 20):
    """Fits base[keys] (mt_psi_caputo.cpp:1892-1953).  Returns (params, misfit,
    rounds, solves)."""
    tau = base["tau"]
    vmax = vmax or [0.0] * len(keys)
    p = dict(base)
    solves = 1
    v0 = run([p], U0, tau, t_end, values)[0]
    if v0 == BIG:
        return p, v0, 0, solves
    step, it = 1.0, 0
    while True:
        sts = [step * (vm if vm != 0 else 1.0) for vm in vmax]
        cands = []
        for k, st in zip(keys, sts):
            q = dict(p)
            q[k] = p[k] + st
            cands.append(q)
        vs = run(cands, U0, tau, t_end, values)  # all perturbations in one batch
        solves += len(cands)
        grad = [(v - v0) / st for v, st in zip(vs, sts)]
        sp = dict(p)
        for k, g in zip(keys, grad):
            p[k] = p[k] - step * g
        vnew = run([p], U0, tau, t_end, values)[0]
        solves += 1
        if vnew >= v0:
            p = sp
            step /= 2.0
            if step < eps:
                break
        else:
            if abs(vnew - v0) < eps:
                return p, vnew, it + 1, solves
            v0 = vnew
        if it > max_iter:
            break
        it += 1
    return p, v0, it, solves


def pso(run, base: dict, keys: list[str], bounds: list[tuple[float, float]], U0: np.ndarray, t_end: float, values,
        n: int = 16, omega: float = 0.7, fi_p: float = 1.4, fi_g: float = 1.4, eps: float = 1e-8,
        max_iter: int = 10, seed: int = 0, adaptive: bool = False, restart_prox: float = 0.0, log=None):
    """Particle swarm over base[keys] (the update of mt_psi_caputo.cpp:2183-2223:
    v = omega v + fi_p rp (p_best - x) + fi_g rg (g_best - x), x += v, random
    numbers in steps of 1e-4; stop when the worst particle is within eps of
    the best).  Synchronous: every particle of an iteration moves with the
    global best of the previous iteration and the swarm is scored as one batch
    (the reference scores particles one by one and lets later ones see the
    best found earlier in the same iteration).  ``adaptive`` applies the
    reference's adaptive schedule (mt_psi_caputo.cpp:2093-2179): omega starts
    at 1 and is divided or multiplied by its initial value as the mean
    velocity runs above or below v0 exp(-(2(it+1)/(max_iter-it))^2), and
    per-coordinate fi_p, fi_g follow the velocity spread against the initial
    population's range (clamped to [0, 2]).  After each move a particle
    restarts at a random position with probability (1 - omega) restart_prox
    when omega < 1 (2203-2209; off by default as in the reference).  The
    search also stops once the best misfit is at most eps (2250).  ``log``
    (a text file) receives the reference's log lines (2056-2244):
    "#initial i - f", "#initial best: f x...", then per iteration
    "it avg A best: f x...".  Returns (params, misfit, iterations, solves)."""
    rng = np.random.default_rng(seed)
    rnd = lambda: int(rng.integers(0, 10000)) / 10000.0  # noqa: E731
    tau = base["tau"]
    size = len(keys)
    x = [[lo + (hi - lo) * rnd() for (lo, hi) in bounds] for _ in range(n)]
    v = [[0.0] * size for _ in range(n)]
    cand = lambda xi: dict(base, **dict(zip(keys, xi)))  # noqa: E731
    f = run([cand(xi) for xi in x], U0, tau, t_end, values)
    solves = n
    pb, pf = [xi[:] for xi in x], list(f)
    g = int(np.argmin(f))
    gb, gf = x[g][:], f[g]
    if log is not None:
        for i in range(n):
            log.write("#initial %d - %g\n" % (i, f[i]))
        log.write("#initial best: " + "".join("%2.2g " % z for z in [gf] + gb) + "\n")
    fp, fg = [fi_p] * size, [fi_g] * size
    clamp = lambda a: min(2.0, max(0.0, a))  # noqa: E731
    if adaptive:
        xa = np.asarray(x)
        v0 = float(np.sqrt(np.sum(xa * xa))) / n  # the reference measures positions here
        v0v = np.sqrt(np.sum(xa * xa, axis=0)) / n
        vmax = [(xa[:, j].max() - xa[:, j].min()) / fi_g for j in range(size)]
        vmax = [vm if vm != 0.0 else 1.0 / fi_g for vm in vmax]
        ad_p, ad_c = omega, fi_p
        omega = 1.0
        fp = [clamp(ad_c * v0v[j] / vmax[j]) for j in range(size)]
        fg = [clamp(ad_c * (1 - v0v[j] / vmax[j])) for j in range(size)]
    it = 0
    for it in range(1, max_iter + 1):
        if adaptive:
            q = np.float32(2 * it) / np.float32(max_iter - (it - 1))  # float arithmetic, as the reference
            ve = v0 * float(np.exp(-float(q * q)))
            va = np.asarray(v)
            vavg = float(np.sqrt(np.sum(va * va))) / n
            vavgc = np.sqrt(np.sum(va * va, axis=0)) / n
            if vavg > ve:
                omega /= ad_p
            if vavg < ve:
                omega *= ad_p
            omega = clamp(omega)
            fp = [clamp(ad_c * vavgc[j] / vmax[j]) for j in range(size)]
            fg = [clamp(ad_c * (1 - vavgc[j] / vmax[j])) for j in range(size)]
        for i in range(n):
            for j in range(size):
                rp, rg = rnd(), rnd()
                v[i][j] = omega * v[i][j] + fp[j] * rp * (pb[i][j] - x[i][j]) + fg[j] * rg * (gb[j] - x[i][j])
            for j in range(size):
                x[i][j] += v[i][j]
            if rnd() < ((1.0 - omega) if omega < 1.0 else 0.0) * restart_prox:
                x[i] = [lo + (hi - lo) * rnd() for (lo, hi) in bounds]
        f = run([cand(xi) for xi in x], U0, tau, t_end, values)  # the swarm in one batch
        solves += n
        for i in range(n):
            if f[i] < pf[i]:
                pb[i], pf[i] = x[i][:], f[i]
            if f[i] < gf:
                gb, gf = x[i][:], f[i]
        if log is not None:
            log.write("%d avg %g best: " % (it - 1, sum(f) / n) + "".join("%g " % z for z in [gf] + gb) + "\n")
        if max(f) - gf < eps or gf <= eps:
            break
    return cand(gb), gf, it, solves
