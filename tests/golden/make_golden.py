"""Generate golden fixtures by running the reference solvers (harnesses in
oracle/ref/, compiled from the read-only reference sources into oracle/_ref/).

Run in a container that has the reference checked out:
    make -C oracle/ref && python tests/golden/make_golden.py
The fixtures (small JSON files) are committed; tests never need the reference.
"""
from __future__ import annotations

import json
import math
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(REPO, "oracle", "_ref")


def run(exe, args, stdin_vals=None, timeout=600):
    inp = None
    if stdin_vals is not None:
        inp = " ".join(repr(float(v)) for v in stdin_vals) + "\n"
    out = subprocess.run([os.path.join(REF, exe)] + [str(a) for a in args], input=inp,
                         capture_output=True, text=True, timeout=timeout, check=True)
    return out.stdout


def parse(out):
    res = {}
    for line in out.splitlines():
        parts = line.split()
        if not parts:
            continue
        key = parts[0]
        vals = [float(x) for x in parts[1:]]
        res.setdefault(key, []).append(vals)
    return res


def dump(name, obj):
    path = os.path.join(HERE, name)
    with open(path, "w") as f:
        json.dump(obj, f, indent=None, separators=(",", ":"))
    print("wrote", path, os.path.getsize(path), "bytes")


def h_solver_case(exe, name, BS, NB, L, tau, alpha, k, steps, hb, extra=()):
    N = BS * NB
    U0 = [-20.0 - 1.5 * math.sin(math.pi * i / N) - 0.3 * math.sin(3 * math.pi * i / N) for i in range(N + 1)]
    res = parse(run(exe, [BS, NB, L, tau, alpha, k, steps, hb, *extra], U0))
    dump(name, {"reference": exe, "BS": BS, "NB": NB, "N": N, "L": L, "tau": tau, "alpha": alpha,
                "k": k, "steps": steps, "Hbottom": hb, "extra": list(extra), "U0": U0,
                "uc": res["uc"][0][0], "U": res["u"][0]})


def main():
    if not os.path.isdir(REF):
        sys.exit("build the harnesses first: make -C oracle/ref")
    # 1D H_solver, L1 weights (mt_minimal.cpp)
    h_solver_case("h_minimal", "h_minimal_l1.json", 10, 2, 3.0, 600.0, 0.8, 1e-4, 40, -20.0)
    # 1D H_solver, psi = t (mt_psi_caputo.cpp, func_in_kernel 0)
    h_solver_case("h_psi", "h_psi_t.json", 10, 2, 3.0, 600.0, 0.8, 1e-4, 40, -20.0, (0, 1.0, 1e-15))
    # 1D H_solver, psi = t^0.7 (func_in_kernel 3) with the series converged (eps 1e-15)
    h_solver_case("h_psi", "h_psi_t07.json", 5, 2, 3.0, 600.0, 0.75, 1e-4, 24, -20.0, (3, 0.7, 1e-15))
    h_solver_case("h_psi", "h_psi_t15.json", 5, 2, 3.0, 600.0, 0.6, 1e-4, 24, -20.0, (3, 1.5, 1e-15))
    # space-fractional derivative in z (gamma < 1, calc_v non-zero)
    h_solver_case("h_minimal", "h_minimal_space.json", 10, 2, 3.0, 600.0, 0.8, 1e-4, 40, -20.0, (0, 1.0, 1e-15, 0.7))
    h_solver_case("h_psi", "h_psi_space.json", 10, 2, 3.0, 600.0, 0.8, 1e-4, 40, -20.0, (0, 1.0, 1e-15, 0.75))
    h_solver_case("h_psi", "h_psi_t07_space.json", 5, 2, 3.0, 600.0, 0.75, 1e-4, 24, -20.0, (3, 0.7, 1e-15, 0.6))
    # psi-Caputo weights from the reference series (calc_int, mt_psi_caputo.cpp:720-741)
    wres = {}
    for (alpha, beta) in [(0.7, 0.6), (0.6, 1.5), (0.9, 2.0), (0.55, 0.8)]:
        r = parse(run("psi_weights", [alpha, beta, 0.01, 1e-15, 1, 24]))
        wres[f"{alpha}_{beta}"] = {"alpha": alpha, "beta": beta, "tau": 0.01,
                                   "w": [[int(a), int(t0), v] for a, t0, v in r["w"]]}
    dump("psi_weights.json", wres)
    # 2D ADI (fr_d_t_g_2d.cpp TG_solver_<0,1,0>)
    rng = np.random.default_rng(1234)
    sN, M = 12, 10
    P = (sN + 2) * (M + 2)
    ii, jj = np.meshgrid(np.arange(sN + 2), np.arange(M + 2), indexing="xy")  # shape (M+2, sN+2): idx = i + j*(sN+2)
    V2 = (0.25 + 0.7 * (0.5 + 0.5 * np.sin(0.7 * ii + 1.3) * np.cos(0.5 * jj - 0.2))) ** 2
    C0 = np.exp(-(((ii - 6.0) / 3.0) ** 2 + ((jj - 5.0) / 2.5) ** 2))
    V2 = V2.reshape(-1)
    C0 = C0.reshape(-1)
    args = [sN, M, 5e-3, 0.7, 0.1, 0.3, 0.05, 12]
    res = parse(run("tg", args, list(V2) + list(C0)))
    dL, dLx, sigma = res["geom"][0]
    dump("tg_adi.json", {"sN": sN, "M": M, "tau": 5e-3, "alpha": 0.7, "d": 0.1, "C1": 0.3, "S": 0.05,
                         "steps": 12, "dL": dL, "dLx": dLx, "sigma": sigma, "V2": list(V2),
                         "C0": list(C0), "C": res["c"][0]})
    # the same problem with restricted summing (dt_alg 2): 40 steps, the sums
    # stop at the first weight below 0.012 (about 12 layers back)
    res = parse(run("tg", args[:7] + [40, 2, 0.012], list(V2) + list(C0)))
    dump("tg_adi_restricted.json", {"sN": sN, "M": M, "tau": 5e-3, "alpha": 0.7, "d": 0.1, "C1": 0.3, "S": 0.05,
                                    "steps": 40, "dt_alg": 2, "dt_eps": 0.012, "dL": dL, "dLx": dLx,
                                    "sigma": sigma, "V2": list(V2), "C0": list(C0), "C": res["c"][0]})
    res = parse(run("tg", args[:7] + [40], list(V2) + list(C0)))
    dump("tg_adi_40.json", {"C": res["c"][0]})
    # series expansion (dt_alg 3, psi = t): 12 terms, 40 steps
    res = parse(run("tg", args[:7] + [40, 3, 12], list(V2) + list(C0)))
    dump("tg_adi_series.json", {"steps": 40, "dt_alg": 3, "dt_eps": 12, "C": res["c"][0]})
    # two-series approximation (dt_alg 4, psi = t): 150 steps at alpha 0.7 and
    # 300 steps at alpha 0.9 (tens of long and short approximations per point)
    two = {}
    for alpha, steps in ((0.7, 150), (0.9, 300)):
        a4 = [sN, M, 5e-3, alpha, 0.1, 0.3, 0.05, steps, 4, 1e-8]
        two[f"{alpha}_{steps}"] = {"alpha": alpha, "steps": steps, "C": parse(run("tg", a4, list(V2) + list(C0)))["c"][0]}
    dump("tg_adi_two_series.json", two)
    # TG_solver_ variants: the mass-exchange stage N1 (massN) and the
    # velocity-dependent diffusion coefficient (TG_solver_<0,0,0>), 40 steps
    var = {}
    for key, extra in (("massN", [0, 0.0, 1, 0.5, 2.0]), ("variable_d", [0, 0.0, 0, 0.1, 0.1, 0]),
                       ("variable_d_massN", [0, 0.0, 1, 0.3, 0.7, 0])):
        r = parse(run("tg", args[:7] + [40] + extra, list(V2) + list(C0)))
        var[key] = {"steps": 40, "massN": extra[2], "massN_a": extra[3], "massN_b": extra[4],
                    "fixed_d": extra[5] if len(extra) > 5 else 1, "dcoef": r["dcoef"][0], "C": r["c"][0]}
    dump("tg_adi_variants.json", var)
    # Atangana-Baleanu: Mittag-Leffler values, lag weights, solve_and_check error
    ml = []
    for (a, b, z) in [(0.5, 1.0, -0.7), (0.8, 1.0, -1.2), (0.6, 2.0, -0.9), (0.9, 5.0, -0.5),
                      (0.5, 5.0, -0.3), (1.0, 1.0, -2.0), (1.0, 1.0, 0.5), (0.7, 1.0, 0.4)]:
        r = parse(run("ab", ["ml", a, b, z, 1e-15]))
        ml.append([a, b, z, r["ml"][0][0]])
    r = parse(run("ab", ["abw", 0.5, 0.01, 50]))
    abw = [[int(l), v] for l, v in r["abw"]]
    # solve_and_check (full history, simple 1): error and the field of the last step
    solves = []
    for (a, T, n, m) in [(0.5, 0.5, 50, 10), (0.6, 1.0, 200, 64)]:
        ii = parse(run("ab", ["ii", a, T / n]))["ii"][0][0]
        r = parse(run("ab", ["field", a, T, n, m]))
        c = [v for _, v in sorted((int(j), v) for j, v in r["c"])]
        assert len(c) == m + 1
        lag = [v for _, v in sorted((int(L), v) for L, v in parse(run("ab", ["ablag", a, T / n, n]))["ablag"])]
        solves.append({"alpha": a, "T": T, "n": n, "m": m, "ii": ii, "err": r["err"][0][0], "C": c, "lagw": lag})
    dump("ab.json", {"ml": ml, "abw": {"alpha": 0.5, "tau": 0.01, "n": 50, "w": abw},
                     "solve": solves[0], "solve2": solves[1]})


if __name__ == "__main__":
    main()
