"""The reference's fitting input file (``fit_input.txt``) and initial profile.

``read_fit_input`` follows the read sequence of mt_minimal.cpp:1955-2043
(the same layout as mt_psi_caputo.cpp:2652-2766):

    to_fit nvalues ninit ncheck nperc nirr nEV_T nEV_F ev_mu
    pso_n pso_o pso_fi_p pso_fi_g pso_eps pso_max_iter
    nvalues lines  T Z F        (F scaled by Hmult)
    ninit lines    Z F          (F scaled by Hmult)
    nperc lines    T A          (precipitation)
    nirr lines     T A          (irrigation)
    ncheck lines   T Z F        (F scaled by Hmult)
    nEV_T lines    T LAI EV_F[0..nEV_F-1]
    up to 20 fixed parameter values

Fields are whitespace-separated numbers, as ``fscanf`` reads them.
``initial_profile`` is the linear interpolation of the initial heads onto the
nodes (mt_psi_caputo.cpp:1700-1733), with linear extrapolation beyond the
first and last depth when more than two depths are given.  ``fit_problem``
turns a file into the inputs of ``fit.steepest_descent`` / ``fit.pso``; the
precipitation, irrigation and evapotranspiration series drive model terms
the batched solver does not have, so a file that uses them is refused.
"""
from __future__ import annotations

import numpy as np

HMULT = 10.0  # the reference's Hmult (mt_psi_caputo.cpp:212)


def read_fit_input(path: str, hmult: float = HMULT) -> dict:
    tok = open(path).read().split()
    pos = 0

    def take(n, conv=float):
        nonlocal pos
        if pos + n > len(tok):
            raise ValueError(f"{path}: truncated at token {pos}")
        out = [conv(t) for t in tok[pos:pos + n]]
        pos += n
        return out

    to_fit, nvalues, ninit, ncheck, nperc, nirr, nEV_T, nEV_F = take(8, int)
    (ev_mu,) = take(1)
    pso_n, = take(1, int)
    pso_o, pso_fi_p, pso_fi_g, pso_eps = take(4)
    pso_max_iter, = take(1, int)
    r = {"to_fit": to_fit, "ev_mu": ev_mu,
         "pso": {"n": pso_n, "omega": pso_o, "fi_p": pso_fi_p, "fi_g": pso_fi_g, "eps": pso_eps,
                 "max_iter": pso_max_iter}}
    v = np.array(take(3 * nvalues)).reshape(nvalues, 3)
    v[:, 2] *= hmult
    r["values"] = [tuple(x) for x in v]
    ini = np.array(take(2 * ninit)).reshape(ninit, 2)
    ini[:, 1] *= hmult
    r["init_Z"], r["init_F"] = ini[:, 0].copy(), ini[:, 1].copy()
    r["perc"] = np.array(take(2 * nperc)).reshape(nperc, 2)
    r["irr"] = np.array(take(2 * nirr)).reshape(nirr, 2)
    c = np.array(take(3 * ncheck)).reshape(ncheck, 3)
    c[:, 2] *= hmult
    r["check"] = [tuple(x) for x in c]
    ev = np.array(take((2 + nEV_F) * nEV_T)).reshape(nEV_T, 2 + nEV_F)
    r["EV_T"], r["LAI"], r["EV_F"] = ev[:, 0].copy(), ev[:, 1].copy(), ev[:, 2:].T.copy()
    r["param_values"] = [float(t) for t in tok[pos:pos + 20]]
    return r


def initial_profile(init_Z, init_F, N: int, dL: float) -> np.ndarray:
    """U[0..N] from the (Z, F) pairs (mt_psi_caputo.cpp:1700-1733)."""
    Z, F = list(init_Z), list(init_F)
    n = len(Z)
    U = np.empty(N + 1)
    for i in range(N + 1):
        x = i * dL
        v = F[0]
        if x >= Z[0]:
            j = 1
            while j < n:
                if Z[j - 1] <= x < Z[j]:
                    k = (x - Z[j - 1]) / (Z[j] - Z[j - 1])
                    v = (1.0 - k) * F[j - 1] + k * F[j]
                    break
                j += 1
            if j == n:
                v = F[n - 1]
                if n > 2:
                    v += (x - Z[n - 1]) * ((F[n - 1] - F[n - 2]) / (Z[n - 1] - Z[n - 2]))
        elif n > 2:
            v -= (Z[0] - x) * ((F[1] - F[0]) / (Z[1] - Z[0]))
        U[i] = v
    return U


def fit_problem(inp: dict, base: dict):
    """(U0, t_end, values) for the fitting drivers from a parsed file and the
    solver parameters ``base`` (N, L, tau, ...): U0 holds N + 2 values (the
    ghost node copies node N), t_end is the latest measurement time."""
    if len(inp["perc"]) or len(inp["irr"]) or inp["EV_F"].size:
        raise NotImplementedError("precipitation, irrigation and evapotranspiration are not modelled by the "
                                  "batched solver")
    N, dL = base["N"], base["L"] / base["N"]
    U = initial_profile(inp["init_Z"], inp["init_F"], N, dL)
    U0 = np.append(U, U[-1])
    t_end = max(T for (T, _, _) in inp["values"])
    return U0, t_end, inp["values"]
