"""The reference's 2D time loop with its result files (fr_d_t_g_2d.cpp
solve(), 4055-4465): several solvers advanced side by side from t = 0 to t
in steps of tau_m, writing

  log2.txt  at every output time (tt >= nout * out_tau, 4354-4432):
            "T <tt> " then per solver "V <C(sN/4, M/2)> t <ms> " and
            " diffs(avgsq,maxabs,global rel for[0,T]) " with, per solver
            after the first, the mean squared and largest difference from
            the first over i <= sN, j <= M and the relative L2 difference
            accumulated over all output times so far;
  log1.txt  at every save time (tt > nsave * save_tau, 4434-4459): per
            node i <= sN the line "<tt> <i dL> " + per solver
            "C(i, M/4) C(i, 2M/4) C(i, 3M/4) " (+ the same of N with the
            mass exchange on).

Both files are appended to, as the reference opens them with "at".  The
time tt of a line is the loop time before the step, as in the reference;
the "t" field is the wall time of that solver's last step in ms.  The loop
advances the solvers in chunks between output and save times (one library
call per chunk); the event times follow the reference's floating-point
accumulation of tt.
"""
from __future__ import annotations

import math
import time

import numpy as np


def event_steps(t: float, save_tau: float, out_tau: float, tau_m: float):
    """The loop times tt and, per step index, whether it outputs / saves."""
    tts, outs, saves = [], [], []
    nout = nsave = 1
    tt = 0.0
    while tt < t:
        o = tt >= nout * out_tau
        s = tt > nsave * save_tau
        tts.append(tt)
        outs.append(o)
        saves.append(s)
        if o:
            nout += 1
        if s:
            nsave += 1
        tt += tau_m
    return tts, outs, saves


def solve(solvers, t: float, save_tau: float, out_tau: float, tau_m: float, log1: str = "log1.txt",
          log2: str = "log2.txt", mass: bool = False) -> int:
    """Runs the solvers (TGSolver objects with their state set) side by side
    and writes log1 / log2; returns the number of steps taken."""
    sN, M = solvers[0].p.sN, solvers[0].p.M
    ld = sN + 2

    def idx(i, j):
        return i + j * ld

    tts, outs, saves = event_steps(t, save_tau, out_tau, tau_m)
    sum_diff2 = sum_s02 = 0.0
    done = 0
    ms = [0] * len(solvers)
    with open(log1, "a") as fi1, open(log2, "a") as fi2:
        for k, tt in enumerate(tts):
            if not (outs[k] or saves[k]):
                continue
            n = k + 1 - done  # steps up to and including step k
            C = []
            for si, s in enumerate(solvers):
                t1 = time.perf_counter()
                s.calc_step(n)
                C.append(s.get_c())
                ms[si] = int(1e3 * (time.perf_counter() - t1) / n)
            done = k + 1
            if outs[k]:
                fi2.write("T %g " % tt)
                for si in range(len(solvers)):
                    fi2.write("V %g t %d " % (C[si][idx(sN // 4, M // 2)], ms[si]))
                fi2.write(" diffs(avgsq,maxabs,global rel for[0,T]) ")
                for si in range(1, len(solvers)):
                    err = mx = 0.0
                    for i in range(sN + 1):
                        for j in range(M + 1):
                            d = C[0][idx(i, j)] - C[si][idx(i, j)]
                            err += d * d
                            sum_diff2 += d * d
                            sum_s02 += C[0][idx(i, j)] * C[0][idx(i, j)]
                            if abs(d) > mx:
                                mx = abs(d)
                    rel1 = math.sqrt(sum_diff2) / math.sqrt(sum_s02) if sum_s02 > 0 else float("nan")
                    err /= sN * M
                    fi2.write("%g %g %g " % (err, mx, rel1))
                fi2.write("\n")
            if saves[k]:
                Ns = [s.get_n() for s in solvers] if mass else None
                for i in range(sN + 1):
                    fi1.write("%g %g " % (tt, i * solvers[0].p.dL))
                    for si in range(len(solvers)):
                        c = C[si]
                        fi1.write("%g %g %g " % (c[idx(i, M * 1 // 4)], c[idx(i, M * 2 // 4)], c[idx(i, M * 3 // 4)]))
                        if mass:
                            nn = Ns[si]
                            fi1.write("%g %g %g " % (nn[idx(i, M * 1 // 4)], nn[idx(i, M * 2 // 4)],
                                                     nn[idx(i, M * 3 // 4)]))
                    fi1.write("\n")
                fi1.flush()
        rest = len(tts) - done
        if rest > 0:
            for s in solvers:
                s.calc_step(rest)
    return len(tts)
