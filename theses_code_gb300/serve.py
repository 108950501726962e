"""Request loop for streams of fractional-history solves (continuous batching).

Requests are 1D H_solver solves (L1 or psi-Caputo, any N) and 2D TG_solver
solves, each with its own step count.  The loop
  * admits requests in arrival order while their history fits the device
    memory budget (history bytes = state doubles x steps x 8, plus working
    buffers), so new work starts as soon as finished work frees memory;
  * groups every admitted 1D request waiting at a scheduling point into a new
    cohort (one HSolverBatch, one CUDA stream); cohorts started at different
    times run side by side, so their GPU work overlaps;
  * gives each 2D request its own TGSolver and stream;
  * advances every active solver by at most `chunk` steps per pass, stopping a
    cohort exactly at each member's own step count to read that member back;
  * records per-request latency = completion time - arrival time.
All GPU work goes through the libfhist C ABI; this module only schedules.
"""
from __future__ import annotations

import dataclasses
import time
from collections import deque

import numpy as np

from . import _lib
from ._lib import Context
from .solvers import HSolverBatch, TGSolver


@dataclasses.dataclass
class Request:
    rid: int
    kind: str            # "1d" or "2d"
    steps: int
    arrival: float       # seconds after the stream start
    params: dict
    U0: np.ndarray | None = None         # 1D initial state (N+2)
    V2: np.ndarray | None = None         # 2D |v|^2
    C0: np.ndarray | None = None         # 2D initial field
    mode: int = _lib.FH_TG_FP64          # 2D history mode

    def history_bytes(self) -> int:
        if self.kind == "1d":
            n = self.params["N"] + 2
            return 8 * n * (self.steps + 1) + 8 * n * 12
        P = (self.params["sN"] + 2) * (self.params["M"] + 2)
        extra = 8 * P * 40 + 16 * self.steps * self.steps  # fields, factors, partials, weight table
        if self.mode == _lib.FH_TG_BLOCKED:
            extra += 8 * P * self.steps + 8 * P * 128  # four bf16 slices per history value
        return 8 * P * self.steps + extra


@dataclasses.dataclass
class Done:
    rid: int
    latency: float
    result: np.ndarray


class _Cohort:
    def __init__(self, device: int, reqs: list[Request]):
        self.ctx = Context(device)
        self.ctx.set_graphs(False)  # chunked stepping: no one-shot graph captures
        self.reqs = sorted(reqs, key=lambda r: r.steps)
        self.solver = HSolverBatch(self.ctx, [r.params for r in self.reqs], self.reqs[-1].steps + 1)
        self.solver.set_u([r.U0 for r in self.reqs])
        self.order = {r.rid: i for i, r in enumerate(self.reqs)}
        self.done_steps = 0
        self.next_member = 0
        self.bytes = sum(r.history_bytes() for r in self.reqs)

    def advance(self, chunk: int):
        target = min(self.reqs[self.next_member].steps, self.done_steps + chunk)
        if target > self.done_steps:
            self.solver.calc_step(target - self.done_steps)
            self.done_steps = target

    def collect(self, now_fn) -> list[Done]:
        out = []
        while self.next_member < len(self.reqs) and self.reqs[self.next_member].steps == self.done_steps:
            i = self.next_member
            u = self.solver.get_u_range(i, 1)[0]
            r = self.reqs[i]
            out.append(Done(r.rid, now_fn() - r.arrival, u))
            self.next_member += 1
        return out

    @property
    def finished(self):
        return self.next_member == len(self.reqs)

    def close(self):
        self.solver.close()
        self.ctx.close()


class _Single2D:
    def __init__(self, device: int, r: Request):
        self.ctx = Context(device)
        self.ctx.set_graphs(False)
        self.r = r
        self.solver = TGSolver(self.ctx, r.params, r.steps, r.mode)
        self.solver.set_state(r.V2, r.C0)
        self.done_steps = 0
        self.bytes = r.history_bytes()
        self.finished = False

    def advance(self, chunk: int):
        n = min(chunk, self.r.steps - self.done_steps)
        if n > 0:
            self.solver.calc_step(n)
            self.done_steps += n

    def collect(self, now_fn) -> list[Done]:
        if self.done_steps == self.r.steps and not self.finished:
            c = self.solver.get_c()
            self.finished = True
            return [Done(self.r.rid, now_fn() - self.r.arrival, c)]
        return []

    def close(self):
        self.solver.close()
        self.ctx.close()


class Server:
    def __init__(self, budget_bytes: float, device: int = 0, chunk: int = 250, max_cohort: int = 1024,
                 max_active: int = 16):
        self.budget = float(budget_bytes)
        self.device = device
        self.chunk = chunk
        self.max_cohort = max_cohort
        self.max_active = max_active

    def run(self, requests: list[Request], realtime: bool = True) -> tuple[list[Done], dict]:
        """Serves `requests` (sorted by arrival).  With realtime=True arrivals
        follow the wall clock; otherwise all requests are present at t = 0."""
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting: deque[Request] = deque()
        active: list = []
        done: list[Done] = []
        used = 0.0
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        for r in requests:
            if r.history_bytes() > self.budget:
                raise ValueError(f"request {r.rid} needs {r.history_bytes()} B > budget {self.budget}")
        peak_active, passes = 0, 0
        while pending or waiting or active:
            t = now() if realtime else float("inf")
            while pending and pending[0].arrival <= t:
                waiting.append(pending.popleft())
            # admission in arrival order, limited by memory and the number of streams
            cohort: list[Request] = []
            cohort_bytes = 0.0
            while waiting and len(active) + (1 if cohort else 0) < self.max_active:
                r = waiting[0]
                b = r.history_bytes()
                if used + cohort_bytes + b > self.budget:
                    break
                waiting.popleft()
                if r.kind == "2d":
                    active.append(_Single2D(self.device, r))
                    used += b
                else:
                    cohort.append(r)
                    cohort_bytes += b
                    if len(cohort) >= self.max_cohort:
                        break
            if cohort:
                active.append(_Cohort(self.device, cohort))
                used += cohort_bytes
            peak_active = max(peak_active, len(active))
            if not active:
                if pending and realtime:
                    time.sleep(max(0.0, min(0.001, pending[0].arrival - now())))
                continue
            # enqueue the next chunk on every active solver (asynchronous, one stream each)
            for a in active:
                a.advance(self.chunk)
            passes += 1
            # collect results as streams finish; retire finished solvers
            still = []
            for a in active:
                done.extend(a.collect(now))
                if a.finished:
                    used -= a.bytes
                    a.close()
                else:
                    still.append(a)
            active = still
        lat = np.array([d.latency for d in done]) if done else np.zeros(1)
        stats = {"requests": len(done), "wall_s": now(), "p50_s": float(np.percentile(lat, 50)),
                 "p99_s": float(np.percentile(lat, 99)), "solves_per_s": len(done) / max(now(), 1e-9),
                 "peak_active_solvers": peak_active, "scheduler_passes": passes}
        return done, stats


def make_mix(n: int, rate: float = 2000.0, seed: int = 3, max_2d: int = 512, steps=(500, 5000),
             nrange=(64, 2048), frac_2d: float = 0.4, mode_2d: int = _lib.FH_TG_FP64) -> list[Request]:
    """Poisson stream of mixed solves: 60 % 1D (L1 or psi-Caputo, N in nrange),
    40 % 2D (grids 64^2 .. max_2d^2), alpha in [0.5, 0.95], steps in `steps`."""
    from . import workloads
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    for rid in range(n):
        t += rng.exponential(1.0 / rate)
        steps_i = int(rng.integers(steps[0], steps[1] + 1))
        alpha = float(rng.uniform(0.5, 0.95))
        if rng.uniform() < frac_2d:
            g = int(rng.integers(min(64, max_2d), max_2d + 1))
            p, V2, C0 = workloads.convection_2d(g, g, alpha=alpha, tau=5e-4, d=0.1, seed=int(rng.integers(1 << 30)))
            reqs.append(Request(rid, "2d", steps_i, t, p, V2=V2, C0=C0, mode=mode_2d))
        else:
            N = int(rng.integers(nrange[0], nrange[1] + 1))
            psi = rng.uniform() < 0.5
            p = dict(N=N, L=1.0, tau=1e-3, alpha=alpha, weights=_lib.FH_W_PSI if psi else _lib.FH_W_L1,
                     beta=float(rng.uniform(0.5, 2.0)) if psi else 1.0, kmodel=_lib.FH_K_CONST, kc=1.0, kgam=0.0,
                     cinv=1.0, gravity=0, al_left=0.0, bt_left=0.0, u_right=0.0)
            x = np.arange(N + 2) / N
            U0 = np.sin(np.pi * x)
            U0[N:] = 0.0
            reqs.append(Request(rid, "1d", steps_i, t, p, U0=U0))
    return reqs
