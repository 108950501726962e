"""Request loop for streams of fractional-history solves (continuous batching).

Requests are 1D H_solver solves (L1 or psi-Caputo, any N) and 2D TG_solver
solves, each with its own step count.  The loop
  * keeps 1D requests in pools: one HSolverBatch whose instances are slots,
    each slot holding one request at a time on the request's own clock
    (fh_h_batch_restart).  A request that arrives while a pool runs takes a
    free slot that holds its N at the next scheduling pass, if the pool's step
    capacity covers its steps; a finished request's slot (and so its history
    memory) goes to the next request at once.  Requests that fit no free
    slot open a new pool when the memory budget allows;
  * gives each 2D request its own TGSolver;
  * charges every solver the device bytes it allocates (an upper estimate
    before creation, checked against the solver's own count after it), so
    the budget holds what the device holds;
  * runs every active solver on its own stream from a pool of contexts made
    once, so their GPU work overlaps;
  * advances each solver by at most `chunk` steps per pass, stopping a pool
    exactly when one of its requests reaches its step count, and records
    per-request latency = completion time - arrival time.
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

_MIB = 1 << 20


def _even(n: int) -> int:
    return n + (n & 1)


def pool_bytes(caps: list[int], max_steps: int) -> int:
    """Upper estimate of the device bytes of a 1D batch (FP64 or DF64
    history: 8 bytes per stored value either way) with instance node counts
    `caps` and `max_steps` history slots: the allocations of
    fh_h_batch_create (state and line buffers, history, weight rows, tables,
    64 partial-sum buffers)."""
    n = len(caps)
    Ptot = sum(_even(c + 2) for c in caps)
    b = 8 * Ptot * (7 + 64 + max_steps)
    b += 24 * n * (max_steps + 1) + 8 * 164 * n + 16 * (max_steps + 2) + 16 * n
    b += 256 * n + 3 * 12 * (Ptot // 256 + n + 1)
    return int(b) + 2 * _MIB


def tg_bytes(sN: int, M: int, steps: int, mode: int) -> int:
    """Upper estimate of the device bytes of a 2D solver (fh_tg_create)."""
    P = (sN + 2) * (M + 2)
    P += P & 1
    fld = 8 * P
    wt = steps if steps <= 4096 else 1
    b = 13 * fld + fld * steps + 16 * steps * wt + 32 * wt + 16 * fld
    if mode == _lib.FH_TG_BLOCKED:
        b += 12 * fld + 32 * fld + 64
        if steps > 64:
            Ppad = -(-P // 128) * 128
            Kcap = -(-steps // 64) * 64
            b += 8 * Ppad * Kcap + 8 * 128 * Kcap + Ppad * (Kcap // 64) + 128 * (Kcap // 64) + 1024 * Ppad + 8
            # split-K partial rows when the 64-point tiles are fewer than the
            # SMs (at most 8 splits; 160 SMs bounds the device's 152)
            ntiles = Ppad // 64
            if ntiles < 160:
                b += 8 * min(8, 160 // ntiles) * 128 * Ppad
    return int(b) + 2 * _MIB


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

    def device_bytes(self) -> int:
        """Device bytes of a solver for this request alone."""
        if self.kind == "1d":
            return pool_bytes([self.params["N"]], self.steps + 1)
        return tg_bytes(self.params["sN"], self.params["M"], self.steps, self.mode)


@dataclasses.dataclass
class Done:
    rid: int
    latency: float
    result: np.ndarray


class _Pool1D:
    """One HSolverBatch of slots.  Slot i holds node counts up to caps[i];
    its occupant (occ[i]) ends at pool step end[i]."""

    def __init__(self, ctx: Context, reqs: list[Request], quantum: int, step_factor: float, min_slots: int):
        self.ctx = ctx
        caps = [max(2, -(-r.params["N"] // quantum) * quantum) for r in reqs]
        # spare slots for later arrivals, sized like the largest first occupant
        while len(caps) < min_slots:
            caps.append(max(caps))
        self.caps = caps
        self.max_steps = int(max(r.steps for r in reqs) * step_factor) + 1
        base = dict(reqs[0].params)
        shapes = [dict(base, N=c) for c in caps]
        self.solver = HSolverBatch(ctx, shapes, self.max_steps)
        self.bytes = self.solver.device_bytes()
        zeros = [np.zeros(c + 2) for c in caps]
        self.solver.set_u(zeros)
        self.occ: list[Request | None] = [None] * len(caps)
        self.end = [0] * len(caps)
        self.done_steps = 0
        # largest first: each takes the smallest free slot that holds it
        for r in sorted(reqs, key=lambda q: -q.params["N"]):
            assert self.place(r)

    def fits(self, r: Request) -> int:
        """Index of the smallest free slot that holds r, or -1."""
        if self.done_steps + r.steps > self.max_steps - 1:
            return -1
        best = -1
        for i, (c, o) in enumerate(zip(self.caps, self.occ)):
            if o is None and c >= r.params["N"] and (best < 0 or c < self.caps[best]):
                best = i
        return best

    def place(self, r: Request) -> bool:
        i = self.fits(r)
        if i < 0:
            return False
        self.solver.restart(i, r.params, r.U0)
        self.occ[i] = r
        self.end[i] = self.done_steps + r.steps
        return True

    def advance(self, chunk: int):
        live = [e for e, o in zip(self.end, self.occ) if o is not None]
        if not live:
            return
        n = min(chunk, min(live) - self.done_steps)
        if n > 0:
            self.solver.calc_step(n)
            self.done_steps += n

    def collect(self, now_fn) -> list[Done]:
        out = []
        for i, o in enumerate(self.occ):
            if o is not None and self.end[i] == self.done_steps:
                u = self.solver.get_u_range(i, 1)[0]
                out.append(Done(o.rid, now_fn() - o.arrival, u))
                self.occ[i] = None
        return out

    @property
    def finished(self) -> bool:
        return all(o is None for o in self.occ)

    def close(self):
        self.solver.close()


class _Single2D:
    def __init__(self, ctx: Context, r: Request):
        self.ctx = ctx
        self.r = r
        self.solver = TGSolver(ctx, r.params, r.steps, r.mode)
        self.bytes = self.solver.device_bytes()
        self.solver.set_state(r.V2, r.C0)
        self.done_steps = 0
        self.finished = False

    def fits(self, r: Request) -> int:
        return -1

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


class Server:
    """budget_bytes: device memory for all solvers together; max_active:
    streams (contexts, made once); chunk: steps per solver per pass;
    max_pool: requests that open one pool together; quantum: slot node counts
    are rounded up to it; step_factor: a pool's step capacity over its
    longest first request (room for later occupants); min_slots: slots of a
    new pool (spares take later arrivals)."""

    def __init__(self, budget_bytes: float, device: int = 0, chunk: int = 250, max_pool: int = 1024,
                 max_active: int = 16, quantum: int = 64, step_factor: float = 2.0, min_slots: int = 16):
        self.budget = float(budget_bytes)
        self.device = device
        self.chunk = chunk
        self.max_pool = max_pool
        self.max_active = max_active
        self.quantum = quantum
        self.step_factor = step_factor
        self.min_slots = min_slots

    def _pool_estimate(self, reqs: list[Request]) -> int:
        caps = [max(2, -(-r.params["N"] // self.quantum) * self.quantum) for r in reqs]
        while len(caps) < self.min_slots:
            caps.append(max(caps))
        return pool_bytes(caps, int(max(r.steps for r in reqs) * self.step_factor) + 1)

    def run(self, requests: list[Request], realtime: bool = True) -> tuple[list[Done], dict]:
        """Serves `requests`.  With realtime=True arrivals follow the wall
        clock; otherwise all requests are present at t = 0."""
        for r in requests:
            if r.device_bytes() > self.budget:
                raise ValueError(f"request {r.rid} needs {r.device_bytes()} B > budget {self.budget}")
        pending = deque(sorted(requests, key=lambda r: r.arrival))
        waiting: list[Request] = []
        active: list = []
        done: list[Done] = []
        free_ctx = [Context(self.device) for _ in range(self.max_active)]
        for c in free_ctx:
            c.set_graphs(False)  # chunked stepping: no one-shot graph captures
        all_ctx = list(free_ctx)
        used = 0.0
        peak_used = 0.0
        t0 = time.perf_counter()

        def now():
            return time.perf_counter() - t0

        peak_active, passes, joined = 0, 0, 0
        try:
            while pending or waiting or active:
                t = now() if realtime else float("inf")
                while pending and pending[0].arrival <= t:
                    waiting.append(pending.popleft())
                # 1) 1D requests into free slots of running pools (any order: a
                #    slot that holds one request may not hold the one before it)
                rest = []
                for r in waiting:
                    pool = None
                    if r.kind == "1d":
                        pool = next((a for a in active if isinstance(a, _Pool1D) and a.fits(r) >= 0), None)
                    if pool is not None:
                        pool.place(r)
                        joined += 1
                    else:
                        rest.append(r)
                waiting = rest
                # 2) new solvers in arrival order while memory and streams allow
                while waiting and free_ctx:
                    r = waiting[0]
                    if r.kind == "2d":
                        est = tg_bytes(r.params["sN"], r.params["M"], r.steps, r.mode)
                        if used + est > self.budget:
                            break
                        waiting.pop(0)
                        a = _Single2D(free_ctx.pop(), r)
                    else:
                        group = [x for x in waiting if x.kind == "1d"][: self.max_pool]
                        while group and used + self._pool_estimate(group) > self.budget:
                            group.pop()
                        if not group or group[0] is not r:
                            break
                        est = self._pool_estimate(group)
                        ids = {x.rid for x in group}
                        waiting = [x for x in waiting if x.rid not in ids]
                        a = _Pool1D(free_ctx.pop(), group, self.quantum, self.step_factor, self.min_slots)
                    assert a.bytes <= est, (a.bytes, est)  # the estimate bounds the allocation
                    used += a.bytes
                    active.append(a)
                peak_active = max(peak_active, len(active))
                peak_used = max(peak_used, used)
                if not active:
                    if pending and realtime:
                        time.sleep(max(0.0, min(0.001, pending[0].arrival - now())))
                    continue
                # 3) the next chunk on every active solver (asynchronous, one stream each)
                for a in active:
                    a.advance(self.chunk)
                passes += 1
                # 4) results as streams finish; free slots go to waiting 1D
                #    requests on the next pass; empty pools and finished 2D
                #    solvers are retired
                still = []
                for a in active:
                    done.extend(a.collect(now))
                    if a.finished and not (isinstance(a, _Pool1D) and any(
                            r.kind == "1d" and a.fits(r) >= 0 for r in waiting)):
                        used -= a.bytes
                        a.close()
                        free_ctx.append(a.ctx)
                    else:
                        still.append(a)
                active = still
        finally:
            for a in active:
                a.close()
            for c in all_ctx:
                c.close()
        lat = np.array([d.latency for d in done]) if done else np.zeros(1)
        stats = {"requests": len(done), "wall_s": now(), "p50_s": float(np.percentile(lat, 50)),
                 "p99_s": float(np.percentile(lat, 99)), "solves_per_s": len(done) / max(now(), 1e-9),
                 "peak_active_solvers": peak_active, "scheduler_passes": passes,
                 "joined_running_pools": joined, "peak_device_bytes": peak_used}
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
