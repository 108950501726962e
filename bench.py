"""Benchmark of the fractional-history hot path on GB300.

Default workload (N=1): the 2D Caputo-Gerasimov convection-diffusion ADI solve
on a 512x512 grid, alpha 0.7, tau 5e-4, 2000 time steps with the full history
(fr_d_t_g_2d.cpp TG_solver path).  One bench step = one complete 2000-step
solve from the initial plume.  Metric: grid-point-steps/s (512*512*2000 per
solve / seconds).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                  [--mode fp64|blocked] [--solve-steps S] [--grid G]

--impl reference times the CPU implementation of the same path (the oracle
port of the reference solver, all host threads) on a bounded sample and prints
the same JSON line with "impl": "reference".
Multi-GPU: replicas only (each rank solves its own instance; no collective on
the data path); value = all ranks' grid-point-steps / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "grid-point-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--mode", default="fp64", choices=["fp64", "blocked"])
    ap.add_argument("--solve-steps", type=int, default=2000)
    ap.add_argument("--grid", type=int, default=512)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-grid", type=int, default=96)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers
class ClockSampler:
    """nvidia-smi clocks/throttle sampling while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            try:
                sm.append(float(s[1]))
                smax.append(float(s[2]))
                for n, v in zip(names, s[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------- CPU baseline
def cpu_baseline(args, threads: int | None = None):
    """Oracle port (C restatement of TG_solver, bit-exact with the reference on
    the golden case) on a reduced grid with the FULL step count, so that the
    per-point history length matches the benchmark workload."""
    from oracle import oracle as O
    from theses_code_gb300 import workloads
    g = args.cpu_grid
    steps = args.solve_steps
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    p, V2, C0 = workloads.convection_2d(g, g, alpha=0.7, tau=5e-4, d=0.1, seed=11)
    t0 = time.perf_counter()
    O.tg_solve(p, V2, C0, steps)
    dt = time.perf_counter() - t0
    nthr = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    return {"value": g * g * steps / dt, "unit": METRIC, "cores": nthr, "kind": "port",
            "sample": f"oracle TG_solver port, {g}x{g} grid, full {steps} steps (same per-point history length), "
                      f"{dt:.1f} s, OpenMP {nthr} threads"}


# ------------------------------------------------------------------- GB300
def run_gb300(args):
    import torch
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_PROF_HISTORY, FH_PROF_SWEEP, FH_PROF_WEIGHTS, FH_TG_BLOCKED, FH_TG_FP64, \
        Context
    from theses_code_gb300.solvers import TGSolver

    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = local
    torch.cuda.set_device(dev)
    G, S = args.grid, args.solve_steps
    p, V2, C0 = workloads.convection_2d(G, G, alpha=0.7, tau=5e-4, d=0.1, seed=11 + rank)
    ctx = Context(dev)
    mode = FH_TG_BLOCKED if args.mode == "blocked" else FH_TG_FP64
    solver = TGSolver(ctx, p, S, mode)
    V2_d = torch.as_tensor(V2, device=f"cuda:{dev}").contiguous()
    C0_d = torch.as_tensor(C0, device=f"cuda:{dev}").contiguous()
    stream = torch.cuda.ExternalStream(ctx.stream, device=f"cuda:{dev}")
    P = V2.size
    gps = float(G) * G * S  # grid-point-steps per solve

    def solve_device():
        solver.set_state_device(V2_d.data_ptr(), C0_d.data_ptr())
        solver.calc_step(S)

    for _ in range(args.warmup):
        solve_device()
    ctx.sync()

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize(dev)

    clocks = ClockSampler(dev)
    ctx.profile(True)
    launches0 = ctx.launches
    barrier()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        solve_device()
    e1.record(stream)
    e1.synchronize()
    barrier()
    clk = clocks.stop()
    launches = ctx.launches - launches0
    t_ms = e0.elapsed_time(e1)
    hist_ms, hist_n = ctx.profile_read(FH_PROF_HISTORY)
    sweep_ms, _ = ctx.profile_read(FH_PROF_SWEEP)
    w_ms, _ = ctx.profile_read(FH_PROF_WEIGHTS)
    ctx.profile(False)
    t_max = t_ms
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_ms], device=f"cuda:{dev}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_max = float(tt.item())
    value = ws * gps * args.steps / (t_max / 1e3)

    # end to end through the C ABI with pinned host buffers
    V2_h = torch.from_numpy(V2.reshape(-1)).pin_memory()
    C0_h = torch.from_numpy(C0.reshape(-1)).pin_memory()
    out_h = torch.empty(P, dtype=torch.float64).pin_memory()
    L = ctx.L
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        L.fh_tg_set_state_host(solver.h, V2_h.data_ptr(), C0_h.data_ptr())
        L.fh_tg_step(solver.h, S)
        L.fh_tg_get_c_host(solver.h, out_h.data_ptr())
    barrier()
    e2e_s = time.perf_counter() - t0
    if ws > 1:
        import torch.distributed as dist
        tt = torch.tensor([e2e_s], device=f"cuda:{dev}")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        e2e_s = float(tt.item())
    assert np.isfinite(out_h.numpy()).all(), "non-finite result"
    e2e = {"value": ws * gps * args.e2e_steps / e2e_s, "unit": METRIC, "h2d_bytes_per_step": 2 * P * 8,
           "d2h_bytes_per_step": P * 8}

    # roofline of the dominant kernel (history sum): algorithmic bytes = the
    # K history layers read once per step plus the two sums written, over the
    # (G-1)^2 interior points where the sums are needed
    pint = (G - 1) * (G - 1)
    alg_bytes_solve = sum(8.0 * j * pint + 16.0 * pint for j in range(1, S))
    achieved = alg_bytes_solve * args.steps / (hist_ms / 1e3) / 1e9 if hist_ms > 0 else None
    peak, peak_kind = peaks()
    traffic = None
    tp = os.path.join(REPO, "profiles", "hist_sum_traffic.txt")
    if os.path.exists(tp):
        # "ratio <dram bytes / algorithmic bytes>" of the captured launch, scaled to the mean launch
        for line in open(tp):
            if line.startswith("ratio"):
                traffic = float(line.split()[1]) * alg_bytes_solve / (S - 1)
    result = {
        "metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"tg2d_adi_{G}x{G}_{S}steps", "grid": [G, G], "solve_steps": S, "alpha": 0.7,
                   "tau": 5e-4, "d": 0.1, "velocity_modes": 8, "mode": args.mode,
                   "l2": "inputs larger than L2 (history up to %.1f GB per solve)" % (S * P * 8 / 1e9),
                   "parallelism": f"replicas x{ws}"},
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clk,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": "k_hist_sum<2>", "peak_kind": peak_kind,
                     "launches": int(hist_n), "kernel_ms": hist_ms, "sweep_ms": sweep_ms, "weights_ms": w_ms,
                     "note": "achieved = sum of per-launch algorithmic bytes / summed event time of the "
                             "history-sum launches over the timed region; traffic is per mean launch"},
    }
    if rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(args)
    if rank == 0:
        print(json.dumps(result))
    solver.close()
    ctx.close()
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    nthr = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(nthr)
    from oracle import oracle as O  # noqa: F401  (builds/loads the port)
    vals = []
    for _ in range(args.warmup):
        cpu_baseline(args, nthr)
    t0 = time.perf_counter()
    last = None
    for _ in range(args.steps):
        last = cpu_baseline(args, nthr)
        vals.append(last["value"])
    dt = time.perf_counter() - t0
    G = args.cpu_grid
    value = G * G * args.solve_steps * args.steps / dt
    res = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
           "config": {"workload": f"tg2d_adi_{args.grid}x{args.grid}_{args.solve_steps}steps",
                      "sample_grid": [G, G], "solve_steps": args.solve_steps},
           "cpu_baseline": {"value": value, "unit": METRIC, "cores": nthr, "kind": "port",
                            "sample": last["sample"] if last else ""},
           "e2e": {"value": value, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(res))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
