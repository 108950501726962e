"""Host-side mirror of the reference solver classes over the libfhist C ABI.

Names follow the reference:
  HSolverBatch  -- H_solver (mt_minimal.cpp / mt_psi_caputo.cpp), many instances
  TGSolver      -- TG_solver_<func,1,kform> 2D ADI (fr_d_t_g_2d.cpp)
  ABSolver      -- solve_and_check Atangana-Baleanu solve (MF_int_series.cpp)
Every compute call goes to the CUDA library; there is no CPU path.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import Context, HParams, TGParams, check


def _hptr(a: np.ndarray) -> int:
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


class HSolverBatch:
    """A batch of H_solver instances advanced in lock step (calc_step)."""

    def __init__(self, ctx: Context, params: list[dict], max_steps: int, mode: int = _lib.FH_H_FP64):
        self.ctx = ctx
        self.params = [HParams(**p) for p in params]
        arr = (HParams * len(params))(*self.params)
        h = C.c_void_p()
        check(ctx.L.fh_h_batch_create(ctx.h, len(params), arr, int(max_steps), C.byref(h)), ctx.h)
        self.h = h
        ctx.adopt(self)
        if mode != _lib.FH_H_FP64:
            check(ctx.L.fh_h_batch_set_mode(h, int(mode)), ctx.h)
        self.sizes = [p.N + 2 for p in self.params]
        self.total = int(ctx.L.fh_h_batch_state_size(h))

    def close(self):
        if self.h and self.ctx.h:
            self.ctx.L.fh_h_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def autotune(self) -> dict:
        """Picks the history-sum launch shape by timing the candidates
        (fh_h_batch_autotune); returns the chosen shape and its time."""
        ms = C.c_float(0.0)
        check(self.ctx.L.fh_h_batch_autotune(self.h, C.byref(ms)), self.ctx.h)
        t, c = C.c_int(0), C.c_int(0)
        check(self.ctx.L.fh_h_batch_launch_shape(self.h, C.byref(t), C.byref(c)), self.ctx.h)
        return {"tile_threads": t.value, "split_cap": c.value, "ms_per_launch": ms.value}

    def set_space_order(self, gamma):
        """Space-derivative order per instance (the reference's gamma; < 1 adds the
        space-fractional Caputo term in z), before the first step."""
        g = np.ascontiguousarray(np.asarray(gamma, dtype=np.float64).reshape(-1))
        assert g.size == len(self.params)
        check(self.ctx.L.fh_h_batch_set_space_order(self.h, _hptr(g)), self.ctx.h)

    def set_u(self, U: np.ndarray | list):
        flat = np.ascontiguousarray(np.concatenate([np.asarray(u, dtype=np.float64) for u in U])
                                    if isinstance(U, list) else U, dtype=np.float64)
        assert flat.size == self.total
        check(self.ctx.L.fh_h_batch_set_u_host(self.h, _hptr(flat)), self.ctx.h)

    def set_u_device(self, ptr: int):
        check(self.ctx.L.fh_h_batch_set_u(self.h, C.c_void_p(ptr)), self.ctx.h)

    def restart(self, i: int, params: dict, U0: np.ndarray):
        """Instance i starts a new solve (continuous batching): its own steps
        count from 1 and its history starts empty while the others go on;
        params["N"] may not exceed the instance's node count at creation."""
        hp = HParams(**params)
        u = np.ascontiguousarray(U0, dtype=np.float64)
        assert u.size == hp.N + 2
        check(self.ctx.L.fh_h_batch_restart(self.h, int(i), C.byref(hp), _hptr(u)), self.ctx.h)
        self.params[i] = hp
        self.sizes[i] = hp.N + 2
        self.total = int(self.ctx.L.fh_h_batch_state_size(self.h))

    def get_u(self) -> list[np.ndarray]:
        out = np.empty(self.total)
        check(self.ctx.L.fh_h_batch_get_u_host(self.h, _hptr(out)), self.ctx.h)
        res, o = [], 0
        for s in self.sizes:
            res.append(out[o:o + s].copy())
            o += s
        return res

    def get_u_range(self, first: int, count: int) -> list[np.ndarray]:
        sizes = self.sizes[first:first + count]
        out = np.empty(sum(sizes))
        check(self.ctx.L.fh_h_batch_get_u_range_host(self.h, int(first), int(count), _hptr(out)), self.ctx.h)
        res, o = [], 0
        for s in sizes:
            res.append(out[o:o + s].copy())
            o += s
        return res

    def calc_step(self, n: int = 1):
        check(self.ctx.L.fh_h_batch_step(self.h, int(n)), self.ctx.h)

    def set_persistent(self, enable: bool):
        """Small FP64 batches: all steps of a call in one launch (default on)."""
        check(self.ctx.L.fh_h_batch_set_persistent(self.h, int(bool(enable))), self.ctx.h)

    def device_bytes(self) -> int:
        """Device memory the batch holds."""
        return int(self.ctx.L.fh_h_batch_device_bytes(self.h))

    @property
    def tstep(self) -> int:
        return self.ctx.L.fh_h_batch_tstep(self.h)


class TGSolver:
    """TG_solver_ 2D ADI with full fractional history."""

    def __init__(self, ctx: Context, params: dict, max_steps: int, mode: int = _lib.FH_TG_FP64):
        self.ctx = ctx
        self.p = TGParams(**params)
        h = C.c_void_p()
        check(ctx.L.fh_tg_create(ctx.h, C.byref(self.p), int(max_steps), int(mode), C.byref(h)), ctx.h)
        self.h = h
        ctx.adopt(self)
        self.shape = (self.p.M + 2, self.p.sN + 2)  # [j][i], idx = i + j*(sN+2)

    def close(self):
        if self.h and self.ctx.h:
            self.ctx.L.fh_tg_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_state(self, V2: np.ndarray, C0: np.ndarray):
        V2 = np.ascontiguousarray(V2, dtype=np.float64).reshape(-1)
        C0 = np.ascontiguousarray(C0, dtype=np.float64).reshape(-1)
        check(self.ctx.L.fh_tg_set_state_host(self.h, _hptr(V2), _hptr(C0)), self.ctx.h)

    def set_state_device(self, V2_ptr: int, C_ptr: int):
        check(self.ctx.L.fh_tg_set_state(self.h, C.c_void_p(V2_ptr), C.c_void_p(C_ptr)), self.ctx.h)

    def set_restricted(self, dt_eps: float):
        """Restricted summing (the reference's dt_alg 2): each history sum stops
        at the first weight below dt_eps, newest layer first; 0 = full history."""
        check(self.ctx.L.fh_tg_set_restricted(self.h, float(dt_eps)), self.ctx.h)

    def set_series(self, nterms: int):
        """Series expansion of the history sums (the reference's dt_alg 3 with
        dt_eps = nterms, psi = t): nterms accumulators per node replace the
        stored layers; 0 = full history."""
        check(self.ctx.L.fh_tg_set_series(self.h, int(nterms)), self.ctx.h)

    def set_mass_exchange(self, enable: bool = True, massN_a: float = 0.1, massN_b: float = 0.1):
        """Mass exchange with a non-soluble phase (the reference's massN, with
        its globals massN_a, massN_b)."""
        check(self.ctx.L.fh_tg_set_mass_exchange(self.h, int(bool(enable)), float(massN_a), float(massN_b)),
              self.ctx.h)

    def set_diffusion(self, fixed_d: bool, lam: float = 0.0, ka0: float = 0.0, k: float = 1.0):
        """fixed_d False: D = lam |v| (ka0 / k) per node (TG_solver_<func,0,0>)."""
        check(self.ctx.L.fh_tg_set_diffusion(self.h, int(bool(fixed_d)), float(lam), float(ka0), float(k)),
              self.ctx.h)

    def set_two_series(self, enable: bool = True):
        """Two-series approximation of the history sums (the reference's
        dt_alg 4, psi = t): per node long and short series absorb each new
        layer difference; only the newest layer is stored."""
        check(self.ctx.L.fh_tg_set_two_series(self.h, int(bool(enable))), self.ctx.h)

    def calc_step(self, n: int = 1):
        check(self.ctx.L.fh_tg_step(self.h, int(n)), self.ctx.h)

    def device_bytes(self) -> int:
        """Device memory the solver holds."""
        return int(self.ctx.L.fh_tg_device_bytes(self.h))

    def get_n(self) -> np.ndarray:
        """The non-soluble phase N (mass exchange on)."""
        out = np.empty(self.shape[0] * self.shape[1])
        check(self.ctx.L.fh_tg_get_n_host(self.h, _hptr(out)), self.ctx.h)
        return out

    def get_c(self) -> np.ndarray:
        out = np.empty(self.shape[0] * self.shape[1])
        check(self.ctx.L.fh_tg_get_c_host(self.h, _hptr(out)), self.ctx.h)
        return out

    @property
    def field_ptr(self) -> int:
        return self.ctx.L.fh_tg_field(self.h)

    @property
    def tstep(self) -> int:
        return self.ctx.L.fh_tg_tstep(self.h)


class ABSolver:
    """solve_and_check-style Atangana-Baleanu convection-diffusion solve."""

    def __init__(self, ctx: Context, m: int, max_steps: int, tau: float, alpha: float, mode: int = _lib.FH_AB_FP64):
        self.ctx = ctx
        self.m = m
        h = C.c_void_p()
        check(ctx.L.fh_ab_create(ctx.h, int(m), int(max_steps), float(tau), float(alpha), C.byref(h)), ctx.h)
        self.h = h
        ctx.adopt(self)
        if mode != _lib.FH_AB_FP64:
            check(ctx.L.fh_ab_set_mode(h, int(mode)), ctx.h)

    def close(self):
        if self.h and self.ctx.h:
            self.ctx.L.fh_ab_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_source(self, src: np.ndarray, bl: np.ndarray, br: np.ndarray):
        src = np.ascontiguousarray(src, dtype=np.float64).reshape(-1, self.m + 1)
        bl = np.ascontiguousarray(bl, dtype=np.float64)
        br = np.ascontiguousarray(br, dtype=np.float64)
        check(self.ctx.L.fh_ab_set_source_host(self.h, src.shape[0], _hptr(src), _hptr(bl), _hptr(br)),
              self.ctx.h)

    def set_c(self, C0: np.ndarray):
        C0 = np.ascontiguousarray(C0, dtype=np.float64)
        check(self.ctx.L.fh_ab_set_c_host(self.h, _hptr(C0)), self.ctx.h)

    def set_c_device(self, ptr: int):
        check(self.ctx.L.fh_ab_set_c(self.h, C.c_void_p(ptr)), self.ctx.h)

    def set_current_coef(self, Ii: float):
        check(self.ctx.L.fh_ab_set_current_coef(self.h, float(Ii)), self.ctx.h)

    def set_lag_weights(self, w):
        """History weights of lags 1..len(w) (the reference's I_cache), before the first step."""
        w = np.ascontiguousarray(np.asarray(w, dtype=np.float64).reshape(-1))
        check(self.ctx.L.fh_ab_set_lag_weights_host(self.h, int(w.size), _hptr(w)), self.ctx.h)

    def calc_step(self, n: int = 1):
        check(self.ctx.L.fh_ab_step(self.h, int(n)), self.ctx.h)

    def get_c(self) -> np.ndarray:
        out = np.empty(self.m + 1)
        check(self.ctx.L.fh_ab_get_c_host(self.h, _hptr(out)), self.ctx.h)
        return out
