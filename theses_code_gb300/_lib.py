"""ctypes binding of libfhist.so (the C ABI declared in include/fhist.h).

Loading fails loudly: there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libfhist.so")

FH_OK, FH_EINVAL, FH_ENOMEM, FH_ECUDA, FH_ENONFINITE, FH_ETIMEOUT, FH_ERANGE, FH_ENOTSUP = range(8)
FH_W_L1, FH_W_PSI = 0, 1
FH_K_CONST, FH_K_EXP = 0, 1
FH_TG_FP64, FH_TG_BLOCKED, FH_TG_DF64 = 0, 1, 2
FH_AB_FP64, FH_AB_BLOCKED = 0, 1
FH_H_FP64, FH_H_DF64, FH_H_BLOCKED = 0, 1, 2
FH_PROF_HISTORY, FH_PROF_SWEEP, FH_PROF_WEIGHTS, FH_PROF_GEMM = 0, 1, 2, 3
FH_NOALLOC_SCRATCH_DOUBLES = 2097152

_vp = C.c_void_p
_dp = C.c_void_p  # device or host double*, passed as raw addresses
_i, _ll, _d = C.c_int, C.c_longlong, C.c_double


class HParams(C.Structure):
    _fields_ = [("N", _i), ("L", _d), ("tau", _d), ("alpha", _d), ("weights", _i), ("beta", _d),
                ("kmodel", _i), ("kc", _d), ("kgam", _d), ("cinv", _d), ("gravity", _i),
                ("al_left", _d), ("bt_left", _d), ("u_right", _d)]


class TGParams(C.Structure):
    _fields_ = [("sN", _i), ("M", _i), ("tau", _d), ("alpha", _d), ("beta", _d), ("sigma", _d),
                ("d", _d), ("C1", _d), ("S", _d), ("dL", _d), ("dLx", _d)]


# name -> (restype, argtypes)
_SIGS = {
    "fh_version": (_i, []),
    "fh_ctx_create": (_i, [_i, C.POINTER(_vp)]),
    "fh_ctx_destroy": (_i, [_vp]),
    "fh_last_error": (C.c_char_p, [_vp]),
    "fh_ctx_sync": (_i, [_vp]),
    "fh_ctx_query": (_i, [_vp]),
    "fh_ctx_set_graphs": (_i, [_vp, _i]),
    "fh_ctx_set_stream": (_i, [_vp, _vp]),
    "fh_ctx_get_stream": (_vp, [_vp]),
    "fh_ctx_launch_count": (_ll, [_vp]),
    "fh_ctx_profile": (_i, [_vp, _i]),
    "fh_ctx_profile_read": (_i, [_vp, _i, C.POINTER(_d), C.POINTER(_ll)]),
    "fh_weights_psi": (_i, [_vp, _i, _d, _d, _d, _d, _d, _d, _d, _dp]),
    "fh_weights_l1": (_i, [_vp, _i, _d, _dp]),
    "fh_weights_ab": (_i, [_vp, _i, _d, _d, _dp]),
    "fh_mittag_leffler": (_i, [_vp, _i, _d, _d, _dp, _dp]),
    "fh_history_sum": (_i, [_vp, _i, _i, _ll, _dp, _i, _dp, _ll, _dp, _ll]),
    "fh_history_sum_layers": (_i, [_vp, _i, _ll, _dp, _dp, _ll, _dp]),
    "fh_series_sum": (_i, [_vp, _i, _ll, _dp, _dp, _d, _dp, _dp, _ll, _dp]),
    "fh_history_sum_noalloc": (_i, [_vp, _i, _i, _ll, _dp, _i, _dp, _ll, _dp, _ll]),
    "fh_history_contract_bf16": (_i, [_vp, _i, _ll, _dp, _i, _dp, _ll, _dp, _ll]),
    "fh_tridiag_batched": (_i, [_vp, _i, _i, _dp, _dp, _dp, _dp, _ll, _dp, _dp, _i, _dp, _dp, _ll]),
    "fh_pcr_solver": (_i, [_vp, _dp, _dp, _dp, _dp, _dp, _i, _i]),
    "fh_h_batch_create": (_i, [_vp, _i, C.POINTER(HParams), _i, C.POINTER(_vp)]),
    "fh_h_batch_destroy": (_i, [_vp]),
    "fh_h_batch_state_size": (_ll, [_vp]),
    "fh_h_batch_device_bytes": (_ll, [_vp]),
    "fh_tg_device_bytes": (_ll, [_vp]),
    "fh_h_batch_set_u_host": (_i, [_vp, _dp]),
    "fh_h_batch_get_u_host": (_i, [_vp, _dp]),
    "fh_h_batch_set_u": (_i, [_vp, _dp]),
    "fh_h_batch_restart": (_i, [_vp, _i, C.POINTER(HParams), _dp]),
    "fh_h_batch_set_persistent": (_i, [_vp, _i]),
    "fh_h_batch_get_u_range_host": (_i, [_vp, _i, _i, _dp]),
    "fh_h_batch_step": (_i, [_vp, _i]),
    "fh_h_batch_tstep": (_i, [_vp]),
    "fh_tg_create": (_i, [_vp, C.POINTER(TGParams), _i, _i, C.POINTER(_vp)]),
    "fh_tg_destroy": (_i, [_vp]),
    "fh_tg_set_state_host": (_i, [_vp, _dp, _dp]),
    "fh_tg_set_state": (_i, [_vp, _dp, _dp]),
    "fh_tg_step": (_i, [_vp, _i]),
    "fh_tg_set_restricted": (_i, [_vp, C.c_double]),
    "fh_h_batch_set_space_order": (_i, [_vp, _dp]),
    "fh_tg_set_series": (_i, [_vp, _i]),
    "fh_tg_set_two_series": (_i, [_vp, _i]),
    "fh_tg_set_mass_exchange": (_i, [_vp, _i, _d, _d]),
    "fh_tg_get_n_host": (_i, [_vp, _dp]),
    "fh_tg_set_diffusion": (_i, [_vp, _i, _d, _d, _d]),
    "fh_tg_two_series_plan": (_i, [_d, _i, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "fh_tg_get_c_host": (_i, [_vp, _dp]),
    "fh_tg_field": (_vp, [_vp]),
    "fh_tg_tstep": (_i, [_vp]),
    "fh_ab_create": (_i, [_vp, _i, _i, _d, _d, C.POINTER(_vp)]),
    "fh_ab_destroy": (_i, [_vp]),
    "fh_ab_set_source_host": (_i, [_vp, _i, _dp, _dp, _dp]),
    "fh_ab_set_c_host": (_i, [_vp, _dp]),
    "fh_ab_set_c": (_i, [_vp, _dp]),
    "fh_ab_set_current_coef": (_i, [_vp, _d]),
    "fh_ab_set_lag_weights_host": (_i, [_vp, _i, _dp]),
    "fh_ab_step": (_i, [_vp, _i]),
    "fh_ab_set_mode": (_i, [_vp, _i]),
    "fh_h_batch_set_mode": (_i, [_vp, _i]),
    "fh_h_batch_autotune": (_i, [_vp, C.POINTER(C.c_float)]),
    "fh_h_batch_launch_shape": (_i, [_vp, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "fh_ab_get_c_host": (_i, [_vp, _dp]),
}

_lib = None


def load(path: str | None = None):
    """Load libfhist.so; raises if it is missing (build it first)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"libfhist.so not built ({path}); run __graft_entry__.build()")
    L = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def declared_symbols() -> list[str]:
    return list(_SIGS)


class FhError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"libfhist error {code}: {msg}")
        self.code = code


def check(rc: int, ctx=None):
    if rc != FH_OK:
        L = load()
        msg = L.fh_last_error(ctx)
        raise FhError(rc, msg.decode() if msg else "")


class Context:
    """Owns an fh_ctx (one CUDA stream)."""

    def __init__(self, device: int = 0):
        L = load()
        h = _vp()
        check(L.fh_ctx_create(device, C.byref(h)))
        self.h = h
        self.L = L
        self._children = weakref.WeakSet()

    def adopt(self, obj):
        """Solver objects register here so that close() destroys them first."""
        self._children.add(obj)

    def close(self):
        if self.h:
            for ch in list(self._children):
                ch.close()
            self.L.fh_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(self.L.fh_ctx_sync(self.h), self.h)

    def set_graphs(self, enable: bool):
        check(self.L.fh_ctx_set_graphs(self.h, int(bool(enable))), self.h)

    def idle(self) -> bool:
        r = self.L.fh_ctx_query(self.h)
        if r < 0:
            check(-r, self.h)
        return r == 1

    @property
    def stream(self) -> int:
        return self.L.fh_ctx_get_stream(self.h) or 0

    def set_stream(self, stream_handle: int):
        check(self.L.fh_ctx_set_stream(self.h, _vp(stream_handle)), self.h)

    @property
    def launches(self) -> int:
        return self.L.fh_ctx_launch_count(self.h)

    def profile(self, enable: bool):
        check(self.L.fh_ctx_profile(self.h, int(bool(enable))), self.h)

    def profile_read(self, kind: int):
        ms, n = _d(0.0), _ll(0)
        check(self.L.fh_ctx_profile_read(self.h, int(kind), C.byref(ms), C.byref(n)), self.h)
        return ms.value, n.value

    def call(self, name, *args):
        rc = getattr(self.L, name)(self.h, *args)
        check(rc, self.h)
        return rc
