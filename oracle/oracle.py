"""ctypes loader for the CPU oracle (test infrastructure only).

The oracle is the checker for the CUDA library: only tests/, the smoke check
and the CPU-baseline leg of bench.py import this module.  It never backs the
product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libfh_oracle.so")
_lib = None

_dp = C.POINTER(C.c_double)

W_L1, W_PSI = 0, 1
K_CONST, K_EXP = 0, 1


class HParams(C.Structure):
    _fields_ = [("N", C.c_int), ("L", C.c_double), ("tau", C.c_double), ("alpha", C.c_double),
                ("weights", C.c_int), ("beta", C.c_double), ("kmodel", C.c_int),
                ("kc", C.c_double), ("kgam", C.c_double), ("cinv", C.c_double),
                ("gravity", C.c_int), ("al_left", C.c_double), ("bt_left", C.c_double),
                ("u_right", C.c_double), ("gamma", C.c_double), ("pert", C.c_double)]


class TGParams(C.Structure):
    _fields_ = [("sN", C.c_int), ("M", C.c_int), ("tau", C.c_double), ("alpha", C.c_double),
                ("beta", C.c_double), ("sigma", C.c_double), ("d", C.c_double), ("C1", C.c_double),
                ("S", C.c_double), ("dL", C.c_double), ("dLx", C.c_double), ("dt_alg", C.c_int),
                ("dt_eps", C.c_double), ("massN", C.c_int), ("massN_a", C.c_double), ("massN_b", C.c_double),
                ("fixed_d", C.c_int), ("lambda_", C.c_double), ("ka0", C.c_double), ("kk", C.c_double)]


def build() -> str:
    """Compile the oracle restatement (make in oracle/)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = C.CDLL(_LIB_PATH)
        L.fho_psi_int.restype = C.c_double
        L.fho_psi_int.argtypes = [C.c_double] * 6
        L.fho_l1_b.restype = C.c_double
        L.fho_l1_b.argtypes = [C.c_int, C.c_double]
        L.fho_mittag_leffler.restype = C.c_double
        L.fho_mittag_leffler.argtypes = [C.c_double] * 3
        L.fho_ab_int.restype = C.c_double
        L.fho_ab_int.argtypes = [C.c_int, C.c_double, C.c_double]
        L.fho_history_sum_layers.restype = None
        L.fho_history_sum_layers.argtypes = [_dp, C.c_int, C.c_int, C.c_int, _dp, _dp]
        L.fho_thomas.restype = None
        L.fho_thomas.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int,
                                 C.c_double, _dp]
        L.fho_h_solve.restype = C.c_int
        L.fho_h_solve.argtypes = [C.POINTER(HParams), _dp, C.c_int, _dp]
        L.fho_tg_solve.restype = C.c_int
        L.fho_tg_solve.argtypes = [C.POINTER(TGParams), _dp, _dp, C.c_int, _dp]
        L.fho_ab_solve.restype = C.c_int
        L.fho_ab_solve.argtypes = [C.c_int, C.c_int, C.c_double, C.c_double, _dp, _dp, _dp, _dp,
                                   _dp, _dp, _dp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def psi_int(x0, x1, X, tau, alpha, beta) -> float:
    return lib().fho_psi_int(float(x0), float(x1), float(X), float(tau), float(alpha), float(beta))


def l1_b(k: int, alpha: float) -> float:
    return lib().fho_l1_b(int(k), float(alpha))


def mittag_leffler(a, b, z) -> float:
    return lib().fho_mittag_leffler(float(a), float(b), float(z))


def ab_int(lag: int, tau: float, alpha: float) -> float:
    return lib().fho_ab_int(int(lag), float(tau), float(alpha))


def ab_weights(n: int, tau: float, alpha: float) -> np.ndarray:
    """w[lag] for lag = 1..n and w[0] = I(1), the current-step coefficient."""
    w = np.zeros(n + 1)
    for lag in range(1, n + 1):
        w[lag] = ab_int(lag, tau, alpha)
    w[0] = w[1]
    return w


def history_sum_layers(H: np.ndarray, w: np.ndarray) -> np.ndarray:
    """H: (K+1, P) layers, w: (K,) -> S: (P,)."""
    H = np.ascontiguousarray(H, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    K = H.shape[0] - 1
    P = H.shape[1]
    S = np.zeros(P)
    lib().fho_history_sum_layers(_ptr(H), K, P, P, _ptr(w), _ptr(S))
    return S


def thomas(A, R, B, Om, al1, bt1, right_mode, u_right, u) -> np.ndarray:
    N = len(A) - 1
    u = np.ascontiguousarray(u, dtype=np.float64).copy()
    arrs = [np.ascontiguousarray(x, dtype=np.float64) for x in (A, R, B, Om)]
    lib().fho_thomas(N, *[_ptr(x) for x in arrs], float(al1), float(bt1), int(right_mode),
                     float(u_right), _ptr(u))
    return u


def h_solve(params: dict, U0: np.ndarray, steps: int):
    """Returns (U, hist) after `steps` H_solver::calc_step calls."""
    p = HParams(**{"gamma": 1.0, "pert": 0.0, **params})  # gamma = 1: classical second derivative in z
    U = np.ascontiguousarray(U0, dtype=np.float64).copy()
    assert U.shape[0] == p.N + 2
    hist = np.zeros((max(steps, 1), p.N + 2))
    rc = lib().fho_h_solve(C.byref(p), _ptr(U), int(steps), _ptr(hist))
    assert rc == 0
    return U, hist


def tg_solve(params: dict, V2: np.ndarray, C0: np.ndarray, steps: int):
    """params: the TG_solver fields; optional massN (with massN_a, massN_b,
    default 0.1 each as the reference's globals) and fixed_d = 0 (with lambda,
    ka0, kk: D = lambda |v| ka0 / kk per node)."""
    q = dict(params)
    q.setdefault("fixed_d", 1)
    q.setdefault("massN_a", 0.1)
    q.setdefault("massN_b", 0.1)
    if "lambda" in q:
        q["lambda_"] = q.pop("lambda")
    p = TGParams(**q)
    P = (p.sN + 2) * (p.M + 2)
    V2 = np.ascontiguousarray(V2, dtype=np.float64).reshape(-1)
    Cf = np.ascontiguousarray(C0, dtype=np.float64).reshape(-1).copy()
    assert V2.size == P and Cf.size == P
    work = np.zeros((steps + 1) * P)
    rc = lib().fho_tg_solve(C.byref(p), _ptr(V2), _ptr(Cf), int(steps), _ptr(work))
    assert rc == 0
    return Cf, work.reshape(steps + 1, P)


def ab_solve(m, n, tau, alpha, w, src, bl, br, C0, exact=None):
    Cc = np.ascontiguousarray(C0, dtype=np.float64).copy()
    err = C.c_double(0.0)
    w = np.ascontiguousarray(w, dtype=np.float64)
    src = np.ascontiguousarray(src, dtype=np.float64).reshape(-1)
    bl = np.ascontiguousarray(bl, dtype=np.float64)
    br = np.ascontiguousarray(br, dtype=np.float64)
    ex = None if exact is None else np.ascontiguousarray(exact, dtype=np.float64).reshape(-1)
    rc = lib().fho_ab_solve(int(m), int(n), float(tau), float(alpha), _ptr(w), _ptr(src), _ptr(bl),
                            _ptr(br), _ptr(Cc), None if ex is None else _ptr(ex), C.byref(err))
    assert rc == 0
    return Cc, err.value
