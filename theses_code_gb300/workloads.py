"""Seeded synthetic inputs for the benchmark configurations of the history path.

Each builder returns plain numpy inputs plus parameter dicts for the solvers in
theses_code_gb300.solvers (and for the CPU oracle, which takes the same keys).
The geometry of the 2D case follows the TG_solver constructor
(fr_d_t_g_2d.cpp:2299-2418): Lx = 5, dL = 2 Lx/(2 sN + 1), dLx = Q/M with
Q = k (L/2 - H), k = 2 sqrt(5)/(2.5 pi), L = 22, H = 1/sqrt(5), sigma = 0.2.
"""
from __future__ import annotations

import math

import numpy as np

from ._lib import FH_K_CONST, FH_K_EXP, FH_W_L1, FH_W_PSI


# --------------------------------------------------------------------- 1D L1
def caputo_1d(N_interior: int = 200, alpha: float = 0.8, D: float = 1.0, tau: float = 1e-3):
    """u_t^alpha = D u_xx on [0,1], u0 = sin(pi x), zero Dirichlet ends, L1 weights
    (H_solver of mt_minimal.cpp with gamma = 1, constant K = D, 1/(dw/dh) = 1)."""
    N = N_interior + 1
    p = dict(N=N, L=1.0, tau=tau, alpha=alpha, weights=FH_W_L1, beta=1.0, kmodel=FH_K_CONST, kc=D,
             kgam=0.0, cinv=1.0, gravity=0, al_left=0.0, bt_left=0.0, u_right=0.0)
    x = np.arange(N + 2) / N
    U0 = np.sin(math.pi * x)
    U0[0] = 0.0
    U0[N] = 0.0
    U0[N + 1] = 0.0
    return p, U0


# ------------------------------------------------------------ 1D psi batch
def psi_batch(n: int = 4096, seed: int = 7, Nmin: int = 64, Nmax: int = 1024, tau: float = 1e-3):
    """Batched psi-Caputo moisture transport: psi(t) = t^beta, D(u) = D0 exp(gamma u),
    gravity term on, no-flux top, Dirichlet 0 bottom.  One seeded draw per instance."""
    rng = np.random.default_rng(seed)
    params, U0s = [], []
    for _ in range(n):
        N = int(rng.integers(Nmin, Nmax + 1))
        alpha = float(rng.uniform(0.5, 0.95))
        beta = float(rng.uniform(0.5, 2.0))
        D0 = float(rng.uniform(0.01, 1.0))
        gam = float(rng.uniform(0.0, 3.0))
        params.append(dict(N=N, L=1.0, tau=tau, alpha=alpha, weights=FH_W_PSI, beta=beta, kmodel=FH_K_EXP,
                           kc=D0, kgam=gam, cinv=1.0, gravity=1, al_left=1.0, bt_left=0.0, u_right=0.0))
        x = np.arange(N + 2) / N
        u = 0.25 * (1.0 + np.cos(math.pi * x))
        u[N] = 0.0
        u[N + 1] = 0.0
        U0s.append(u)
    return params, U0s


# ----------------------------------------------------------------- 2D ADI
def tg_geometry(sN: int, M: int):
    k = 2.0 * math.sqrt(5.0) / (math.pi * 2.5)
    L, H, Lx = 22.0, 1.0 / math.sqrt(5.0), 5.0
    Q = k * (0.5 * L - H)
    return 2 * Lx / (2.0 * sN + 1.0), Q / M


def convection_2d(sN: int = 512, M: int = 512, alpha: float = 0.7, tau: float = 5e-4, d: float = 0.1,
                  seed: int = 11, modes: int = 8, C1: float = 0.0, S: float = 0.0):
    """2D Caputo-Gerasimov convection-diffusion: V2 = |v|^2 of a seeded sum of
    `modes` Fourier modes normalised to max |v| = 1, Gaussian plume with a seeded
    centre.  Arrays are (M+2, sN+2) so that flat index = i + j*(sN+2)."""
    rng = np.random.default_rng(seed)
    dL, dLx = tg_geometry(sN, M)
    i = np.arange(sN + 2)
    j = np.arange(M + 2)
    X = (i * dL)[None, :]
    Y = ((j - 0.5) * dLx)[:, None]
    Lx_ext, Ly_ext = (sN + 1) * dL, (M + 1) * dLx
    vx = np.zeros((M + 2, sN + 2))
    vy = np.zeros((M + 2, sN + 2))
    for _ in range(modes):
        kx = 2 * math.pi * rng.integers(1, 5) / Lx_ext
        ky = 2 * math.pi * rng.integers(1, 5) / Ly_ext
        a, b = rng.normal(size=2)
        ph1, ph2 = rng.uniform(0, 2 * math.pi, size=2)
        vx += a * np.cos(kx * X + ky * Y + ph1)
        vy += b * np.sin(kx * X - ky * Y + ph2)
    mag2 = vx ** 2 + vy ** 2
    V2 = mag2 / mag2.max()
    cx = rng.uniform(0.3, 0.7) * Lx_ext
    cy = rng.uniform(0.3, 0.7) * Ly_ext
    sig = 0.08 * min(Lx_ext, Ly_ext)
    C0 = np.exp(-((X - cx) ** 2 + (Y - cy) ** 2) / (2 * sig * sig))
    params = dict(sN=sN, M=M, tau=tau, alpha=alpha, beta=1.0, sigma=0.2, d=d, C1=C1, S=S, dL=dL, dLx=dLx)
    return params, np.ascontiguousarray(V2), np.ascontiguousarray(C0)


# -------------------------------------------------------- 1D Atangana-Baleanu
def ab_1d(m: int = 2048, alpha: float = 0.6, tau: float = 1e-4, seed: int = 5, modes: int = 16):
    """AB diffusion on [0,1] with a seeded smooth source of `modes` sine modes,
    zero Dirichlet ends, C0 = 0 (solve_and_check structure, MF_int_series.cpp)."""
    rng = np.random.default_rng(seed)
    x = np.arange(m + 1) / m
    src = np.zeros(m + 1)
    for q in range(1, modes + 1):
        src += rng.normal() / q * np.sin(q * math.pi * x + rng.uniform(0, 0.5))
    src[0] = src[-1] = 0.0
    return dict(m=m, alpha=alpha, tau=tau), src[None, :].copy(), np.zeros(1), np.zeros(1), np.zeros(m + 1)
