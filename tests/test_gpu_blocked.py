"""Tensor-core blocked contraction (tcgen05, exact bf16 slices) against FP64.

The slices are exact integers relative to per-chunk power-of-two scales, so the
tensor-core sums are exact; what remains is the slicing into four 8-bit slices,
~2^-32 of the chunk MAXIMA (max_k |W| and max_k |D| over each 64-layer chunk)
per term, which for zero-mean random data is up to ~10x the per-term magnitude.
Bound used: 2e-8 * sum_k |W[m,k]| |D[k,p]| elementwise (measured max 1.3e-9)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from conftest import torch_ordered_context
    c = torch_ordered_context(0)
    yield c
    c.close()


@pytest.mark.parametrize("K,P", [(64, 128), (128, 100), (192, 1000), (640, 5000), (1984, 2222)])
def test_contract_bf16_matches_fp64(ctx, K, P):
    import torch
    rng = np.random.default_rng(K + P)
    W = rng.uniform(0.0, 1.0, size=(128, K)) * np.exp(-np.arange(K) / 300.0)[None, :]
    D = rng.normal(size=(K, P)) * 1e-3
    Wd = torch.as_tensor(W, device="cuda")
    Dd = torch.as_tensor(D, device="cuda")
    S = torch.full((128, P), np.nan, dtype=torch.float64, device="cuda")
    ctx.call("fh_history_contract_bf16", K, P, Wd.data_ptr(), K, Dd.data_ptr(), P, S.data_ptr(), P)
    ctx.sync()
    got = S.cpu().numpy()
    ref = W @ D
    scale = np.abs(W) @ np.abs(D)
    assert np.isfinite(got).all()
    err = np.abs(got - ref) / scale
    print(f"K={K} P={P} max rel err {err.max():.3e}")
    assert err.max() <= 2e-8, err.max()


def test_contract_rejects_bad_k(ctx):
    import torch
    from theses_code_gb300._lib import FhError
    W = torch.zeros((128, 100), dtype=torch.float64, device="cuda")
    D = torch.zeros((100, 10), dtype=torch.float64, device="cuda")
    S = torch.zeros((128, 10), dtype=torch.float64, device="cuda")
    with pytest.raises(FhError):
        ctx.call("fh_history_contract_bf16", 100, 10, W.data_ptr(), 100, D.data_ptr(), 10, S.data_ptr(), 10)


@pytest.mark.parametrize("sN,M,steps", [(64, 48, 200), (96, 80, 330)])
def test_tg_blocked_mode_vs_fp64_oracle(ctx, sN, M, steps):
    """Blocked 2D ADI (far history on the tensor cores, the layers of the current
    64-step block in double-float) against the FP64 oracle: relative max-norm
    <= 1e-9 (the mixed-precision bound)."""
    from oracle import oracle as O
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(sN, M, alpha=0.7, tau=5e-4, d=0.1, seed=sN + 1, C1=0.2)
    s = TGSolver(ctx, p, steps, FH_TG_BLOCKED)
    s.set_state(V2, C0)
    s.calc_step(steps)
    got = s.get_c()
    ref, _ = O.tg_solve(p, V2, C0, steps)
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"blocked {sN}x{M} {steps} steps: rel max-norm err {err:.3e}")
    assert err <= 1e-9, err


@pytest.mark.parametrize("n", [100, 300, 520])
def test_ab_blocked_mode_vs_oracle(ctx, n):
    """Atangana-Baleanu solve with the entries older than the current 128-step
    block contracted on the tensor cores: relative max-norm <= 1e-9 vs the
    FP64 oracle."""
    from oracle import oracle as O
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_AB_BLOCKED
    from theses_code_gb300.solvers import ABSolver
    cfg, src, bl, br, C0 = workloads.ab_1d(m=256, alpha=0.6, tau=1e-3, seed=2)
    s = ABSolver(ctx, cfg["m"], n, cfg["tau"], cfg["alpha"], FH_AB_BLOCKED)
    s.set_source(src, bl, br)
    s.set_c(C0)
    s.calc_step(n)
    w = O.ab_weights(n, cfg["tau"], cfg["alpha"])
    srcs = np.repeat(src, n, axis=0)
    ref, _ = O.ab_solve(cfg["m"], n, cfg["tau"], cfg["alpha"], w, srcs, np.zeros(n), np.zeros(n), C0)
    got = s.get_c()
    err = np.max(np.abs(got - ref)) / np.max(np.abs(ref))
    print(f"AB blocked {n} steps: rel max-norm err {err:.3e}")
    assert err <= 1e-9, err


def test_full_size_modes_agree(ctx):
    """The benchmark workload (512 x 512, 2000 steps) at full size: the blocked
    and double-float modes against the plain FP64 path, which the oracle pins
    at 1e-12 on the smaller parity cases (a size-independent cross-check)."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED, FH_TG_DF64, FH_TG_FP64
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(512, 512, alpha=0.7, tau=5e-4, d=0.1, seed=11)
    out = {}
    for mode in (FH_TG_FP64, FH_TG_DF64, FH_TG_BLOCKED):
        s = TGSolver(ctx, p, 2000, mode)
        s.set_state(V2, C0)
        s.calc_step(2000)
        out[mode] = s.get_c()
        s.close()
    ref = out[FH_TG_FP64]
    den = np.max(np.abs(ref))
    e_df = np.max(np.abs(out[FH_TG_DF64] - ref)) / den
    e_blk = np.max(np.abs(out[FH_TG_BLOCKED] - ref)) / den
    print(f"512^2 x 2000: df64 {e_df:.3e}, blocked {e_blk:.3e}")
    assert np.isfinite(out[FH_TG_BLOCKED]).all()
    assert e_df <= 1e-12 and e_blk <= 1e-9, (e_df, e_blk)


def test_contract_large_vs_torch_fp64(ctx):
    """Exact-slice contraction at a size beyond the CPU oracle's reach, against
    torch's FP64 matmul on the GPU (2e-8 of sum |W||D|)."""
    import torch
    K, P = 1024, 300000
    g = torch.Generator(device="cuda").manual_seed(5)
    W = torch.rand((128, K), dtype=torch.float64, device="cuda", generator=g) * torch.exp(
        -torch.arange(K, device="cuda", dtype=torch.float64) / 300.0)
    D = torch.randn((K, P), dtype=torch.float64, device="cuda", generator=g) * 1e-3
    S = torch.empty((128, P), dtype=torch.float64, device="cuda")
    ctx.call("fh_history_contract_bf16", K, P, W.data_ptr(), K, D.data_ptr(), P, S.data_ptr(), P)
    ctx.sync()
    ref = W @ D
    scale = W.abs() @ D.abs()
    err = float(((S - ref).abs() / scale).max())
    print(f"K={K} P={P} max rel err {err:.3e}")
    assert err <= 2e-8, err


def _blocked_vs_fp64(ctx, p, V2, C0, calls):
    from theses_code_gb300._lib import FH_TG_BLOCKED, FH_TG_FP64
    from theses_code_gb300.solvers import TGSolver
    steps = sum(calls)
    out = {}
    for mode in (FH_TG_FP64, FH_TG_BLOCKED):
        s = TGSolver(ctx, p, steps, mode)
        s.set_state(V2, C0)
        for n in (calls if mode == FH_TG_BLOCKED else [steps]):
            s.calc_step(n)
        out[mode] = s.get_c()
        s.close()
    ref = out[FH_TG_FP64]
    return np.max(np.abs(out[FH_TG_BLOCKED] - ref)) / np.max(np.abs(ref)), out[FH_TG_BLOCKED]


def test_tg_blocked_uneven_step_calls(ctx):
    """Steps advanced in calls that start and end inside 8-step sub-blocks and
    64-step blocks give the same field as one call over all steps."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_TG_BLOCKED
    from theses_code_gb300.solvers import TGSolver
    p, V2, C0 = workloads.convection_2d(64, 48, alpha=0.7, tau=5e-4, d=0.1, seed=7, C1=0.2)
    err, got = _blocked_vs_fp64(ctx, p, V2, C0, [1, 3, 7, 13, 50, 1, 62, 63])
    one = TGSolver(ctx, p, 200, FH_TG_BLOCKED)
    one.set_state(V2, C0)
    one.calc_step(200)
    whole = one.get_c()
    diff = np.max(np.abs(got - whole)) / np.max(np.abs(whole))
    print(f"uneven calls: vs one call {diff:.3e}, vs FP64 {err:.3e}")
    assert diff <= 1e-13, diff
    assert err <= 1e-9, err


def test_tg_blocked_psi_beta(ctx):
    """psi(t) = t^1.3 in blocked mode: the factorization changes every step, so
    the per-step double-float sweeps run (with the sub-block history rows)."""
    from theses_code_gb300 import workloads
    p, V2, C0 = workloads.convection_2d(64, 48, alpha=0.6, tau=1e-3, d=0.1, seed=5, C1=0.1)
    p["beta"] = 1.3
    err, _ = _blocked_vs_fp64(ctx, p, V2, C0, [150])
    print(f"blocked psi beta 1.3: {err:.3e}")
    assert err <= 1e-9, err


def test_tg_blocked_wide_grid(ctx):
    """Lines longer than 513 nodes: the per-step double-float sweeps (the fused
    sub-block kernel holds at most 513-node lines in shared memory)."""
    from theses_code_gb300 import workloads
    p, V2, C0 = workloads.convection_2d(600, 40, alpha=0.7, tau=5e-4, d=0.1, seed=9, C1=0.2)
    err, _ = _blocked_vs_fp64(ctx, p, V2, C0, [130])
    print(f"blocked 600x40: {err:.3e}")
    assert err <= 1e-9, err


def test_ab_blocked_uneven_step_calls(ctx):
    """AB blocked mode advanced in calls that start and end inside 8-step
    sub-blocks and 128-step blocks: the same field as one call over all steps."""
    from theses_code_gb300 import workloads
    from theses_code_gb300._lib import FH_AB_BLOCKED
    from theses_code_gb300.solvers import ABSolver
    cfg, src, bl, br, C0 = workloads.ab_1d(m=256, alpha=0.6, tau=1e-3, seed=3)
    out = []
    for calls in ([1, 7, 13, 50, 100, 129], [300]):
        s = ABSolver(ctx, cfg["m"], 300, cfg["tau"], cfg["alpha"], FH_AB_BLOCKED)
        s.set_source(src, bl, br)
        s.set_c(C0)
        for n in calls:
            s.calc_step(n)
        out.append(s.get_c())
        s.close()
    diff = np.max(np.abs(out[0] - out[1])) / np.max(np.abs(out[1]))
    print(f"AB uneven calls vs one call: {diff:.3e}")
    assert diff <= 1e-13, diff
