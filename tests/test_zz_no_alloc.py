"""fh_history_sum_noalloc: the history sum for callers that cannot allocate
device memory when they call it (memory held by their own pool or budget, or
loops where cudaMalloc/cudaFree would synchronise the device).  Its partial sums
live in a fixed device array inside the library, so its result must equal the
allocating fh_history_sum, call after call.  This file is collected last."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(ctx, torch, name, M, K, P, W, D):
    Wd = torch.as_tensor(W, device="cuda")
    Dd = torch.as_tensor(D, device="cuda")
    S = torch.full((M, P), -1.0, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()  # the library's stream is not torch's: inputs complete first
    ctx.call(name, M, K, P, Wd.data_ptr(), W.shape[1], Dd.data_ptr(), P, S.data_ptr(), P)
    ctx.sync()
    return S.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice_in_a_row():
    import torch
    from theses_code_gb300._lib import Context
    ctx = Context(0)
    rng = np.random.default_rng(2024)
    # the second call reuses the array the first one left behind
    for M, K, P in [(2, 700, 50000), (1, 333, 120002)]:
        D = rng.normal(size=(K, P))
        W = rng.uniform(0.1, 1.0, size=(M, K))
        ref = _run(ctx, torch, "fh_history_sum", M, K, P, W, D)
        got = _run(ctx, torch, "fh_history_sum_noalloc", M, K, P, W, D)
        scale = np.abs(W) @ np.abs(D)
        # same tolerance as the history-sum parity test
        assert np.all(np.abs(got - ref) <= 1e-14 * scale * K ** 0.5)
        assert np.all(np.abs(got - W @ D) <= 1e-14 * scale * K ** 0.5)
    ctx.close()


@pytest.mark.parametrize("M,K,P", [(2, 3000, 500000), (2, 2100, 1 << 20)])
def test_noalloc_with_the_array_limiting_the_splits(M, K, P):
    """Sizes where the fixed array holds fewer split partials than
    fh_history_sum plans: (2, 3000, 500000) gets 2 splits of 1500 layers
    (fh_history_sum: 4), (2, 2100, 2^20) one split of 2100 layers, walked in
    two weight stages.  The partials are added in another order, so the two
    entry points agree within FP64 rounding; both calls in a row are checked
    against W @ D in FP64 (inputs generated on the device: 12-18 GB)."""
    import torch
    from theses_code_gb300._lib import Context
    ctx = Context(0)
    g = torch.Generator(device="cuda").manual_seed(7)
    D = torch.randn((K, P), dtype=torch.float64, device="cuda", generator=g)
    W = torch.rand((M, K), dtype=torch.float64, device="cuda", generator=g) * 0.9 + 0.1
    ref = W @ D
    scale = (W.abs() @ D.abs()).mul_(1e-14 * K ** 0.5)
    for name in ("fh_history_sum", "fh_history_sum_noalloc", "fh_history_sum_noalloc"):
        S = torch.full((M, P), -1.0, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()  # the library's stream is not torch's: inputs complete first
        ctx.call(name, M, K, P, W.data_ptr(), K, D.data_ptr(), P, S.data_ptr(), P)
        ctx.sync()
        assert bool(((S - ref).abs() <= scale).all()), name
        del S
    del D, W, ref, scale
    torch.cuda.empty_cache()
    ctx.close()


def test_noalloc_rejects_sizes_beyond_the_scratch():
    import torch
    from theses_code_gb300._lib import FH_ERANGE, FH_NOALLOC_SCRATCH_DOUBLES, Context, FhError
    ctx = Context(0)
    P = FH_NOALLOC_SCRATCH_DOUBLES  # M = 2 needs 2P doubles
    W = torch.ones((2, 1), dtype=torch.float64, device="cuda")
    D = torch.zeros(16, dtype=torch.float64, device="cuda")
    with pytest.raises(FhError) as e:
        ctx.call("fh_history_sum_noalloc", 2, 1, P, W.data_ptr(), 1, D.data_ptr(), P, D.data_ptr(), P)
    assert e.value.code == FH_ERANGE
    ctx.close()
