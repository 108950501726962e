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
