"""Allocation-free SBD assignment (tc_sbd_assign_noalloc).

Some callers cannot allocate device memory on the call path: a serving loop that
has reserved all of HBM for resident jobs up front, or a latency-critical thread
that cannot take cudaMalloc's implicit device synchronisation.  For them the
library keeps the assignment's scratch in one static device array.  This test
calls that entry point through the C ABI twice in a row (different shapes, so the
shared array is reused with other contents) and checks each result against the
context-based tc_sbd_assign with TC_PREC_FP32: both paths run the same kernels on
twiddle tables from the same device kernel, so labels and distances must be
identical bit for bit (the context path's screening keeps exactly the unscreened
result).  It runs last so a failure here leaves every other test already run,
and it passes alone in a fresh process too.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _compare(T, O, ctx, n, m, k, mode, seed):
    """One allocation-free call against the context path on the same inputs."""
    import torch
    data, _ = T.generate(n, m, k, noise=0.3, seed=seed)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    rng = np.random.default_rng(seed)
    C = X[rng.choice(n, k, replace=False)] + 0.3 * rng.standard_normal((k, m)).astype(np.float32)
    x = torch.from_numpy(X).cuda()
    c = torch.from_numpy(C).cuda()
    lab_ref = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist_ref = torch.zeros(n, dtype=torch.float32, device="cuda")
    ctx.sbd_assign(x, c, mode=mode, labels=lab_ref, dist=dist_ref)
    lab = torch.full((n,), -7, dtype=torch.int32, device="cuda")
    dist = torch.full((n,), -7.0, dtype=torch.float32, device="cuda")
    T.sbd_assign_noalloc(x, c, lab, dist, mode=mode)
    torch.cuda.synchronize()
    assert np.array_equal(lab.cpu().numpy(), lab_ref.cpu().numpy())
    assert np.array_equal(dist.cpu().numpy(), dist_ref.cpu().numpy())


def test_noalloc_matches_context_assign_twice(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    T, O = built
    ctx = T.Context(0)
    try:
        _compare(T, O, ctx, 4000, 512, 32, T.MODE_COMPAT, seed=1)     # first call: sets the device up
        _compare(T, O, ctx, 1500, 300, 7, T.MODE_CANONICAL, seed=2)  # second call reuses the array
    finally:
        ctx.close()


def test_noalloc_rejects_oversize(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    T, _ = built
    x = torch.zeros((8, 4096), dtype=torch.float32, device="cuda")
    c = torch.zeros((300, 4096), dtype=torch.float32, device="cuda")  # 300 spectra of 2049 bins: > 4 MiB
    lab = torch.zeros(8, dtype=torch.int32, device="cuda")
    with pytest.raises(T.TimescError) as e:
        T.sbd_assign_noalloc(x, c, lab, mode=T.MODE_COMPAT)
    assert e.value.code == T.ERR_UNSUPPORTED and "static array" in str(e.value)
