"""GPU parity of the tensor-core (tcgen05, BF16 operands, FP32 accumulation) SBD
assignment against the FP64 oracle.

The kernel correlates BF16-rounded series and centroids and divides by the FP32
norms of the unrounded data.  The oracle therefore runs on the BF16-rounded
inputs, and its NCC is rescaled by |x_bf16||c_bf16| / (|x||c|); what is left is
FP32 accumulation error:
  distances   abs 3e-5
  labels      identical wherever the oracle's best-vs-second margin exceeds 1e-4
Against the plain FP32 path on unrounded data the distances agree to 4e-3.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MARGIN = 1e-4


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def bf16_round(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).bfloat16().float().numpy()


def oracle_bf16(O, X, C, F, clamp2):
    """Oracle labels/distances of the BF16 correlation with FP32 norms."""
    Xr, Cr = bf16_round(X).astype(np.float64), bf16_round(C).astype(np.float64)
    X64, C64 = X.astype(np.float64), C.astype(np.float64)
    n, k = X.shape[0], C.shape[0]
    nx, nxr = np.linalg.norm(X64, axis=1), np.linalg.norm(Xr, axis=1)
    nc, ncr = np.linalg.norm(C64, axis=1), np.linalg.norm(Cr, axis=1)
    D = np.empty((n, k))
    for j in range(k):
        # per-centroid distances from the oracle with that centroid alone
        _, dj, _, _ = O.assign(Xr, Cr[j:j + 1], F, clamp2=False)
        with np.errstate(invalid="ignore", divide="ignore"):
            s = np.where((nx > 0) & (nc[j] > 0), (nxr * ncr[j]) / (nx * nc[j]), 0.0)
        D[:, j] = 1.0 - (1.0 - dj) * s
    if clamp2:
        D = np.minimum(D, 2.0)
    lab = np.argmin(D, axis=1)  # first minimum on ties, like get_pos_idx
    srt = np.sort(D, axis=1)
    margin = srt[:, 1] - srt[:, 0] if k > 1 else np.full(n, np.inf)
    return lab, D[np.arange(n), lab], margin


CASES = [
    # (mode, m, k, n): FFT length 128..1024, ragged last tile, several tiles per CTA
    (0, 100, 5, 1000), (0, 200, 3, 300), (0, 333, 8, 700), (0, 512, 33, 1500),
    (1, 33, 4, 500), (1, 64, 2, 129), (1, 100, 6, 900), (1, 333, 3, 400), (1, 512, 8, 1100),
    (0, 128, 1, 100), (1, 200, 4, 20000),
]


@pytest.mark.parametrize("mode,m,k,n", CASES)
def test_tc_assign_matches_oracle(gpu_ctx, mods_tc, mode, m, k, n):
    import torch
    T, O = mods_tc
    F = T.fft_size(m, mode)
    assert 128 <= F <= 1024
    data, truth = T.generate(n, m, max(k, 2), noise=0.3, seed=m + 7 * k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    rng = np.random.default_rng(m + k)
    C = X[rng.choice(n, k, replace=False)] + 0.4 * rng.standard_normal((k, m)).astype(np.float32)
    if k > 2:
        C[1] = 0.0  # zero centroid: NCC 0, distance 1
    X[3] = 0.0      # zero series
    x, c = dev(X), dev(C)
    lab = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    old = torch.from_numpy(np.minimum(truth, k - 1).astype(np.int32)).cuda()
    changed = torch.zeros(1, dtype=torch.int32, device="cuda")
    dsum = torch.zeros(1, dtype=torch.float64, device="cuda")
    gpu_ctx.sbd_assign(x, c, mode=mode, precision=T.PREC_BF16, labels=lab, dist=dist, old_labels=old,
                       changed=changed, dist_sum=dsum)
    torch.cuda.synchronize()
    L, D = lab.cpu().numpy(), dist.cpu().numpy()
    clamp2 = mode == 0 and 2 * m - 1 < 512
    ol, od, om = oracle_bf16(O, X, C, F, clamp2)
    clear = om > MARGIN
    tag = "mode=%d m=%d k=%d n=%d" % (mode, m, k, n)
    assert clear.mean() > 0.9, tag
    assert np.array_equal(L[clear], ol[clear]), (tag, np.flatnonzero((L != ol) & clear)[:10])
    np.testing.assert_allclose(D, od, atol=3e-5, err_msg=tag)
    assert L[3] == 0 and abs(D[3] - 1.0) < 1e-6  # zero series: every NCC 0, first centroid
    assert changed.item() == int((L != old.cpu().numpy()).sum())
    assert abs(dsum.item() - D.astype(np.float64).sum()) < 1e-6 * n

    # against the FP32 FFT path on the unrounded data
    dist32 = torch.zeros(n, dtype=torch.float32, device="cuda")
    lab32 = torch.zeros(n, dtype=torch.int32, device="cuda")
    gpu_ctx.sbd_assign(x, c, mode=mode, labels=lab32, dist=dist32)
    torch.cuda.synchronize()
    assert np.abs(dist32.cpu().numpy() - D).max() < 4e-3, tag


def test_tc_assign_shift_request_uses_fft(gpu_ctx, mods_tc):
    """A shift output is only produced by the FFT correlation: asking for it
    with BF16 gives the FP32 results exactly."""
    import torch
    T, O = mods_tc
    n, m, k = 300, 128, 4
    data, _ = T.generate(n, m, k, noise=0.3, seed=3)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    C = X[:k].copy()
    x, c = dev(X), dev(C)
    out = []
    for prec in (T.PREC_FP32, T.PREC_BF16):
        lab = torch.zeros(n, dtype=torch.int32, device="cuda")
        dist = torch.zeros(n, dtype=torch.float32, device="cuda")
        sh = torch.zeros(n, dtype=torch.int32, device="cuda")
        gpu_ctx.sbd_assign(x, c, mode=1, precision=prec, labels=lab, dist=dist, shift=sh)
        torch.cuda.synchronize()
        out.append((lab.cpu().numpy(), dist.cpu().numpy(), sh.cpu().numpy()))
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("mode", [0, 1])
def test_tc_kshape_loop_bf16(gpu_ctx, mods_tc, mode):
    """The whole loop with BF16 correlation and Gram matrices reaches the same
    partition as the FP32 loop on well-separated data."""
    T, O = mods_tc
    data, truth = T.generate(2000, 256, 6, noise=0.2, seed=11)
    init = np.random.default_rng(5).integers(0, 6, 2000).astype(np.int32)
    g32 = gpu_ctx.kshape_run(data, 6, mode=mode, init_labels=init, max_iter=50)
    g16 = gpu_ctx.kshape_run(data, 6, mode=mode, precision=T.PREC_BF16, init_labels=init, max_iter=50)
    assert O.ari(g16["labels"], g32["labels"]) >= 0.99
    assert O.ari(g16["labels"], truth) >= O.ari(g32["labels"], truth) - 0.02


@pytest.fixture(scope="module")
def mods_tc(built):
    return built


def test_tc_prepared_series(gpu_ctx, mods_tc):
    """Assignments on prepared series match unprepared ones; assigning other
    series in between drops the prepared copy instead of reusing it."""
    import torch
    T, O = mods_tc
    n, m, k = 3000, 256, 5
    d1, _ = T.generate(n, m, k, noise=0.3, seed=21)
    d2, _ = T.generate(n, m, k, noise=0.3, seed=22)
    x1 = dev(O.znorm(d1.astype(np.float64)).astype(np.float32))
    x2 = dev(O.znorm(d2.astype(np.float64)).astype(np.float32))
    c = x1[:k].clone()

    def run(x):
        lab = torch.zeros(n, dtype=torch.int32, device="cuda")
        dist = torch.zeros(n, dtype=torch.float32, device="cuda")
        gpu_ctx.sbd_assign(x, c, mode=1, precision=T.PREC_BF16, labels=lab, dist=dist)
        torch.cuda.synchronize()
        return lab.cpu().numpy(), dist.cpu().numpy()

    ref1, ref2 = run(x1), run(x2)
    gpu_ctx.prepare_series(x1)
    for _ in range(2):
        a = run(x1)
        assert np.array_equal(a[0], ref1[0]) and np.array_equal(a[1], ref1[1])
    b = run(x2)
    assert np.array_equal(b[1], ref2[1])
    x1.mul_(-1.0)  # changed after its copy was dropped: the next call converts again
    a = run(x1)
    assert not np.array_equal(a[1], ref1[1])
