"""The screened FP32 assignment against the unscreened FP32 kernel (TIMESC_NO_SCREEN).

The BF16 tensor-core pass keeps, per series, every centroid whose BF16 distance is
within 2D of the BF16 minimum, D being a rigorous bound on |d_BF16 - d_FP32|; the FP32
FFT pass evaluates those in ascending order.  So labels (first centroid on ties),
distances, the change count and the distance sum must equal the unscreened kernel's
bit for bit.  Cases: ordinary data in both modes (compat with and without the pad
value 2), exact ties (duplicate centroids), near ties that overflow the candidate list
(all centroids within the threshold), zero rows, and whole k-Shape runs.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _assign(ctx, X, C, mode, old, monkeypatch, screen):
    import torch
    if screen:
        monkeypatch.delenv("TIMESC_NO_SCREEN", raising=False)
    else:
        monkeypatch.setenv("TIMESC_NO_SCREEN", "1")
    n = X.shape[0]
    lab = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    changed = torch.zeros(1, dtype=torch.int32, device="cuda")
    dsum = torch.zeros(1, dtype=torch.float64, device="cuda")
    ctx.sbd_assign(dev(X), dev(C), mode=mode, precision=0, labels=lab, dist=dist, old_labels=dev(old),
                   changed=changed, dist_sum=dsum)
    torch.cuda.synchronize()
    monkeypatch.delenv("TIMESC_NO_SCREEN", raising=False)
    return lab.cpu().numpy(), dist.cpu().numpy(), changed.item(), dsum.item()


def _same(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    assert a[2] == b[2]
    assert a[3] == b[3]


def _data(T, O, n, m, k, seed):
    data, truth = T.generate(n, m, k, noise=0.4, seed=seed)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    return X, truth.astype(np.int32)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("m,k,n", [(512, 32, 20000), (300, 12, 8000), (128, 5, 5000), (200, 64, 6000)])
def test_screened_equals_unscreened(gpu_ctx, built, monkeypatch, mode, m, k, n):
    T, O = built
    X, truth = _data(T, O, n, m, k, seed=m + k)
    rng = np.random.default_rng(k)
    C = X[rng.choice(n, k, replace=False)].copy()
    old = rng.integers(0, k, n).astype(np.int32)
    a = _assign(gpu_ctx, X, C, mode, old, monkeypatch, True)
    b = _assign(gpu_ctx, X, C, mode, old, monkeypatch, False)
    _same(a, b)


def test_ties_overflow_and_zero_rows(gpu_ctx, built, monkeypatch):
    T, O = built
    n, m, k = 6000, 256, 20
    X, _ = _data(T, O, n, m, k, seed=3)
    X[:50] = 0.0  # zero rows: NCC 0 against every centroid, all tie
    rng = np.random.default_rng(4)
    C = X[rng.choice(np.arange(100, n), k, replace=False)].copy()
    C[1] = C[0]  # exact tie: centroid 0 must win
    C[7] = C[3]
    base = X[200]
    for j in range(10, 20):  # near ties: more candidates than the list holds
        C[j] = base + 1e-4 * rng.standard_normal(m).astype(np.float32)
    old = np.zeros(n, np.int32)
    for mode in (0, 1):
        a = _assign(gpu_ctx, X, C, mode, old, monkeypatch, True)
        b = _assign(gpu_ctx, X, C, mode, old, monkeypatch, False)
        _same(a, b)
        assert a[0][200] >= 10  # series 200 sits on the near-tied group


@pytest.mark.parametrize("mode", [0, 1])
def test_whole_run_screened_equals_unscreened(gpu_ctx, built, monkeypatch, mode):
    T, _ = built
    data, _ = T.generate(8000, 256, 8, noise=0.3, seed=21)
    out = []
    for screen in (True, False):
        if screen:
            monkeypatch.delenv("TIMESC_NO_SCREEN", raising=False)
        else:
            monkeypatch.setenv("TIMESC_NO_SCREEN", "1")
        out.append(gpu_ctx.kshape_run(data, 8, mode=mode, precision=0, seed=2, max_iter=8))
    monkeypatch.delenv("TIMESC_NO_SCREEN", raising=False)
    np.testing.assert_array_equal(out[0]["labels"], out[1]["labels"])
    np.testing.assert_array_equal(out[0]["centroids"], out[1]["centroids"])
    assert out[0]["iterations"] == out[1]["iterations"]
