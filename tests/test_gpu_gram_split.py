"""The tensor-core Gram with its K range split across CTAs (shares summed in a fixed
order) against one share per strip (TIMESC_GRAM_NOSPLIT) and the FP64 oracle.

Every strip of w column tiles runs as w * base shares (base from the launch's wave
occupancy, each share keeping at least 64 K blocks on average).  A different
summation order moves the Gram by rounding only: centroids within 2e-5 (3xTF32) /
1e-4 (BF16) of the one-share launch, and the FP32 form within 1e-4 of the oracle.
Cases: m = 512, k = 2, n = 40000 (one diagonal strip of 4 tiles and its neighbours)
and m = 300, k = 3, n = 60000 (3 row tiles, a partial last tile).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _extract(ctx, X, labels, k, prec, monkeypatch, split):
    import torch
    if split:
        monkeypatch.delenv("TIMESC_GRAM_NOSPLIT", raising=False)
    else:
        monkeypatch.setenv("TIMESC_GRAM_NOSPLIT", "1")
    c = dev(np.zeros((k, X.shape[1]), np.float32))
    sc = ctx.extract_shapes(dev(X), dev(labels), c, mode=0, precision=prec)
    torch.cuda.synchronize()
    monkeypatch.delenv("TIMESC_GRAM_NOSPLIT", raising=False)
    return sc, c.cpu().numpy()


@pytest.mark.parametrize("m,k,n", [(512, 2, 40000), (300, 3, 60000)])
@pytest.mark.parametrize("prec,tol", [(0, 2e-5), (1, 1e-4)])
def test_split_gram_matches_unsplit_and_oracle(gpu_ctx, built, monkeypatch, m, k, n, prec, tol):
    T, O = built
    data, truth = T.generate(n, m, k, noise=0.3, seed=m + k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    labels = truth.astype(np.int32)
    sc1, a = _extract(gpu_ctx, X, labels, k, prec, monkeypatch, True)
    sc2, b = _extract(gpu_ctx, X, labels, k, prec, monkeypatch, False)
    assert sc1 == sc2
    assert np.abs(a - b).max() < tol
    if prec == 0:
        refC, _, refsc = O.extract(X.astype(np.float64), labels, np.zeros((k, m)), 0)
        assert sc1 == refsc
        assert np.abs(a - refC).max() < 1e-4
