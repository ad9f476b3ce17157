"""Power iteration by repeated squaring (M^e v0 through 3xTF32 tensor-core squarings,
then plain steps to convergence) for the converging forms (canonical mode,
cal_select=1), against the plain power iteration (TIMESC_NO_SQUARING) and the FP64
oracle's converged eigenvector: centroids to 1e-4 per unit vector.  The compat form's
fixed m steps never square (checked: identical with and without the switch).
Cases: m a power of two and not, an empty cluster (keeps its centroid), a
three-member cluster, m = 5, and the BF16 form.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _extract(ctx, X, labels, C, mode, cal_select, prec, monkeypatch, squaring):
    import torch
    if squaring:
        monkeypatch.delenv("TIMESC_NO_SQUARING", raising=False)
    else:
        monkeypatch.setenv("TIMESC_NO_SQUARING", "1")
    c = dev(C)
    sc = ctx.extract_shapes(dev(X), dev(labels), c, mode=mode, cal_select=cal_select, precision=prec)
    torch.cuda.synchronize()
    monkeypatch.delenv("TIMESC_NO_SQUARING", raising=False)
    return sc, c.cpu().numpy()


@pytest.mark.parametrize("mode,cal_select", [(1, 0), (0, 1)])
@pytest.mark.parametrize("m,k,n", [(512, 6, 3000), (333, 5, 1500), (96, 4, 400), (5, 3, 60)])
def test_squaring_matches_stepping_and_oracle(gpu_ctx, built, monkeypatch, mode, cal_select, m, k, n):
    T, O = built
    data, truth = T.generate(n, m, k, noise=0.3, seed=m + 17 * k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    labels = truth.astype(np.int32).copy()
    labels[labels == k - 1] = 0  # an empty cluster
    if n > 100:
        labels[:3] = k - 1  # ... made a three-member one
    C = np.zeros((k, m), np.float32)
    sc1, g_sq = _extract(gpu_ctx, X, labels, C, mode, cal_select, 0, monkeypatch, True)
    sc2, g_st = _extract(gpu_ctx, X, labels, C, mode, cal_select, 0, monkeypatch, False)
    refC, _, refsc = O.extract(X.astype(np.float64), labels, C.astype(np.float64), mode, cal_select)
    assert sc1 == sc2 == refsc
    scale = 1.0 if mode == 0 else np.sqrt(m)
    e_sq = np.abs(g_sq - refC).max() / scale
    e_st = np.abs(g_st - refC).max() / scale
    assert e_sq < 1e-4, (e_sq, e_st)
    assert np.abs(g_sq - g_st).max() / scale < 2e-4


def test_squaring_bf16_form(gpu_ctx, built, monkeypatch):
    """The BF16 form's Gram feeds the same FP32-class squaring (canonical mode)."""
    T, O = built
    n, m, k = 4000, 512, 8
    data, truth = T.generate(n, m, k, noise=0.3, seed=5)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    C = np.zeros((k, m), np.float32)
    _, g_sq = _extract(gpu_ctx, X, truth.astype(np.int32), C, 1, 0, 1, monkeypatch, True)
    _, g_st = _extract(gpu_ctx, X, truth.astype(np.int32), C, 1, 0, 1, monkeypatch, False)
    refC, _, _ = O.extract(X.astype(np.float64), truth.astype(np.int32), C.astype(np.float64), 1)
    scale = np.sqrt(m)
    assert np.abs(g_sq - refC).max() / scale < 1e-3
    assert np.abs(g_sq - g_st).max() / scale < 1e-3


def test_compat_never_squares(gpu_ctx, built, monkeypatch):
    """Compat (cal_select 0) runs the m plain steps whatever the switch says."""
    T, O = built
    n, m, k = 1500, 128, 4
    data, truth = T.generate(n, m, k, noise=0.3, seed=8)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    C = np.zeros((k, m), np.float32)
    _, a = _extract(gpu_ctx, X, truth.astype(np.int32), C, 0, 0, 0, monkeypatch, True)
    _, b = _extract(gpu_ctx, X, truth.astype(np.int32), C, 0, 0, 0, monkeypatch, False)
    np.testing.assert_array_equal(a, b)
