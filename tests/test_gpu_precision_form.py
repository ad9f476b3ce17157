"""The precision form against the FP64 oracle, on the precision configuration's series
length (m = 512) and generator with fewer series.

* One iteration from the same state: the mixed form (BF16 tensor-core correlation and
  Gram, FP32 accumulation) and the plain FP32 form extract centroids from the oracle
  loop's final labels and assign against the oracle's final centroids.  Centroid error
  <= 1e-3 for BF16 and <= 1e-4 for FP32 (per unit-norm vector), label ARI >= 0.99 for
  both, SBD distance error <= 4e-3 for BF16 and 2e-5 for FP32.
* Whole runs in compat mode from the same initial labels: label ARI >= 0.99 for both
  forms.  (In canonical mode ten iterations from random labels do not converge, and
  BF16 rounding of near-tie distances sends the run along another path: the ARI of two
  such runs measures the path, not the arithmetic, so it is only reported.)
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.fixture(scope="module")
def state(built):
    T, O = built
    n, m, k = 4000, 512, 16
    data, _ = T.generate(n, m, k, noise=0.3, seed=123)
    init = np.random.default_rng(9).integers(0, k, n).astype(np.int32)
    runs = {mode: O.kshape(data, k, mode, init, max_iter=10) for mode in (0, 1)}
    X = O.znorm(data.astype(np.float64))
    return data, init, X, runs, k


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("prec,cerr,derr", [(1, 1e-3, 4e-3), (0, 1e-4, 2e-5)])
def test_one_iteration_vs_fp64_oracle(gpu_ctx, built, state, mode, prec, cerr, derr):
    import torch
    T, O = built
    data, init, X, runs, k = state
    n, m = X.shape
    o = runs[mode]
    lab, Cprev = o["labels"], o["centroids"]
    # extraction from the oracle's labels, with the oracle's centroids as the previous ones
    refC, _, _ = O.extract(X, lab, Cprev, mode)
    x = dev(X.astype(np.float32))
    c = dev(Cprev.astype(np.float32))
    gpu_ctx.extract_shapes(x, dev(lab), c, mode=mode, precision=prec)
    torch.cuda.synchronize()
    scale = 1.0 if mode == 0 else np.sqrt(m)
    err = np.abs(c.cpu().numpy() - refC).max() / scale
    assert err <= cerr, (prec, mode, err)
    # assignment against the oracle's centroids
    F = T.fft_size(m, mode)
    ol, od, _, _ = O.assign(X, refC, F, clamp2=(mode == 0 and 2 * m - 1 < 512))
    labels = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    gpu_ctx.sbd_assign(x, dev(refC.astype(np.float32)), mode=mode, precision=prec, labels=labels, dist=dist)
    torch.cuda.synchronize()
    L, D = labels.cpu().numpy(), dist.cpu().numpy()
    assert O.ari(L, ol) >= 0.99, (prec, mode, O.ari(L, ol))
    assert np.abs(D - od).max() <= derr, (prec, mode, np.abs(D - od).max())


@pytest.mark.parametrize("prec", [1, 0])
def test_whole_run_compat_vs_fp64_oracle(gpu_ctx, built, state, prec):
    T, O = built
    data, init, X, runs, k = state
    g = gpu_ctx.kshape_run(data, k, mode=0, precision=prec, init_labels=init, max_iter=10)
    assert O.ari(g["labels"], runs[0]["labels"]) >= 0.99
