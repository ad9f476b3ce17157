"""GPU parity: every stage and the whole loop through the C ABI against the
FP64 oracle on the same inputs.

Tolerances (FP32 kernels vs the FP64 restatement):
  z-norm values           abs 2e-6
  SBD distances           abs 2e-6 (m <= 1024), 1e-5 (longer series)
  labels                  identical wherever the oracle's best-vs-second margin
                          exceeds 1e-5 (five times the distance tolerance: below
                          that FP32 rounding may pick either); the number of
                          series under the margin is printed
  shifts                  identical, or the GPU lag's NCC within 2e-6 of the max
  centroids               1e-5 relative: max |c - c_oracle| <= 1e-5 max |c_oracle|
  whole loops             labels identical when no assignment of the oracle's run
                          came within 1e-5 of a tie; otherwise ARI >= 0.99, and the
                          test prints that the fallback was taken
"""
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MARGIN = 1e-5
CENTROID_REL = 1e-5


def dist_tol(m):
    return 2e-6 if m <= 1024 else 1e-5


@pytest.fixture(scope="module")
def mods(built):
    return built


def dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def make_data(T, n, m, k, seed, noise=0.2):
    data, truth = T.generate(n, m, k, noise=noise, seed=seed)
    return data, truth


@pytest.mark.parametrize("m", [5, 64, 128, 333, 512, 1024, 1500, 2709, 4096, 8192])
def test_znorm(gpu_ctx, mods, m):
    T, O = mods
    n = 64 if m > 2048 else 300
    data, _ = make_data(T, n, m, 3, seed=m)
    data[5] = 3.25  # constant row -> zeros
    x = dev(data)
    gpu_ctx.znorm(x, ddof=1)
    ref = O.znorm(data.astype(np.float64), ddof=1)
    np.testing.assert_allclose(x.cpu().numpy(), ref, atol=2e-6)
    assert np.all(x.cpu().numpy()[5] == 0)


def test_init_labels_deterministic(gpu_ctx):
    import torch
    a = torch.zeros(100000, dtype=torch.int32, device="cuda")
    b = torch.zeros_like(a)
    gpu_ctx.init_labels(a, 7)
    gpu_ctx.init_labels(b, 7)
    assert torch.equal(a, b)
    h = a.cpu().numpy()
    assert h.min() == 0 and h.max() == 6
    cnt = np.bincount(h, minlength=7)
    assert cnt.min() > 0.9 * 100000 / 7


def _check_assign(O, X, C, F, labels, dist, shift, clamp2, tag):
    ol, od, osh, om = O.assign(X, C, F, clamp2=clamp2)
    clear = om > MARGIN
    m = X.shape[1]
    derr = float(np.abs(dist[clear] - od[clear]).max()) if clear.any() else 0.0
    print("%s: %d of %d series within %.0e of a tie, labels differ elsewhere %d, max distance error %.2e"
          % (tag, int((~clear).sum()), len(labels), MARGIN, int((labels != ol)[clear].sum()), derr))
    assert np.array_equal(labels[clear], ol[clear]), (tag, np.flatnonzero((labels != ol) & clear)[:10])
    assert derr <= dist_tol(m), (tag, derr)
    # shift: same lag, or a lag whose NCC is within the distance tolerance of the max
    bad = 0
    for i in np.flatnonzero(clear & (shift != osh)):
        c = C[ol[i]]
        ncc_align = O.ncc(c, X[i], F)  # NCC(center, member): slot j <-> shift j - m + 1
        if ncc_align.max() - ncc_align[shift[i] + m - 1] > dist_tol(m):
            bad += 1
    assert bad == 0, (tag, bad)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("m,k,n", [(5, 3, 200), (16, 2, 300), (64, 8, 500), (100, 5, 400), (128, 4, 300),
                                   (129, 6, 300), (300, 3, 200), (512, 32, 600), (1000, 4, 100),
                                   (2709, 8, 60), (4096, 3, 30)])
def test_sbd_assign(gpu_ctx, mods, mode, m, k, n):
    import torch
    T, O = mods
    data, truth = make_data(T, n, m, k, seed=m + k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    rng = np.random.default_rng(m)
    C = X[rng.choice(n, k, replace=False)] + 0.5 * rng.standard_normal((k, m)).astype(np.float32)
    if k > 2:
        C[1] = 0.0  # empty / zero centroid: NCC 0, distance 1
    X[3] = 0.0      # zero series
    F = T.fft_size(m, mode)
    x, c = dev(X), dev(C)
    lab = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    sh = torch.zeros(n, dtype=torch.int32, device="cuda")
    old = torch.from_numpy(truth).cuda()
    changed = torch.zeros(1, dtype=torch.int32, device="cuda")
    dsum = torch.zeros(1, dtype=torch.float64, device="cuda")
    gpu_ctx.sbd_assign(x, c, mode=mode, labels=lab, dist=dist, shift=sh, old_labels=old, changed=changed,
                       dist_sum=dsum)
    torch.cuda.synchronize()
    L, D, S = lab.cpu().numpy(), dist.cpu().numpy(), sh.cpu().numpy()
    _check_assign(O, X.astype(np.float64), C.astype(np.float64), F, L, D, S, mode == 0 and 2 * m - 1 < 512,
                  "m=%d k=%d mode=%d" % (m, k, mode))
    assert changed.item() == int((L != truth).sum())
    assert abs(dsum.item() - D.astype(np.float64).sum()) < 1e-6 * n


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("m,k,n,cinit", [(64, 3, 300, "zero"), (128, 4, 400, "raw"), (128, 4, 400, "unit"),
                                         (333, 5, 500, "raw"), (512, 8, 1200, "unit"), (1500, 3, 150, "raw")])
def test_extract_shapes(gpu_ctx, mods, mode, m, k, n, cinit):
    import torch
    T, O = mods
    data, truth = make_data(T, n, m, k, seed=7 * m + k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    labels = truth.copy()
    labels[labels == k - 1] = 0  # one empty cluster: keeps its centroid
    rng = np.random.default_rng(1)
    if cinit == "zero":
        C = np.zeros((k, m), np.float32)
    elif cinit == "raw":  # un-normalised rows (the init_chose=1 start): compat gate opens
        C = data[rng.choice(n, k, replace=False)].copy()
    else:  # unit vectors: compat gate closed, canonical gate open
        C = rng.standard_normal((k, m)).astype(np.float32)
        C /= np.linalg.norm(C, axis=1, keepdims=True)
    x, lab, c = dev(X), dev(labels), dev(C)
    counts = torch.zeros(k, dtype=torch.int32, device="cuda")
    sc = gpu_ctx.extract_shapes(x, lab, c, mode=mode, counts=counts)
    torch.cuda.synchronize()
    refC, refcnt, refsc = O.extract(X.astype(np.float64), labels, C.astype(np.float64), mode)
    assert sc == refsc
    np.testing.assert_array_equal(counts.cpu().numpy(), refcnt)
    got = c.cpu().numpy()
    rel = float(np.abs(got - refC).max() / np.abs(refC).max())
    print("extract m=%d k=%d mode=%d start=%s: centroid error %.2e relative" % (m, k, mode, cinit, rel))
    assert rel <= CENTROID_REL, rel


@pytest.mark.parametrize("prec,tol", [(2, 2e-3), (1, 1e-2)])
@pytest.mark.parametrize("m,k,n", [(128, 4, 700), (300, 3, 500), (512, 8, 3000), (1000, 2, 200)])
def test_extract_tensor_core_gram(gpu_ctx, mods, prec, tol, m, k, n):
    """Mixed-precision extraction: TF32 (prec 2) / BF16 (prec 1) Gram on tcgen05."""
    import torch
    T, O = mods
    data, truth = make_data(T, n, m, k, seed=3 * m + k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    C = np.zeros((k, m), np.float32)
    x, lab, c = dev(X), dev(truth), dev(C)
    sc = gpu_ctx.extract_shapes(x, lab, c, mode=0, precision=prec)
    torch.cuda.synchronize()
    refC, _, refsc = O.extract(X.astype(np.float64), truth, C.astype(np.float64), 0)
    assert sc == refsc
    err = np.abs(c.cpu().numpy() - refC).max()
    assert err < tol, err


@pytest.mark.parametrize("m,k,n", [(512, 8, 4000), (2709, 3, 400)])
def test_fp32_gram_3xtf32_matches_simt(gpu_ctx, mods, m, k, n, monkeypatch):
    """The plain FP32 extraction's 3xTF32 tensor-core Gram against the SIMT FP32 Gram."""
    import torch
    T, O = mods
    data, truth = make_data(T, n, m, k, seed=11 * m + k)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    out = []
    for simt in (False, True):
        if simt:
            monkeypatch.setenv("TIMESC_SIMT_GRAM", "1")
        c = dev(np.zeros((k, m), np.float32))
        gpu_ctx.extract_shapes(dev(X), dev(truth), c, mode=0)
        torch.cuda.synchronize()
        out.append(c.cpu().numpy())
    monkeypatch.delenv("TIMESC_SIMT_GRAM", raising=False)
    assert np.abs(out[0] - out[1]).max() < 2e-5


def _cpu_labels_via_gpu_init(ctx, n, k):
    import torch
    t = torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx.init_labels(t, k)
    return t.cpu().numpy()


@pytest.mark.parametrize("mode,init_chose,seed", [(0, 0, 0), (0, 1, 1), (1, 0, 0), (1, 1, 2)])
def test_kshape_loop_matches_oracle(gpu_ctx, mods, mode, init_chose, seed):
    T, O = mods
    data, truth = make_data(T, 300, 128, 4, seed=0)
    init = _cpu_labels_via_gpu_init(gpu_ctx, 300, 4)
    g = gpu_ctx.kshape_run(data, 4, mode=mode, init_chose=init_chose, seed=seed, max_iter=100)
    o = O.kshape(data, 4, mode, init, init_chose=init_chose, seed=seed, max_iter=100)
    assert g["restarted"] == o["restarted"]
    rel = float(np.abs(g["centroids"] - o["centroids"]).max() / np.abs(o["centroids"]).max())
    print("loop mode=%d init=%d seed=%d: oracle min margin %.1e, labels differ %d, centroid error %.2e relative"
          % (mode, init_chose, seed, o["min_margin"], int((g["labels"] != o["labels"]).sum()), rel))
    if o["min_margin"] > MARGIN:
        np.testing.assert_array_equal(g["labels"], o["labels"])
        assert g["iterations"] == o["iterations"] and g["sum_class"] == o["sum_class"]
        assert rel <= CENTROID_REL, rel
    else:
        print("  fallback taken: the oracle's run came within %.0e of a tie; ARI %.4f"
              % (MARGIN, O.ari(g["labels"], o["labels"])))
        assert O.ari(g["labels"], o["labels"]) >= 0.99


def test_kshape_given_init_labels_and_restart(gpu_ctx, mods):
    T, O = mods
    data, _ = make_data(T, 300, 128, 4, seed=0)
    init = np.zeros(300, np.int32)  # one cluster -> sum_class 1 -> restart with the full eigensolver
    g = gpu_ctx.kshape_run(data, 4, init_labels=init, max_iter=10)
    o = O.kshape(data, 4, 0, init, max_iter=10)
    assert g["restarted"] == 1 and o["restarted"] == 1


def test_cli_labeled_file(gpu_ctx, mods, tmp_path):
    T, O = mods
    data, truth = make_data(T, 300, 128, 4, seed=0)
    path = tmp_path / "c1.txt"
    with open(path, "w") as f:
        for l, row in zip(truth + 1, data):
            f.write("%d," % l + ",".join("%.8g" % v for v in row) + "\n")
    parsed, _ = T.read_file(str(path), True)
    out = tmp_path / "labels.txt"
    cen = tmp_path / "cent.txt"
    cli = os.path.join(os.path.dirname(T.LIB_PATH), "..", "bin", "test")
    r = subprocess.run([cli, "-d", "0", str(path), "4", "0", "0", "--labels-out", str(out),
                        "--centroids-out", str(cen)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    labels = np.array([int(v) for v in open(out).read().split(",") if v != ""]) - 1
    init = _cpu_labels_via_gpu_init(gpu_ctx, 300, 4)
    o = O.kshape(parsed, 4, 0, init, max_iter=10)
    if o["min_margin"] > MARGIN:
        np.testing.assert_array_equal(labels, o["labels"])
    else:
        print("cli: fallback taken (oracle min margin %.1e)" % o["min_margin"])
        assert O.ari(labels, o["labels"]) >= 0.99
    C, _ = T.read_file(str(cen), False)
    assert C.shape == (4, 128)


def test_errors_are_status_codes(gpu_ctx, mods):
    import torch
    T, _ = mods
    x = torch.zeros((10, 3), dtype=torch.float32, device="cuda")
    c = torch.zeros((2, 3), dtype=torch.float32, device="cuda")
    lab = torch.zeros(10, dtype=torch.int32, device="cuda")
    with pytest.raises(T.TimescError) as e:  # compat FFT length 4 < 8
        gpu_ctx.sbd_assign(x, c, mode=0, labels=lab)
    assert e.value.code == T.ERR_UNSUPPORTED
    with pytest.raises(T.TimescError):
        gpu_ctx.kshape_run(np.zeros((3, 16), np.float32), 5, init_chose=1)  # k > n
    # the context stays usable
    y = torch.randn(4, 32, device="cuda")
    gpu_ctx.znorm(y)
    torch.cuda.synchronize()
