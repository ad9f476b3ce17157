"""The oracle pinned against the reference's own code (CPU only).

Golden outputs in tests/golden/reference_golden.npz were produced by
tests/golden/make_golden.py from the reference's test_timesC.py functions and
from its host-side C++ (readFile/writeFile/randomSelectK/fft-size rule,
compiled into oracle/_ref).
"""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def O(built):
    return built[1]


def test_ncc_matches_reference_python(O, golden):
    for m in (7, 33, 64, 128):
        x, y, ref = golden["ncc_m%d_x" % m], golden["ncc_m%d_y" % m], golden["ncc_m%d_out" % m]
        F = O.fft_size(m, O.MODE_CANONICAL)
        for j in range(y.shape[0]):
            for i in range(x.shape[0]):
                np.testing.assert_allclose(O.ncc(x[i], y[j], F), ref[j][i], atol=1e-12)


def test_ncc_fft_equals_direct_sum_with_wraparound(O):
    rng = np.random.default_rng(5)
    for m in (5, 64, 100, 128, 129, 300):
        x, y = rng.standard_normal(m), rng.standard_normal(m)
        for mode in (O.MODE_COMPAT, O.MODE_CANONICAL):
            F = O.fft_size(m, mode)
            np.testing.assert_allclose(O.ncc(x, y, F), O.ncc(x, y, F, naive=True), atol=1e-12)


def test_znorm_matches_reference_zscore(O, golden):
    a = golden["zscore_in"]
    np.testing.assert_allclose(O.znorm(a, ddof=0), golden["zscore_ddof0"], atol=1e-12)
    np.testing.assert_allclose(O.znorm(a, ddof=1), golden["zscore_ddof1"], atol=1e-12)


def test_zero_fill_shift_matches_roll_zeropad(O, golden):
    v = golden["roll_in"]
    for s, ref in zip(golden["roll_shifts"], golden["roll_out"]):
        np.testing.assert_array_equal(O.shift_row(v, int(s)), ref)


def test_alignment_matches_reference_sbd(O, golden):
    c = golden["sbd_center"]
    F = O.fft_size(c.shape[0], O.MODE_CANONICAL)
    for mem, ref_shifted, ref_d in zip(golden["sbd_members"], golden["sbd_shifted"], golden["sbd_dist"]):
        s, out = O.align(c, mem, F)
        np.testing.assert_allclose(out, ref_shifted, atol=1e-12)
        assert abs((1 - O.ncc(c, mem, F).max()) - ref_d) < 1e-12


def test_extract_shape_matches_reference(O, golden):
    mem = golden["extract_members"]
    C, counts, sc = O.extract(mem, np.zeros(mem.shape[0], np.int32), np.zeros((1, mem.shape[1])), O.MODE_PYREF)
    assert sc == 1 and counts[0] == mem.shape[0]
    np.testing.assert_allclose(C[0], golden["extract_out"], atol=1e-6)


def test_center_merge_matches_reference(O, golden):
    mem, cen = golden["merge_members"], golden["merge_center"]
    C, _, _ = O.extract(mem, np.zeros(mem.shape[0], np.int32), cen[None, :], O.MODE_PYREF)
    np.testing.assert_allclose(C[0], golden["merge_out"], atol=1e-6)


@pytest.mark.parametrize("seed", [0, 1])
def test_whole_cpu_loop_matches_reference(O, golden, seed):
    data = golden["c1_data"]
    r = O.kshape(data, 4, O.MODE_PYREF, golden["loop%d_init" % seed], max_iter=10)
    np.testing.assert_array_equal(r["labels"], golden["loop%d_labels" % seed])
    np.testing.assert_allclose(r["centroids"], golden["loop%d_centroids" % seed], atol=1e-6)


def test_fft_size_rule_matches_reference_build(O, golden):
    for m, f in zip(golden["fftsize_m"], golden["fftsize_ref"]):
        assert O.fft_size(int(m), O.MODE_COMPAT) == f


def test_random_rows_match_reference(O, golden):
    for i in range(5):
        row = golden["select_%d" % i]
        n, k, seed = int(row[0]), int(row[1]), int(row[2])
        np.testing.assert_array_equal(O.random_select(n, k, seed), row[3:])


def test_top_eigenvector_against_numpy(O):
    rng = np.random.default_rng(3)
    A = rng.standard_normal((40, 40))
    A = A @ A.T
    lam, v = O.top_eig(A)
    w, V = np.linalg.eigh(A)
    assert abs(lam - w[-1]) < 1e-9 * w[-1]
    assert abs(abs(v @ V[:, -1]) - 1) < 1e-10


def test_k_from_labels(O):
    assert O.k_from_labels(np.array([1, 2, 3])) == 3
    assert O.k_from_labels(np.array([0, 1, 2])) == 3
    assert O.k_from_labels(np.array([-1, 1, 1])) == 2


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("init_chose", [0, 1])
def test_loop_runs_and_clusters(O, golden, mode, init_chose):
    data, truth = golden["c1_data"], golden["c1_truth"]
    rng = np.random.default_rng(11)
    init = rng.integers(0, 4, size=data.shape[0]).astype(np.int32)
    r = O.kshape(data, 4, mode, init, init_chose=init_chose, seed=1, max_iter=100)
    assert r["labels"].min() >= 0 and r["labels"].max() < 4
    if init_chose == 0:
        assert O.ari(r["labels"], truth) > 0.5
    else:
        # raw (offset) rows as first centroids often leave exactly k/2 clusters;
        # the reference then stops without its restart (sum_class < k/2 is false)
        assert r["sum_class"] >= 2


def test_restart_rule(O, golden):
    """k_shape breaks at sum_class <= k/2; the driver restarts only below k/2."""
    data = golden["c1_data"]
    init = np.zeros(data.shape[0], np.int32)  # one cluster: sum_class = 1 -> restart
    r = O.kshape(data, 4, O.MODE_COMPAT, init, max_iter=10)
    assert r["restarted"] == 1
