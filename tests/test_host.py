"""Host-side product code and the C ABI surface (CPU only, no GPU calls)."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN_DIR = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def T(built):
    return built[0]


def header_symbols():
    with open(os.path.join(ROOT, "include", "timesc.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|void|uint64_t|const char\s*\*)\s+(tc_[a-z_0-9]+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(T):
    syms = header_symbols()
    assert len(syms) >= 15
    L = T.lib()
    for s in syms:
        assert hasattr(L, s), s
    assert set(syms) <= set(T.SIGNATURES), set(syms) - set(T.SIGNATURES)
    assert L.tc_version() == 1


def test_nm_shows_c_linkage():
    out = subprocess.run(["nm", "-D", "--defined-only", os.path.join(ROOT, "times-c_gb300", "lib", "libtimesc.so")],
                         capture_output=True, text=True).stdout
    for s in header_symbols():
        assert re.search(r"\bT %s$" % s, out, re.M), s


@pytest.mark.parametrize("name", ["parse_labeled_a", "parse_unlabeled_a", "parse_labeled_zero"])
def test_parser_matches_reference_reader(T, golden, name):
    labeled = "_labeled" in name
    data, labels = T.read_file(os.path.join(GOLDEN_DIR, name + ".txt"), labeled)
    np.testing.assert_array_equal(data, golden[name + "__data"])
    if labeled:
        np.testing.assert_array_equal(labels, golden[name + "__labels"])


def test_parser_whitespace_and_crlf(T, golden, tmp_path):
    ref = golden["parse_labeled_a__data"]
    lab = golden["parse_labeled_a__labels"]
    p = tmp_path / "ws.txt"
    with open(p, "w") as f:
        for l, row in zip(lab, ref):
            f.write(("%d\t" % l) + "  ".join("%.9g" % v for v in row) + "\r\n")
        f.write("\n\n")
    data, labels = T.read_file(str(p), True)
    np.testing.assert_array_equal(data, ref)
    np.testing.assert_array_equal(labels, lab)


def test_parser_errors(T, tmp_path):
    p = tmp_path / "ragged.txt"
    p.write_text("1,2,3\n4,5\n")
    with pytest.raises(T.TimescError) as e:
        T.read_file(str(p), False)
    assert e.value.code == T.ERR_IO and "row 2" in str(e.value)
    p2 = tmp_path / "badlabel.txt"
    p2.write_text("x,1,2\n")
    with pytest.raises(T.TimescError):
        T.read_file(str(p2), True)
    with pytest.raises(T.TimescError):
        T.read_file(str(tmp_path / "missing.txt"), False)
    p3 = tmp_path / "empty.txt"
    p3.write_text("\n\n")
    with pytest.raises(T.TimescError):
        T.read_file(str(p3), False)


def test_label_writer_matches_reference(T, golden, tmp_path):
    p = str(tmp_path / "labels.txt")
    T.write_labels(p, np.array([1, 2, 10, 3, -1]))
    with open(p, "rb") as f:
        assert f.read() == bytes(golden["writefile"])


def test_centroid_writer_roundtrip(T, tmp_path):
    C = np.random.default_rng(0).standard_normal((3, 17)).astype(np.float32)
    p = str(tmp_path / "c.txt")
    T.write_centroids(p, C)
    back, _ = T.read_file(p, False)
    np.testing.assert_array_equal(back, C)


def test_random_rows_match_reference(T, golden):
    for i in range(5):
        row = golden["select_%d" % i]
        n, k, seed = int(row[0]), int(row[1]), int(row[2])
        np.testing.assert_array_equal(T.random_select(n, k, seed), row[3:])
    with pytest.raises(T.TimescError):
        T.random_select(3, 4, 0)


def test_fft_size_rules(T, golden):
    for m, f in zip(golden["fftsize_m"], golden["fftsize_ref"]):
        assert T.fft_size(int(m), T.MODE_COMPAT) == f
    for m in (3, 64, 128, 512, 2709, 4096, 8192):
        F = T.fft_size(m, T.MODE_CANONICAL)
        assert F >= 2 * m - 1 and F // 2 < 2 * m - 1 and F & (F - 1) == 0


def test_k_from_labels(T):
    assert T.k_from_labels(np.array([1, 2, 3, 3])) == 3
    assert T.k_from_labels(np.array([0, 1, 2])) == 3
    assert T.k_from_labels(np.array([-1, 1, -1])) == 2


def test_generator_is_deterministic_and_shaped(T):
    a, la = T.generate(5000, 96, 4, noise=0.2, dirichlet=2.0, seed=3)
    b, lb = T.generate(5000, 96, 4, noise=0.2, dirichlet=2.0, seed=3)
    c, _ = T.generate(5000, 96, 4, noise=0.2, dirichlet=2.0, seed=4)
    np.testing.assert_array_equal(a, b)
    np.testing.assert_array_equal(la, lb)
    assert not np.array_equal(a, c)
    assert la.min() >= 0 and la.max() < 4
    e, le = T.generate(400, 64, 4, seed=0)
    assert np.array_equal(np.bincount(le), [100, 100, 100, 100])
    assert np.isfinite(a).all()


def test_create_without_gpu_returns_error(T):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(T.TimescError) as e:
        T.Context(0)
    assert e.value.code == T.ERR_CUDA


def test_cli_argument_handling():
    cli = os.path.join(ROOT, "times-c_gb300", "bin", "test")
    assert subprocess.run([cli]).returncode == 0            # no "-d": silent exit like the reference
    assert subprocess.run([cli, "-d", "0", "x"], capture_output=True).returncode == 2
    assert subprocess.run([cli, "-d", "0", "f", "4", "1", "0", "--mode", "bogus"],
                          capture_output=True).returncode == 2


def test_job_footprint_estimate(built):
    """tc_job_footprint (pool admission) is a host computation: it grows with n, m
    and k, counts the BF16 series copy of the tensor-core path, and is 0 for an
    invalid job."""
    T, _ = built
    lib = T.lib()

    def fp(n, m, k, prec=0, mode=0):
        j = T.Job(None, None, n, m, k, mode, prec, 0, 0, 10, 1, None)
        return int(lib.tc_job_footprint(ctypes.byref(j)))

    base = fp(10000, 512, 8)
    assert base > 2 * 10000 * 512 * 4
    assert fp(20000, 512, 8) > base and fp(10000, 1024, 8) > base and fp(10000, 512, 16) > base
    # BF16 at m <= 512: the BF16 series copy (n*512*2) on top of the FP32 buffers and BF16 Gram planes
    assert fp(10000, 512, 8, prec=1) >= 2 * 10000 * 512 * 4 + 2 * 10000 * 512 * 2
    assert fp(0, 512, 8) == 0 and fp(100, 1, 8) == 0
    # the serving form's large request (n=2e5, m=1024, k=16) stays in the single-digit GB
    assert 2e9 < fp(200000, 1024, 16) < 1e10


def _load_bench():
    import importlib.util
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(root, "bench.py"))
    b = importlib.util.module_from_spec(spec)
    argv = sys.argv
    sys.argv = ["bench.py"]
    try:
        spec.loader.exec_module(b)
    finally:
        sys.argv = argv
    return b


def test_bench_clock_window(tmp_path):
    """bench.py's clock record keeps only the nvidia-smi samples taken inside the timed
    region (with 25 ms of slack), collects the throttle reasons seen there, and falls
    back to every sample, saying so, when none landed inside."""
    import datetime
    import tempfile
    b = _load_bench()

    class FakeProc:
        def terminate(self):
            pass

        def wait(self):
            pass

    def clocks_with(samples, t0, t1):
        c = b.Clocks.__new__(b.Clocks)
        c.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False, dir=tmp_path)
        for ts, mhz, cap in samples:
            c.f.write("%s, %d, 2070, 900.0, Not Active, Not Active, Not Active, %s\n"
                      % (ts.strftime("%Y/%m/%d %H:%M:%S.%f")[:-3], mhz, "Active" if cap else "Not Active"))
        c.f.flush()
        c.p = FakeProc()
        c.t0, c.t1 = t0, t1
        return c.stop()

    now = datetime.datetime(2026, 1, 1, 12, 0, 0)
    ms = lambda x: now + datetime.timedelta(milliseconds=x)
    samples = [(ms(0), 1000, False), (ms(100), 2070, False), (ms(120), 2070, True), (ms(140), 2070, False),
               (ms(400), 1200, False)]
    r = clocks_with(samples, ms(90), ms(150))
    assert r["samples"] == 3 and r["sm_mhz"] == 2070.0
    assert r["reasons"] == ["sw_power_cap"]
    assert r["window"].startswith("timed region")
    r = clocks_with(samples, ms(200), ms(300))  # nothing inside: all samples, flagged
    assert r["samples"] == 5 and r["window"].startswith("no sample inside")
