"""Generates tests/golden/reference_golden.npz from the reference's own code.

Run where the Times-C tree is present (TIMESC_REFERENCE, else the directory
`reference` beside the repository):  python tests/golden/make_golden.py

* Code/test/test_timesC.py is imported (numpy >= 2 removed np.Inf, which it
  uses: the alias is restored before import).  Its functions are run on seeded
  inputs: _ncc_c_3dim, zscore, roll_zeropad, _sbd, _extract_shape,
  centerMerge and the whole _kshape loop (np.random seeded; its initial
  labels are the first randint draw and are stored with the result).
* oracle/_ref/ref_harness (the reference's readFile/read_unlabeled_File/
  writeFile, randomSelectK and FFT-size expression, compiled by
  oracle/build.py) is run on the parse fixtures in tests/golden/ and on a few
  (n, k, seed) draws.

The inputs are stored next to the outputs, so the tests never need the
reference tree.  Series data come from the engine's synthetic generator.
"""
import contextlib
import importlib.util
import io
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("TIMESC_REFERENCE", os.path.join(os.path.dirname(ROOT), "reference"))
sys.path.insert(0, os.path.join(ROOT, "times-c_gb300"))
import timesc  # noqa: E402


def load_reference_py():
    if not hasattr(np, "Inf"):
        np.Inf = np.inf
    path = os.path.join(REF, "Code", "test", "test_timesC.py")
    spec = importlib.util.spec_from_file_location("test_timesC", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def quiet(fn, *a):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a)


def harness():
    h = os.path.join(ROOT, "oracle", "_ref", "ref_harness")
    if not os.path.exists(h):
        raise SystemExit("build oracle/_ref first: python oracle/build.py")
    return h


def parse_fixtures(out):
    """The reference's text reader on the committed parse fixtures."""
    h = harness()
    for name in sorted(os.listdir(HERE)):
        if not name.startswith("parse_") or not name.endswith(".txt"):
            continue
        labeled = 1 if "_labeled" in name else 0
        tmp = os.path.join(HERE, "_tmp.bin")
        subprocess.run([h, "read", os.path.join(HERE, name), str(labeled), tmp], check=True)
        raw = np.fromfile(tmp, dtype=np.int32)
        os.remove(tmp)
        rows, cols, nl = raw[:3]
        labels = raw[3:3 + nl]
        data = raw[3 + nl:].view(np.float32).reshape(rows, cols)
        key = name[:-4]
        out[key + "__data"] = data
        out[key + "__labels"] = labels.astype(np.int32)


def main():
    ref = load_reference_py()
    out = {}
    rng = np.random.default_rng(2024)

    # NCC over all lags with the Python padding (= canonical FFT length)
    for m in (7, 33, 64, 128):
        x = rng.standard_normal((5, m))
        y = rng.standard_normal((3, m))
        y[2] = 0.0  # zero norm -> inf denominator -> 0
        out["ncc_m%d_x" % m] = x
        out["ncc_m%d_y" % m] = y
        out["ncc_m%d_out" % m] = ref._ncc_c_3dim(x, y)

    # zscore ddof 0/1 (with a constant row)
    a = rng.standard_normal((6, 50)) * 3 + 1
    a[3] = 2.5
    out["zscore_in"] = a
    out["zscore_ddof0"] = ref.zscore(a, axis=1, ddof=0)
    out["zscore_ddof1"] = ref.zscore(a, axis=1, ddof=1)

    # roll_zeropad
    v = rng.standard_normal(20)
    shifts = np.array([-25, -20, -19, -7, -1, 0, 1, 5, 19, 20, 25])
    out["roll_in"] = v
    out["roll_shifts"] = shifts
    out["roll_out"] = np.stack([ref.roll_zeropad(v, int(s)) for s in shifts])

    # _sbd(center, member): k-Shape alignment of a member to a centroid
    m = 64
    cen = rng.standard_normal(m)
    mem = np.stack([np.roll(cen, s) + 0.3 * rng.standard_normal(m) for s in (-9, -1, 0, 3, 17)])
    out["sbd_center"] = cen
    out["sbd_members"] = mem
    res = [ref._sbd(cen, mm) for mm in mem]
    out["sbd_dist"] = np.array([r[0] for r in res])
    out["sbd_shifted"] = np.stack([r[1] for r in res])

    # data for the extraction / loop fixtures (the configuration with n=300, m=128, k=4)
    data, truth = timesc.generate(300, 128, 4, noise=0.2, dirichlet=0.0, seed=0)
    out["c1_data"] = data
    out["c1_truth"] = truth
    x64 = data.astype(np.float64)
    xz = ref.zscore(x64, axis=1, ddof=0)
    # _extract_shape of one class (zero centroid -> no alignment)
    members = xz[truth == 1][:40].copy()
    np.random.seed(7)
    out["extract_members"] = members
    out["extract_out"] = quiet(ref._extract_shape, members.copy(), members.shape[1])
    # centerMerge: reversed alignment to a non-zero centroid, then extraction
    np.random.seed(8)
    center = out["extract_out"].copy()
    mem2 = xz[truth == 1][40:70].copy()
    out["merge_members"] = mem2
    out["merge_center"] = center
    out["merge_out"] = quiet(ref.centerMerge, mem2.copy(), center.copy(), mem2.shape[1])

    # the whole CPU loop
    for seed in (0, 1):
        np.random.seed(seed)
        init = np.random.randint(0, 4, size=300)
        np.random.seed(seed)
        idx, clusters, _ = quiet(ref.kshape, x64.copy(), 4)
        out["loop%d_init" % seed] = init.astype(np.int32)
        out["loop%d_labels" % seed] = np.asarray(idx, dtype=np.int32)
        out["loop%d_centroids" % seed] = np.stack([c[0] for c in clusters])

    # reference host code through the harness
    h = harness()
    parse_fixtures(out)
    for i, (n, k, seed) in enumerate([(300, 4, 0), (300, 4, 1), (20000, 8, 1), (50, 50, 3), (1000000, 32, 12345)]):
        r = subprocess.run([h, "select", str(n), str(k), str(seed)], check=True, capture_output=True, text=True)
        out["select_%d" % i] = np.array([n, k, seed] + [int(t) for t in r.stdout.split()], dtype=np.int64)
    ms = list(range(1, 300)) + [512, 1000, 1024, 1025, 2709, 4096, 4097, 8192]
    fs = [int(subprocess.run([h, "fftsize", str(mm)], check=True, capture_output=True, text=True).stdout)
          for mm in ms]
    out["fftsize_m"] = np.array(ms)
    out["fftsize_ref"] = np.array(fs)
    tmp = os.path.join(HERE, "_tmp_labels.txt")
    subprocess.run([h, "write", tmp, "1", "2", "10", "3", "-1"], check=True)
    out["writefile"] = np.frombuffer(open(tmp, "rb").read(), dtype=np.uint8)
    os.remove(tmp)
    np.savez_compressed(os.path.join(HERE, "reference_golden.npz"), **out)
    print("wrote", os.path.join(HERE, "reference_golden.npz"))


if __name__ == "__main__":
    main()
