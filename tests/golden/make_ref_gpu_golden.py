"""Generates tests/golden/ref_gpu_golden.npz from the reference's own GPU code.

Runs on a GPU host, after `python oracle/build.py ref_gpu` has compiled
oracle/_ref/ref_gpu (the reference's z-norm, NCC_3D + get_pos_idx,
extract_shape and k_shape / k_shape_tsl around our driver; see
oracle/ref_gpu_harness.cu).  The reference headers reach the GPU host as the
git-ignored copy staged under oracle/_ref/src by oracle/build.py.

    python tests/golden/make_ref_gpu_golden.py OUT_DIR [--time]

Writes OUT_DIR/ref_gpu_golden.npz; copy it to tests/golden/.  Series come from
the engine's synthetic generator and are stored with the outputs, so the tests
never need the reference or its build.  Cases (compat FFT lengths all wrap:
F < 2m - 1):

* c1: n=300, m=128, k=4 (the labelled CPU-sized configuration, F=128);
* w100, w129, w300, w512: m = 100 (F=128), 129 (F=256), 300 (F=512),
  512 (F=512); the first two also take the pad-with-2 rule of get_pos_idx
  (2m - 1 < 512).

Per case:
* init: the curand labels of init_chose=0 (idx_init), 1-based;
* loop: the reference's whole path after parsing (z-norm, k_shape or
  k_shape_tsl, the cal_select=1 restart) from the raw series: init_chose=0
  (curand labels) and init_chose=1 with mt19937 seeds 0 and 1 (the seeded
  random_device shim); iteration cap 10 for c1 (labelled driver) and 20
  otherwise (unlabelled driver);
* znorm: z_norm_gpu_x on the raw series;
* extract: extract_shape on FP64-z-normalised series (rounded to float) with
  the generator's class labels, from zero centroids (gate closed), raw rows
  (gate open: members aligned by sbd3D) and unit-norm centroids, with
  cal_select 0 and 1;
* assign: NCC_3D + get_pos_idx of the same series against the centroids the
  zero-start extraction produced and against raw rows.

--time adds the reference's whole path at n=20,000, m=2709, k=8 (Dirichlet(2)
class sizes, noise 0.2, generator seed 1) with init_chose=1 (mt19937 seed 1) and
init_chose=0 (twice), iteration cap 20: timings to OUT_DIR/ref_gpu_times.json,
labels, the curand initial labels and a SHA-256 of the series to
OUT_DIR/ref_gpu_c2.npz, with two runs of the reference's extraction (class
labels, zero centroids) on the same FP64-z-normalised series.
"""
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "times-c_gb300"))

CASES = [
    # name, n, m, k, noise, iteration cap of the matching driver
    ("c1", 300, 128, 4, 0.2, 10),
    ("w100", 400, 100, 5, 0.2, 20),
    ("w129", 400, 129, 4, 0.2, 20),
    ("w300", 300, 300, 6, 0.2, 20),
    ("w512", 240, 512, 8, 0.3, 20),
]


def _ref_gpu():
    import importlib.util
    spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(ROOT, "oracle", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    path = b.build_ref_gpu()
    if path is None:
        raise SystemExit("reference headers are not staged under oracle/_ref/src")
    return path


def _run(exe, args, tmp, log):
    t = time.time()
    r = subprocess.run([exe] + [str(a) for a in args], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True, cwd=tmp)
    log.write("$ ref_gpu %s  (%.2f s, rc %d)\n" % (" ".join(str(a) for a in args[:7]), time.time() - t,
                                                   r.returncode))
    log.write(r.stdout[-4000:] + "\n")
    if r.returncode != 0:
        raise SystemExit("ref_gpu %s failed (rc %d); see the log" % (args[0], r.returncode))


def _znorm64(x):
    x = x.astype(np.float64)
    mu = x.mean(axis=1, keepdims=True)
    sd = x.std(axis=1, ddof=1, keepdims=True)
    sd[sd == 0] = 1.0
    return ((x - mu) / sd).astype(np.float32)


def _loop(exe, tmp, log, x, k, init_chose, cap, seed):
    n, m = x.shape
    xp, op = os.path.join(tmp, "x.f32"), os.path.join(tmp, "loop.out")
    x.tofile(xp)
    _run(exe, ["loop", n, m, k, init_chose, cap, seed, xp, op], tmp, log)
    raw = np.fromfile(op, np.uint8)
    labels = raw[:4 * n].view(np.int32).copy()
    info = raw[4 * n:4 * n + 12].view(np.int32).copy()
    ms = raw[4 * n + 12:4 * n + 20].view(np.float32).copy()
    return labels, info, ms


def main():
    if len(sys.argv) < 2 or sys.argv[1].startswith("-"):
        sys.exit("usage: make_ref_gpu_golden.py OUT_DIR [--time]")
    out_dir = sys.argv[1]
    os.makedirs(out_dir, exist_ok=True)
    exe = _ref_gpu()
    import timesc
    g = {}
    tmp = tempfile.mkdtemp()
    log = open(os.path.join(out_dir, "ref_gpu_golden.log"), "w")
    for name, n, m, k, noise, cap in CASES:
        x, truth = timesc.generate(n, m, k, noise=noise, seed=1000 + m)
        g[name + "__x"] = x
        g[name + "__truth"] = truth
        g[name + "__meta"] = np.array([n, m, k, cap], np.int32)
        ip = os.path.join(tmp, "init.i32")
        _run(exe, ["init", n, k, ip], tmp, log)
        g[name + "__init"] = np.fromfile(ip, np.int32)
        for init_chose, seed in ((0, 0), (1, 0), (1, 1)):
            lab, info, ms = _loop(exe, tmp, log, x, k, init_chose, cap, seed)
            key = "%s__loop_i%d_s%d" % (name, init_chose, seed)
            g[key + "__labels"] = lab
            g[key + "__info"] = info
            g[key + "__ms"] = ms
        xp, op = os.path.join(tmp, "x.f32"), os.path.join(tmp, "z.out")
        x.tofile(xp)
        _run(exe, ["znorm", n, m, xp, op], tmp, log)
        g[name + "__znorm"] = np.fromfile(op, np.float32).reshape(n, m)

        xz = _znorm64(x)
        g[name + "__xz"] = xz
        lab1 = (truth + 1).astype(np.int32)
        rng = np.random.default_rng(7 + m)
        rows = rng.choice(n, size=k, replace=False)
        unit = rng.standard_normal((k, m))
        unit /= np.linalg.norm(unit, axis=1, keepdims=True)
        starts = {"zero": np.zeros((k, m), np.float32), "raw": x[rows].copy(), "unit": unit.astype(np.float32)}
        g[name + "__raw_rows"] = rows.astype(np.int32)
        g[name + "__unit"] = starts["unit"]
        xzp, lp, cp, op = (os.path.join(tmp, f) for f in ("xz.f32", "l.i32", "c.f32", "e.out"))
        xz.tofile(xzp)
        lab1.tofile(lp)
        for sname, c0 in starts.items():
            for cal in (0, 1):
                c0.astype(np.float32).tofile(cp)
                _run(exe, ["extract", n, m, k, cal, xzp, lp, cp, op], tmp, log)
                raw = np.fromfile(op, np.uint8)
                key = "%s__extract_%s_cal%d" % (name, sname, cal)
                g[key + "__centroids"] = raw[:4 * k * m].view(np.float32).reshape(k, m).copy()
                g[key + "__counts"] = raw[4 * k * m:4 * k * m + 4 * k].view(np.int32).copy()
                g[key + "__sum_class"] = raw[4 * k * m + 4 * k:].view(np.int32).copy()
        for cname, C in (("ext", g[name + "__extract_zero_cal0__centroids"]), ("raw", starts["raw"])):
            C.astype(np.float32).tofile(cp)
            _run(exe, ["assign", n, m, k, xzp, cp, op], tmp, log)
            raw = np.fromfile(op, np.uint8)
            key = "%s__assign_%s" % (name, cname)
            g[key + "__labels"] = raw[:4 * n].view(np.int32).copy()
            g[key + "__dist"] = raw[4 * n:].view(np.float32).copy()
    dst = os.path.join(out_dir, "ref_gpu_golden.npz")
    np.savez_compressed(dst, **g)
    print("wrote", dst, len(g), "arrays")

    if "--time" in sys.argv:
        import hashlib
        n, m, k = 20000, 2709, 8
        x, truth = timesc.generate(n, m, k, noise=0.2, dirichlet=2.0, seed=1)
        sha = np.frombuffer(hashlib.sha256(x.tobytes()).digest(), np.uint8)
        rec = {}
        c2 = dict(x_sha256=sha)
        # init_chose=1 stops after its first assignment here (<= k/2 clusters left), so
        # its labels do not depend on an extraction; init_chose=0 runs twice (two
        # processes) because the reference's extraction at this length is not
        # reproducible (below)
        for init_chose, tag in ((1, "init1"), (0, "init0_run_a"), (0, "init0_run_b")):
            t = time.time()
            lab, info, ms = _loop(exe, tmp, log, x, k, init_chose, 20, 1)
            wall = time.time() - t
            rec["c2_" + tag] = dict(
                workload="n=20000 m=2709 k=8 init_chose=%d seed=1 cap 20" % init_chose, iter_num=int(info[0]),
                sum_class=int(info[1]), restarted=int(info[2]), norm_ms=float(ms[0]), loop_ms=float(ms[1]),
                process_wall_s=wall)
            c2["labels_" + tag] = lab
            c2["info_" + tag] = info
            c2["ms_" + tag] = ms
        ip = os.path.join(tmp, "init.i32")
        _run(exe, ["init", n, k, ip], tmp, log)
        c2["init"] = np.fromfile(ip, np.int32)
        # the reference's extraction at this length, twice on the same input: norm_vec
        # rescales the vector from three blocks that read it while others write it
        # (shapeExtract.cuh:287-323, m > 1024), so runs need not agree
        xz = _znorm64(x)
        xzp, lp, cp, op = (os.path.join(tmp, f) for f in ("xz.f32", "l.i32", "c.f32", "e.out"))
        xz.tofile(xzp)
        (truth + 1).astype(np.int32).tofile(lp)
        np.zeros((k, m), np.float32).tofile(cp)
        for run in (0, 1):
            _run(exe, ["extract", n, m, k, 0, xzp, lp, cp, op], tmp, log)
            c2["extract_zero_cal0_run%d" % run] = np.fromfile(op, np.float32, count=k * m).reshape(k, m)
        key = "c1__loop_i0_s0"
        rec["c1_init0"] = dict(iter_num=int(g[key + "__info"][0]), norm_ms=float(g[key + "__ms"][0]),
                               loop_ms=float(g[key + "__ms"][1]))
        with open(os.path.join(out_dir, "ref_gpu_times.json"), "w") as f:
            json.dump(rec, f, indent=1)
        np.savez_compressed(os.path.join(out_dir, "ref_gpu_c2.npz"), **c2)
        print(json.dumps(rec))
    log.close()


if __name__ == "__main__":
    main()
