"""k-Shape benchmark on GB300.

Workload (default): the precision workload, n = 1,000,000 series, m = 512,
k = 32, synthetic data (the prototype generator
of times-c_gb300/csrc/gen.cpp, noise 0.3), in the mixed-precision form (BF16
tensor-core correlation and Gram, FP32 accumulation); the plain FP32 form runs
beside it on the same series and the line reports both and how far apart their
results are.  A step is one whole k-Shape iteration in the reference's loop order
(extract shapes -> SBD assignment -> convergence read-back) over all series,
with the series resident in HBM.

  value      SBD pairs/s = n*k / (iteration time), whole iterations
  e2e        the same through tc_kshape_run with pinned host buffers
             (host->device copy of the series, z-norm, loop, labels and
             centroids back), pairs/s = n*k*iterations / wall time
  roofline   the dominant kernel (the fused SBD assignment), CUDA events on
             the launching stream; algorithmic work per launch: 2*n*k*F*m
             flops for the tensor-core correlation (m products per lag, F
             lags), the FFT flop count of fft_flops() for the FP32 kernel
  cpu_baseline  the FP64 oracle (a restatement, "port") on the host cores,
             one iteration on a bounded sample of the same workload

`--impl reference` times the reference's CPU implementation of the path.  Its
own CPU code (Code/test/test_timesC.py) is not present on GPU hosts, so the
FP64 port of it (oracle/) runs instead, on all host threads.

Multi-GPU: the path is run as independent replicas (one per rank).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "times-c_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

WORKLOADS = {
    # name: (n, m, k, noise, dirichlet, description)
    "c3": (1_000_000, 512, 32, 0.3, 0.0, "precision form: n=1e6 m=512 k=32, FP32 series, noise 0.3"),
    "c2": (20_000, 2709, 8, 0.2, 2.0, "at scale: n=2e4 m=2709 k=8, Dirichlet(2) classes"),
    "c1": (300, 128, 4, 0.2, 0.0, "CPU-runnable: n=300 m=128 k=4"),
    # profiling case: the precision form with a tenth of the series (still larger than L2)
    "c3s": (100_000, 512, 32, 0.3, 0.0, "profiling case: n=1e5 m=512 k=32, noise 0.3"),
}
PREC = {"fp32": 0, "bf16": 1, "tf32": 2}
MODES = {"compat": 0, "canonical": 1}


def fft_flops(n, k, F):
    """Algorithmic FP32 flops of the FFT-form assignment (per launch)."""
    L = int(np.log2(F))
    return n * (2.5 * F * L) + n * k * (6 * (F // 2 + 1) + 2.5 * F * L + F)


def assign_bytes(n, m, k):
    """Irreducible HBM bytes of one assignment: series in, centroids in, label/dist/shift out."""
    return 4 * n * m + 4 * k * m + 12 * n


def tc_flops(n, m, k, F):
    """Algorithmic flops of the tensor-core correlation: m products per lag, F lags."""
    return 2.0 * n * k * F * m


def tc_supported(m, F, prec):
    """Shapes the tensor-core correlation takes (others run the FP32 FFT kernel)."""
    return prec == PREC["bf16"] and m <= 512 and 128 <= F <= 1024


def screened(m, F, k, prec):
    """The FP32 form's assignment with the BF16 tensor-core screening pass (exact)."""
    return (prec == PREC["fp32"] and k >= 2 and tc_supported(m, F, PREC["bf16"])
            and not os.environ.get("TIMESC_NO_SCREEN"))


def load_peaks():
    """HBM GB/s and the burst bf16 TFLOP/s (the assignment kernel runs for a few ms
    inside a step of about a dozen ms, well short of the power-capped loop of the
    sustained figure)."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


def bf16_nominal_tflops(sm_mhz):
    """Dense BF16 tensor rate at the given SM clock: 8192 flop/clk per SM, 152 SMs."""
    return 152 * 8192 * sm_mhz * 1e6 / 1e12


def profiled_traffic(workload, mode, prec):
    """dram bytes per launch of the assignment kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "assign_%s_%s_%s.txt" % (prec, workload, mode))
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1])
            except ValueError:
                return None
    return None


class Clocks:
    """nvidia-smi sampling (every 20 ms, timestamped).  Start it before the warm-up
    and bracket the timed region with begin()/end(): only samples inside that window
    count (all samples when begin() was not called)."""
    Q = ("timestamp,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.t0 = self.t1 = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "20"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def begin(self):
        import datetime
        self.t0 = datetime.datetime.now()

    def end(self):
        import datetime
        self.t1 = datetime.datetime.now()

    def stop(self):
        import datetime
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        self.f.close()
        with open(self.f.name) as fh:
            lines = fh.readlines()
        for line in lines:
            parts = [t.strip() for t in line.split(",")]
            if len(parts) != 8:
                continue
            try:
                ts = datetime.datetime.strptime(parts[0], "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                continue
            rows.append((ts, parts[1:]))
        os.unlink(self.f.name)
        window = "all samples"
        if self.t0 is not None and self.t1 is not None:
            lo, hi = self.t0 - datetime.timedelta(milliseconds=25), self.t1 + datetime.timedelta(milliseconds=25)
            inside = [r for r in rows if lo <= r[0] <= hi]
            if inside:
                rows, window = inside, "timed region (%.0f ms)" % ((self.t1 - self.t0).total_seconds() * 1e3)
            else:
                window = "no sample inside the timed region: all samples (warm-up included)"
        rows = [r[1] for r in rows]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in rows for j in range(4) if r[3 + j].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows), "window": window}


def cufft_assign_ms(x, C, F, chunk=32768, reps=3):
    """Library baseline (not the product): the reference's materialising NCC_3D +
    get_pos_idx (ncc.cuh:469-517, kshape.cuh:35-96) in plain FP32 on cuFFT via
    torch.fft, in chunks of series so the n*k*F spectra fit in memory.
    Returns (ms per full assignment, labels)."""
    import torch
    n, m = x.shape
    k = C.shape[0]
    L = 2 * m - 1
    slots = (torch.arange(L, device=x.device) - (m - 1)) % F
    cn = torch.linalg.norm(C, dim=1)
    Cs = torch.fft.rfft(C, n=F)
    labels = torch.empty(n, dtype=torch.int64, device=x.device)

    def run():
        for i0 in range(0, n, chunk):
            xs = x[i0:i0 + chunk]
            xn = torch.linalg.norm(xs, dim=1)
            P = torch.fft.rfft(xs, n=F)[:, None, :] * torch.conj(Cs)[None, :, :]
            r = torch.fft.irfft(P, n=F)[:, :, slots]
            den = xn[:, None] * cn[None, :]
            den = torch.where(den == 0, torch.full_like(den, 1e10), den)
            d = (1.0 - r / den[:, :, None]).amin(dim=2)
            labels[i0:i0 + chunk] = d.argmin(dim=1)

    run()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        run()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps, labels


def cpu_iteration(O, X, C, labels, mode, F, ns):
    m = X.shape[1]
    om = O.MODE_COMPAT if mode == 0 else O.MODE_CANONICAL
    t0 = time.perf_counter()
    Cs, _, _ = O.extract(X[:ns], labels[:ns], C, om)
    O.assign(X[:ns], Cs, F, clamp2=(mode == 0 and 2 * m - 1 < 512))
    return time.perf_counter() - t0


def arm_config(args, wl, F, world):
    """The `config` both arms print (the driver compares them)."""
    n, m, k, noise, dirich, desc = wl
    return {"workload": desc, "mode": args.mode, "precision": args.precision, "fft_length": F,
            "parallelism": "replicas" if world > 1 else "single GPU",
            "l2": "inputs larger than L2 (%.1f GB of series)" % (4 * n * m / 1e9)}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def max_over_ranks(value, dist):
    """The largest of every rank's value (the slowest replica's time), on all ranks:
    a GPU tensor under NCCL, a host tensor under gloo."""
    import torch
    if dist is None:
        return value
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.item()


def run_reference(args, wl):
    """The reference's CPU implementation of the path, rank 0 only.  Its own CPU code
    (Code/test/test_timesC.py) does not reach GPU hosts (and at this size would need
    ~0.5 TB per temporary), so the FP64 port of the reference's GPU path (oracle/)
    runs on all host threads.  The series come from the oracle library's copy of
    the generator: nothing of the engine is loaded.  Warm-up steps run on a tenth
    of the series; every timed step is one whole iteration (extraction + SBD
    assignment) over all n series."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_NUM_THREADS", str(host_threads()))
    from oracle import oracle as O
    n, m, k, noise, dirich, desc = wl
    data, _ = O.generate(n, m, k, noise=noise, dirichlet=dirich, seed=0)
    X = O.znorm(data.astype(np.float64))
    del data
    rng = np.random.default_rng(0)
    labels = rng.integers(0, k, size=n).astype(np.int32)
    C = X[rng.choice(n, k, replace=False)].copy()
    C /= np.linalg.norm(C, axis=1, keepdims=True)
    md = MODES[args.mode]
    F = O.fft_size(m, md)
    nw = max(k, n // 10)
    for _ in range(args.warmup):
        cpu_iteration(O, X, C, labels, md, F, nw)
    times = [cpu_iteration(O, X, C, labels, md, F, n) for _ in range(args.steps)]
    t = statistics.mean(times)
    value = n * k / t
    line = {"impl": "reference", "metric": "SBD pairs/s (whole k-Shape iterations)", "value": value,
            "unit": "pairs/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (prototype generator)",
            "config": arm_config(args, wl, F, int(os.environ.get("WORLD_SIZE", "1"))),
            "cpu_baseline": {"value": value, "unit": "pairs/s", "cores": int(os.environ["OMP_NUM_THREADS"]),
                             "kind": "port",
                             "sample": "every timed step one whole extract + assign iteration of the FP64 port "
                                       "over all %d series and %d centroids (no extrapolation); warm-up steps "
                                       "over %d series" % (n, k, nw),
                             "step_s": times},
            "e2e": {"value": value, "unit": "pairs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def ari(a, b):
    """Adjusted Rand index of two labelings (contingency table in numpy)."""
    a = np.asarray(a, np.int64)
    b = np.asarray(b, np.int64)
    nb = int(b.max()) + 1
    cont = np.bincount(a * nb + b, minlength=(int(a.max()) + 1) * nb).reshape(-1, nb).astype(np.float64)
    c2 = lambda v: v * (v - 1) / 2.0
    s_ij, s_a, s_b = c2(cont).sum(), c2(cont.sum(1)).sum(), c2(cont.sum(0)).sum()
    exp = s_a * s_b / c2(float(len(a)))
    mx = 0.5 * (s_a + s_b)
    return 1.0 if mx == exp else float((s_ij - exp) / (mx - exp))


def bf16_assign_ms(ctx, x, C, k, mode, stream, reps=3):
    """CUDA-event time of the full BF16 tensor-core assignment on these series (every
    pair evaluated: distance bounds off; outputs to scratch)."""
    import torch
    n = x.shape[0]
    lab = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    os.environ["TIMESC_NO_BOUNDS"] = "1"
    try:
        ctx.sbd_assign(x, C, mode=mode, precision=PREC["bf16"], labels=lab, dist=dist, stream=stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            ctx.sbd_assign(x, C, mode=mode, precision=PREC["bf16"], labels=lab, dist=dist, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
    finally:
        del os.environ["TIMESC_NO_BOUNDS"]
    return e0.elapsed_time(e1) / reps


def dense_iterations(ctx, x, labels, C, n, k, mode, prec, stream, steps):
    """The same iterations from the same state with the distance bounds off (every pair
    evaluated): ms per whole iteration and per assignment, for comparison."""
    import torch
    lab = labels.clone()
    old = labels.clone()
    Cw = C.clone()
    dist = torch.empty((n,), dtype=torch.float32, device="cuda")
    ch = torch.zeros(1, dtype=torch.int32, device="cuda")
    e0, e1, a0, a1 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
    os.environ["TIMESC_NO_BOUNDS"] = "1"
    try:
        a_tot = 0.0
        e0.record(stream)
        for _ in range(steps):
            ctx.extract_shapes(x, lab, Cw, mode=mode, precision=prec)
            ch.zero_()
            a0.record(stream)
            ctx.sbd_assign(x, Cw, mode=mode, precision=prec, labels=lab, dist=dist, old_labels=old, changed=ch)
            a1.record(stream)
            ch.item()
            a_tot += a0.elapsed_time(a1)
        e1.record(stream)
        torch.cuda.synchronize()
    finally:
        del os.environ["TIMESC_NO_BOUNDS"]
    return e0.elapsed_time(e1) / steps, a_tot / steps


def plain_fp32_compare(ctx, x, labels, C, n, m, k, mode, prec, stream, ms_mixed, a_ms_mixed, steps=2):
    """Times the plain FP32 form on the same series and state (whole iterations and the
    assignment alone), and measures how far the mixed form is from it over all n: one
    extraction and one assignment from the same labels in both forms (centroid error,
    distance error, label agreement and ARI)."""
    import torch
    lab0 = labels.clone()
    C32 = C.clone()  # the extraction aligns members to the centroids it is given
    C16 = C.clone()
    ctx.extract_shapes(x, lab0, C32, mode=mode, precision=PREC["fp32"])
    ctx.extract_shapes(x, lab0, C16, mode=mode, precision=prec)
    l32 = torch.empty_like(labels)
    l16 = torch.empty_like(labels)
    d32 = torch.empty((n,), dtype=torch.float32, device="cuda")
    d16 = torch.empty_like(d32)
    ctx.sbd_assign(x, C32, mode=mode, precision=PREC["fp32"], labels=l32, dist=d32)
    ctx.sbd_assign(x, C32, mode=mode, precision=prec, labels=l16, dist=d16)
    torch.cuda.synchronize()
    L32, L16 = l32.cpu().numpy(), l16.cpu().numpy()
    rep = {"centroid_max_abs_err": float((C16 - C32).abs().max().item()),
           "sbd_max_abs_err": float((d16 - d32).abs().max().item()),
           "label_agreement": float((L32 == L16).mean()), "ari": ari(L32, L16),
           "what": "mixed vs plain FP32 over all n: extraction from the same labels, assignment against "
                   "the same FP32 centroids (the FP32 form is parity-tested against the FP64 oracle)"}
    # timing: whole iterations and the assignment in FP32, screened (the product's FP32
    # form) and unscreened (every centroid through the FFT kernel: the plain FP32 form)
    def time_fp32():
        e0, e1, a0, a1 = (torch.cuda.Event(enable_timing=True) for _ in range(4))
        lab = lab0.clone()
        old = lab0.clone()
        Cw = C32.clone()
        ch = torch.zeros(1, dtype=torch.int32, device="cuda")
        ds = torch.zeros(1, dtype=torch.float64, device="cuda")
        dist = torch.empty_like(d32)
        for _ in range(2):  # warm
            ctx.extract_shapes(x, lab, Cw, mode=mode, precision=PREC["fp32"])
            ctx.sbd_assign(x, Cw, mode=mode, precision=PREC["fp32"], labels=lab, dist=dist)
        torch.cuda.synchronize()
        a_tot = 0.0
        e0.record(stream)
        for _ in range(steps):
            ctx.extract_shapes(x, lab, Cw, mode=mode, precision=PREC["fp32"])
            ch.zero_()
            ds.zero_()
            a0.record(stream)
            ctx.sbd_assign(x, Cw, mode=mode, precision=PREC["fp32"], labels=lab, dist=dist, old_labels=old,
                           changed=ch, dist_sum=ds)
            a1.record(stream)
            ch.item()
            a_tot += a0.elapsed_time(a1)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, a_tot / steps

    ms32, a32 = time_fp32()
    os.environ["TIMESC_NO_SCREEN"] = "1"
    try:
        ms_u, a_u = time_fp32()
    finally:
        del os.environ["TIMESC_NO_SCREEN"]
    rep.update({"ms_per_iteration": ms32, "assign_ms": a32, "assign_pairs_per_s": n * k / (a32 / 1e3),
                "pairs_per_s_whole_iterations": n * k / (ms32 / 1e3),
                "mixed_vs_plain_fp32_assign_speedup": a32 / a_ms_mixed,
                "mixed_vs_plain_fp32_iteration_speedup": ms32 / ms_mixed,
                "unscreened": {"ms_per_iteration": ms_u, "assign_ms": a_u,
                               "pairs_per_s_whole_iterations": n * k / (ms_u / 1e3),
                               "assign_pairs_per_s": n * k / (a_u / 1e3),
                               "mixed_speedup_iteration": ms_u / ms_mixed,
                               "mixed_speedup_assign": a_u / a_ms_mixed,
                               "what": "the plain FP32 form: every centroid through the FP32 FFT kernel "
                                       "(TIMESC_NO_SCREEN=1), the denominator of the mixed form's speed-up"}})
    return rep


def oracle_iteration_report(ctx, data, x, labels, C, n, m, k, mode, F, prec):
    """One whole iteration of the FP64 oracle over all n series from the timed run's
    final state (labels, centroids): its time is the CPU baseline (all host threads,
    no extrapolation), its outputs the reference for the GPU forms' errors.  Each
    GPU form runs the same iteration from the same state: its centroid error, its
    SBD error (assignment against the oracle's centroids, so that only the
    assignment's arithmetic differs) and the ARI of its own iteration's labels."""
    import torch
    from oracle import oracle as O
    X = O.znorm(data.astype(np.float64))
    lab_h = labels.cpu().numpy().astype(np.int32)
    C_h = C.cpu().numpy().astype(np.float64)
    om = O.MODE_COMPAT if mode == 0 else O.MODE_CANONICAL
    clamp2 = mode == 0 and 2 * m - 1 < 512
    t0 = time.perf_counter()
    C_o, _, _ = O.extract(X, lab_h, C_h, om)
    l_o, d_o, _, margin = O.assign(X, C_o, F, clamp2=clamp2)
    t = time.perf_counter() - t0
    del X
    base = {"value": n * k / t, "unit": "pairs/s", "cores": host_threads(), "kind": "port",
            "sample": "one whole extract + assign iteration of the FP64 oracle over all %d series and %d centroids "
                      "(%.1f s, no extrapolation), from the timed run's final state" % (n, k, t)}
    rep = {"what": "one iteration (extraction from the timed run's final labels and centroids, then assignment) "
                   "of each GPU form against the FP64 oracle over all %d series" % n,
           "oracle_min_margin": float(margin.min()) if k > 1 else None}
    c_o = torch.from_numpy(C_o.astype(np.float32)).cuda()
    forms = [("fp32", PREC["fp32"])] + ([(args_prec_name(prec), prec)] if prec != PREC["fp32"] else [])
    for name, p in forms:
        Cg = C.clone()
        ctx.extract_shapes(x, labels.clone(), Cg, mode=mode, precision=p)
        lg = torch.empty_like(labels)
        dg = torch.empty((n,), dtype=torch.float32, device="cuda")
        ctx.sbd_assign(x, Cg, mode=mode, precision=p, labels=lg, dist=dg)
        ls = torch.empty_like(labels)
        ds = torch.empty_like(dg)
        ctx.sbd_assign(x, c_o, mode=mode, precision=p, labels=ls, dist=ds)
        torch.cuda.synchronize()
        L = lg.cpu().numpy()
        rep[name] = {"centroid_max_abs_err": float(np.abs(Cg.cpu().numpy() - C_o).max()),
                     "sbd_max_abs_err": float(np.abs(ds.cpu().numpy() - d_o).max()),
                     "ari": ari(L, l_o), "label_agreement": float((L == l_o).mean()),
                     "labels_vs_oracle_on_oracle_centroids": float((ls.cpu().numpy() == l_o).mean())}
    return base, rep


def args_prec_name(prec):
    return {v: k for k, v in PREC.items()}[prec]


# ---------------------------------------------------------------- many jobs (batch, serving)
def c4_sizes(count, seed=2024):
    """Job sizes of the batched form: n log-uniform in [64, 5e4], m log-uniform in
    [32, 4096], k uniform in [2, 64]; job i uses generator seed i."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(64), np.log(5e4), count)).astype(np.int64)
    m = np.exp(rng.uniform(np.log(32), np.log(4096), count)).astype(np.int64)
    k = rng.integers(2, 65, count)
    return [(int(a), int(b), int(c)) for a, b, c in zip(n, m, k)]


def make_specs(timesc, sizes, precision, max_iter, seed0=0, noise=0.2):
    """JobSpecs with generator data, generated on all host threads."""
    from concurrent.futures import ThreadPoolExecutor

    def one(i):
        n, m, k = sizes[i]
        data, _ = timesc.generate(n, m, k, noise=noise, seed=seed0 + i)
        return timesc.JobSpec(data, k, mode=0, precision=precision, seed=seed0 + i, max_iter=max_iter)

    with ThreadPoolExecutor(max_workers=host_threads()) as ex:
        return list(ex.map(one, range(len(sizes))))


def run_batched(args):
    """Batched form: many independent jobs in one pool, all to convergence (or the
    iteration cap); a step is the whole batch."""
    import timesc
    prec = PREC[args.precision]
    sizes = c4_sizes(args.jobs)
    specs = make_specs(timesc, sizes, prec, args.max_iter)
    warm = make_specs(timesc, sorted(sizes)[: min(16, len(sizes))], prec, 2, seed0=10_000)
    pool = timesc.Pool(device=0, workers=args.workers)
    clk = Clocks(0)
    for _ in range(args.warmup):
        pool.run_batch(warm)
    clk.begin()
    l0 = timesc.lib().tc_launch_count()
    walls = []
    bad = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        st = pool.run_batch(specs)
        walls.append(time.perf_counter() - t0)
        bad += [i for i, v in enumerate(st) if v != timesc.OK]
    clk.end()
    launches = timesc.lib().tc_launch_count() - l0
    clocks = clk.stop()
    pool.close()  # every job has ended before any failure is reported
    assert not bad, "failed jobs: %s" % [sizes[i] for i in sorted(set(bad))]
    wall = statistics.mean(walls)
    iters = [s.res.iterations for s in specs]
    pairs = sum(n * k * it for (n, m, k), it in zip(sizes, iters))
    out = {"metric": "SBD pairs/s (batched jobs, whole k-Shape loops)", "value": pairs / wall, "unit": "pairs/s",
           "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": wall * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if prec == 0 else args.precision, "data": "synthetic (prototype generator), seeds 0..%d"
           % (len(sizes) - 1),
           "config": {"workload": "batched form: %d jobs, n log-U[64,5e4], m log-U[32,4096], k U[2,64]"
                      % len(sizes), "workers": args.workers, "max_iter": args.max_iter, "mode": "compat",
                      "precision": args.precision, "graphs": "per-job iteration stages replayed"},
           "jobs_per_s": len(sizes) / wall, "iterations_total": int(sum(iters)),
           "gpu_launches": int(launches / max(args.steps, 1)), "clocks": clocks,
           "e2e": {"value": pairs / wall, "unit": "pairs/s",
                   "h2d_bytes_per_step": int(sum(4 * n * m for n, m, k in sizes)),
                   "d2h_bytes_per_step": int(sum(4 * n + 4 * k * m for n, m, k in sizes)),
                   "call": "tc_pool_run_batch (host buffers in, labels/centroids out)"}}
    return out


def run_serving(args):
    """Serving form: Poisson arrivals at 80% of the measured capacity; 95% of the
    requests are batched-form jobs, 5% n=2e5 m=1024 k=16; HBM admission budget
    150 GB; latency = submission to completion."""
    import threading
    import timesc
    prec = PREC[args.precision]
    rng = np.random.default_rng(7)
    small = c4_sizes(48, seed=99)
    lib_small = make_specs(timesc, small, prec, args.max_iter, seed0=1000)
    big_data = [timesc.generate(200_000, 1024, 16, noise=0.2, seed=2000 + i)[0] for i in range(2)]
    pick = ["L%d" % (i % 2) if rng.random() < 0.05 else "S%d" % rng.integers(0, len(small))
            for i in range(args.jobs)]

    def spec_for(key):
        if key[0] == "L":
            return timesc.JobSpec(big_data[int(key[1:])], 16, mode=0, precision=prec, seed=7, max_iter=args.max_iter)
        src = lib_small[int(key[1:])]
        return timesc.JobSpec(src.data, src.k, mode=0, precision=prec, seed=src.job.seed, max_iter=args.max_iter)

    budget = 150 * 10**9
    pool = timesc.Pool(device=0, workers=args.workers, hbm_budget_bytes=budget)
    # warm-up, then capacity: a saturated batch with the request mix
    for _ in range(max(1, args.warmup - 2)):
        pool.run_batch([spec_for(k) for k in pick[:8]])
    # saturated, in arrival order (first in, first out, as the served requests are taken),
    # on the first quarter of the request list (at least 64) so that its share of large
    # requests is close to the whole run's
    cap_keys = pick[: min(max(64, len(pick) // 4), len(pick))]
    cap_specs = [spec_for(k) for k in cap_keys]
    t0 = time.perf_counter()
    cap_tickets = [pool.submit(sp) for sp in cap_specs]
    for t in cap_tickets:
        pool.wait(t)
    capacity = len(cap_keys) / (time.perf_counter() - t0)
    rate = 0.8 * capacity
    gaps = rng.exponential(1.0 / rate, len(pick))
    specs = [spec_for(k) for k in pick]
    tickets = [None] * len(specs)
    held = []
    clk = Clocks(0)
    time.sleep(0.3)  # nvidia-smi up before the first request
    clk.begin()
    start = time.perf_counter()

    def producer():
        t_next = start
        for i, sp in enumerate(specs):
            t_next += gaps[i]
            d = t_next - time.perf_counter()
            if d > 0:
                time.sleep(d)
            tickets[i] = pool.submit(sp)
            held.append(pool.stats()["held_bytes"])

    th = threading.Thread(target=producer)
    th.start()
    th.join()
    res = [pool.wait(t) for t in tickets]
    end = time.perf_counter()
    clk.end()
    clocks = clk.stop()
    pool.close()  # every job has ended before any failure is reported
    assert all(r[0] == timesc.OK for r in res), [r[0] for r in res]
    lat = np.array([r[2] for r in res])
    que = np.array([r[1] for r in res])
    pairs = sum(sp.job.n * sp.job.k * sp.res.iterations for sp in specs)
    out = {"metric": "served jobs/s at 80% load (Poisson arrivals), request latency p50/p99",
           "value": len(specs) / (end - start), "unit": "jobs/s", "n_gpus": 1, "steps": 1, "warmup": args.warmup,
           "ms_per_step": (end - start) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32" if prec == 0 else args.precision + " mixed",
           "data": "synthetic (prototype generator)",
           "config": {"workload": "serving form: %d requests, 95%% batched-form sizes, 5%% n=2e5 m=1024 k=16"
                      % len(specs), "workers": args.workers, "hbm_budget_bytes": budget,
                      "arrival_rate_per_s": rate, "measured_capacity_jobs_per_s": capacity,
                      "max_iter": args.max_iter, "precision": args.precision},
           "latency_s": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                         "mean": float(lat.mean()), "max": float(lat.max())},
           "queue_s": {"p50": float(np.percentile(que, 50)), "p99": float(np.percentile(que, 99))},
           "large_requests": int(sum(k[0] == "L" for k in pick)), "max_held_bytes": int(max(held) if held else 0),
           "pairs_per_s": pairs / (end - start), "clocks": clocks,
           "e2e": {"value": len(specs) / (end - start), "unit": "jobs/s",
                   "h2d_bytes_per_step": int(sum(4 * sp.job.n * sp.job.m for sp in specs)),
                   "d2h_bytes_per_step": int(sum(4 * sp.job.n + 4 * sp.job.k * sp.job.m for sp in specs)),
                   "call": "tc_pool_submit / tc_pool_wait"}}
    return out


def many_jobs_samples(args):
    """The batched and serving forms on bounded samples (128 jobs each), recorded in the
    default line beside the single-job figures: their own lines come from
    --workload c4 / c5 (512 jobs).  A failure here is recorded, not raised."""
    import copy
    res = {}
    for name, fn, prec in (("batched", run_batched, "fp32"), ("serving", run_serving, "bf16")):
        a = copy.copy(args)
        a.jobs, a.workers, a.max_iter, a.precision, a.steps = 128, 8, 10, prec, 1
        try:
            line = fn(a)
            keep = ("metric", "value", "unit", "ms_per_step", "config", "latency_s", "queue_s", "pairs_per_s",
                    "jobs_per_s", "e2e", "clocks")
            res[name] = {key: line[key] for key in keep if key in line}
        except Exception as e:  # noqa: BLE001 - recorded in the line
            res[name] = {"error": "%s: %s" % (type(e).__name__, e)}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c3", choices=sorted(WORKLOADS) + ["c4", "c5"])
    ap.add_argument("--jobs", type=int, default=512, help="c4/c5: number of jobs")
    ap.add_argument("--workers", type=int, default=8, help="c4/c5: jobs in flight")
    ap.add_argument("--max-iter", type=int, default=10, help="c4/c5: k-Shape iteration cap per job")
    ap.add_argument("--precision", default=None, choices=sorted(PREC),
                    help="default per workload: c3 and c5 the mixed-precision form (bf16; for c3 the plain FP32 "
                         "form is timed beside it), c1, c2 and c4 fp32")
    ap.add_argument("--mode", default="compat", choices=sorted(MODES))
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-cufft", action="store_true")
    ap.add_argument("--no-many-jobs", action="store_true",
                    help="leave out the 128-job samples of the batched and serving forms (c3 line)")
    ap.add_argument("--no-compare", action="store_true",
                    help="leave out the plain FP32 form and dense comparisons (the timed loop is unchanged)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.precision is None:
        args.precision = "bf16" if args.workload in ("c3", "c3s", "c5") else "fp32"
    if args.workload == "c4":
        print(json.dumps(run_batched(args)), flush=True)
        return
    if args.workload == "c5":
        print(json.dumps(run_serving(args)), flush=True)
        return
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl)

    import torch
    import timesc
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    n, m, k, noise, dirich, desc = wl
    mode, prec = MODES[args.mode], PREC[args.precision]
    F = timesc.fft_size(m, mode)
    data, truth = timesc.generate(n, m, k, noise=noise, dirichlet=dirich, seed=rank)
    ctx = timesc.Context(local)
    stream = torch.cuda.current_stream()
    x = torch.from_numpy(data).cuda()
    ctx.znorm(x, ddof=1)
    if tc_supported(m, F, prec) or screened(m, F, k, prec):
        ctx.prepare_series(x)  # the series are fixed for the run: BF16 copy kept resident
    labels = torch.zeros(n, dtype=torch.int32, device="cuda")
    ctx.init_labels(labels, k)
    old = labels.clone()
    C = torch.zeros((k, m), dtype=torch.float32, device="cuda")
    dist_b = torch.zeros(n, dtype=torch.float32, device="cuda")
    changed = torch.zeros(1, dtype=torch.int32, device="cuda")
    dsum = torch.zeros(1, dtype=torch.float64, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]

    def iteration(rec=None):
        ctx.extract_shapes(x, labels, C, mode=mode, precision=prec)
        changed.zero_()
        dsum.zero_()
        if rec:
            rec[0].record(stream)
        ctx.sbd_assign(x, C, mode=mode, precision=prec, labels=labels, dist=dist_b,
                       old_labels=old, changed=changed, dist_sum=dsum)
        if rec:
            rec[1].record(stream)
        return changed.item(), dsum.item()  # the reference reads its convergence flag back every iteration

    clk = Clocks(local)  # sampling from the warm-up on; the timed window is marked below
    for _ in range(args.warmup):
        iteration()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    snap = (labels.clone(), C.clone())  # the state the timed iterations start from
    clk.begin()
    st0 = ctx.assign_stats()
    l0 = timesc.lib().tc_launch_count()
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    per_step = []  # host counters after each step (no device work)
    t_start.record(stream)
    for s in range(args.steps):
        iteration(ev[s])
        per_step.append(ctx.assign_stats())
    t_end.record(stream)
    torch.cuda.synchronize()
    clk.end()
    launches = timesc.lib().tc_launch_count() - l0
    st1 = ctx.assign_stats()
    clocks = clk.stop()
    ms = t_start.elapsed_time(t_end)
    assign_ms = [a.elapsed_time(b) for a, b in ev]
    if dist:
        ms = max_over_ranks(ms, dist)
        dist.barrier()
    ms_step = ms / args.steps
    value = world * n * k / (ms_step / 1e3)
    a_ms = statistics.mean(assign_ms)

    out = None
    if rank == 0:
        hbm, bf16, peak_kind = load_peaks()
        flops = fft_flops(n, k, F)
        nbytes = assign_bytes(n, m, k)
        achieved_gbs = nbytes / (a_ms / 1e3) / 1e9
        sm_mhz = clocks.get("sm_mhz") or 2070.0
        fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
        full_full, full_bnd, pairs_bnd = (b - a for a, b in zip(st0, st1))
        if tc_supported(m, F, prec):
            # the kernel at full work (every pair), timed on its own; the timed iterations
            # mostly run the bounded pass (see "bounds")
            t_full = bf16_assign_ms(ctx, x, C, k, mode, stream)
            tflops = tc_flops(n, m, k, F) / (t_full / 1e3) / 1e12
            mp = (m + 63) // 64 * 64
            tc_bytes = 2 * n * mp + 8 * n + 2 * k * (F // 8) * (mp + 56)  # BF16 series, labels+dist, buffers
            nominal = bf16_nominal_tflops(sm_mhz)
            roof = {"kernel": "k_assign_tc (fused SBD assignment, tcgen05 BF16, FP32 accumulation)",
                    "bound": "tensor", "achieved": tflops, "peak": bf16, "unit": "TFLOP/s",
                    "frac": tflops / bf16, "traffic": profiled_traffic(args.workload, args.mode, args.precision),
                    "peak_source": peak_kind + " (cuBLAS bf16 burst); the kernel can exceed it: it holds "
                                   "a higher clock than the power-capped cuBLAS run",
                    "nominal_at_median_clock": nominal, "frac_of_nominal": tflops / nominal,
                    "algorithmic_flops_per_launch": tc_flops(n, m, k, F), "launch_ms": t_full,
                    "hbm": {"achieved": tc_bytes / (t_full / 1e3) / 1e9, "peak": hbm,
                            "algorithmic_bytes_per_launch": tc_bytes},
                    "note": "a full assignment (every pair, distance bounds off) timed on its own: launch_ms "
                            "covers the shifted centroid buffers and the correlation kernel; the BF16 copy of "
                            "the (fixed) series is made once per run (tc_prepare_series)"}
        elif screened(m, F, k, prec):
            # the screening pass alone: the same tensor-core kernel as the BF16 assignment
            tc_ms = bf16_assign_ms(ctx, x, C, k, mode, stream)
            tflops = tc_flops(n, m, k, F) / (tc_ms / 1e3) / 1e12
            nominal = bf16_nominal_tflops(sm_mhz)
            roof = {"kernel": "k_assign_tc screening pass of the FP32 assignment (tcgen05 BF16, FP32 "
                              "accumulation)",
                    "bound": "tensor", "achieved": tflops, "peak": bf16, "unit": "TFLOP/s", "frac": tflops / bf16,
                    "traffic": profiled_traffic(args.workload, args.mode, "bf16"),
                    "peak_source": peak_kind + " (cuBLAS bf16 burst)",
                    "nominal_at_median_clock": nominal, "frac_of_nominal": tflops / nominal,
                    "algorithmic_flops_per_launch": tc_flops(n, m, k, F), "launch_ms": tc_ms,
                    "screened_assignment": {"ms": a_ms, "tensor_pass_ms": tc_ms,
                                            "fft_candidate_pass_ms": a_ms - tc_ms},
                    "note": "FP32 assignment = BF16 tensor-core pass keeping every centroid whose FP32 "
                            "distance can be the minimum (rigorous BF16 error bound) + the FP32 FFT kernel on "
                            "those; labels and distances equal the unscreened FP32 kernel's bit for bit. "
                            "launch_ms times the tensor pass alone (a BF16 assignment on the same data)"}
        else:
            roof = None
        roof = roof or {"kernel": "k_assign_fft (fused SBD assignment, SIMT FP32)", "bound": "hbm",
                "achieved": achieved_gbs, "peak": hbm, "unit": "GB/s", "frac": achieved_gbs / hbm,
                "traffic": profiled_traffic(args.workload, args.mode, args.precision),
                "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": nbytes, "launch_ms": a_ms,
                "fp32_simt": {"achieved_tflops": flops / (a_ms / 1e3) / 1e12, "peak_tflops_at_median_clock":
                              fp32_peak, "frac": flops / (a_ms / 1e3) / 1e12 / fp32_peak,
                              "algorithmic_flops_per_launch": flops},
                "note": "the FFT-form assignment is FP32-compute bound (about 475 flop/B); the HBM fraction is "
                        "reported as the schema asks and the FP32 fraction beside it"}
        out = {"metric": "SBD pairs/s (whole k-Shape iterations)", "value": value, "unit": "pairs/s",
               "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
               "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
               "dtype": ("bf16 operands, f32 accumulation" if tc_supported(m, F, prec) else
                         "f32 (exact BF16 screening pass)" if screened(m, F, k, prec) else "f32"),
               "data": "synthetic (prototype generator: sinusoids + bump, shifted/scaled/offset, noise)",
               "config": arm_config(args, wl, F, world),
               "kshape_iters_per_s": 1e3 / ms_step,
               "assign_pairs_per_s": n * k / (a_ms / 1e3),
               "assign_ms": a_ms,
               "roofline": roof, "gpu_launches": int(launches), "clocks": clocks}
        if full_bnd:
            out["bounds"] = {
                "full_passes": int(full_full), "bounded_passes": int(full_bnd),
                "evaluated_fraction_in_bounded_passes": pairs_bnd / (full_bnd * n * k),
                "evaluated_fraction_all_timed": (pairs_bnd + full_full * n * k) / (args.steps * n * k),
                "passes": [("full" if b[0] > a[0] else "bounded %.3f" % ((b[2] - a[2]) / (n * k)))
                           for a, b in zip([st0] + per_step[:-1], per_step)],
                "what": "the assignment keeps lower bounds on every (series, centroid) distance across "
                        "iterations and evaluates only the pairs they do not rule out (labels and distances "
                        "equal to evaluating every pair, tested bit for bit); value counts every pair "
                        "decided; dense_*: the same iterations from the same state with the bounds off"}
            if not args.no_compare:
                dense_ms, dense_a = dense_iterations(ctx, x, snap[0], snap[1], n, k, mode, prec, stream, args.steps)
                out["bounds"].update({"dense_ms_per_iteration": dense_ms, "dense_assign_ms": dense_a,
                                      "speedup_vs_dense_iteration": dense_ms / ms_step})
        ex = ctx.extract_stats()
        out["extraction_memo"] = {
            "clusters_reused_all_run": int(ex[2]), "clusters_compared_all_run": int(ex[1]),
            "what": "clusters whose members and centroid equal the previous extraction's reuse its output "
                    "(bit for bit; counted over the whole run, warm-up included)"}

    # the plain FP32 form on the same series, and the mixed form's agreement with it
    if out is not None and prec != PREC["fp32"] and not args.no_compare:
        out["plain_fp32_fused"] = plain_fp32_compare(ctx, x, labels, C, n, m, k, mode, prec, stream,
                                                     ms_step, a_ms)

    # library baseline: the reference's cuFFT formulation in plain FP32
    if out is not None and not args.no_cufft:
        cu_ms, cu_lab = cufft_assign_ms(x, C, F)
        agree = float((cu_lab.to(torch.int32) == labels).float().mean().item())
        out["plain_fp32_cufft"] = {"assign_pairs_per_s": n * k / (cu_ms / 1e3), "ms": cu_ms,
                                   "label_agreement_with_fused": agree,
                                   "what": "materialising NCC_3D + get_pos_idx on cuFFT (torch.fft), FP32, chunked"}
        out["fused_vs_cufft_assign_speedup"] = cu_ms / a_ms

    # end-to-end through the public C ABI with pinned host buffers: every step is one
    # call that copies the series in, z-normalises them, runs one whole iteration and
    # copies labels and centroids out
    if not args.no_e2e:
        pinned = torch.empty((n, m), dtype=torch.float32, pin_memory=True)
        pinned.numpy()[:] = data
        for _ in range(2):  # warm: the first call issues its stages directly, the second captures their graphs
            ctx.kshape_run(pinned.numpy(), k, mode=mode, precision=prec, max_iter=1, restart=False)
        walls = []
        for _ in range(3):
            t0 = time.perf_counter()
            r = ctx.kshape_run(pinned.numpy(), k, mode=mode, precision=prec, max_iter=1, restart=False)
            walls.append(time.perf_counter() - t0)
        wall = statistics.mean(walls)
        t0 = time.perf_counter()
        r3 = ctx.kshape_run(pinned.numpy(), k, mode=mode, precision=prec, max_iter=3, restart=False)
        wall3 = time.perf_counter() - t0
        e2e_val = max_over_ranks(wall, dist)  # every rank takes part
        if out is not None:
            out["e2e"] = {"value": world * n * k * r["iterations"] / e2e_val, "unit": "pairs/s",
                          "h2d_bytes_per_step": 4 * n * m, "d2h_bytes_per_step": 4 * n + 4 * k * m,
                          "step": "one tc_kshape_run call (h_data pinned, max_iter=1, restart=0): series in, "
                                  "z-norm, one whole iteration, labels and centroids out",
                          "wall_s_per_call": walls,
                          "three_iteration_call": {"iterations": r3["iterations"], "wall_s": wall3,
                                                   "pairs_per_s": n * k * r3["iterations"] / wall3}}
    if out is not None and not args.no_cpu:
        out["cpu_baseline"], out["fp64_oracle_report"] = oracle_iteration_report(ctx, data, x, labels, C, n, m, k,
                                                                                 mode, F, prec)
    ctx.close()
    if out is not None and world == 1 and args.workload == "c3" and not args.no_many_jobs:
        out["many_jobs"] = many_jobs_samples(args)
    if out is not None:
        print(json.dumps(out))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
