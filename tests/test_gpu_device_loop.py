"""The k-Shape loop run as one CUDA graph gives exactly the host-driven loop's results.

Once an iteration's extraction and assignment have been captured as graphs,
tc_kshape_run runs the remaining iterations as one launch: a WHILE node over the
stages whose control kernels restate, on the device, the host loop's decisions
(kshape.cuh:235-311 / :383-455) - class-count stop, convergence with the inertia rule
and the old-label copy, and the bounded assignment's refresh / regroup rule.
TIMESC_DEVICE_LOOP=1 turns it on (by default every iteration is driven by the host).
Both must agree bit for bit: labels, centroids, iteration count and inertia, in both loop orders, both
precision forms, with the restart.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _env(device_loop):
    if device_loop:
        os.environ["TIMESC_DEVICE_LOOP"] = "1"
    else:
        os.environ.pop("TIMESC_DEVICE_LOOP", None)


def _run(T, data, k, device_loop, **kw):
    _env(device_loop)
    ctx = T.Context(0)
    try:
        r = ctx.kshape_run(data, k, **kw)
        r["assign_stats"] = ctx.assign_stats()
        r["loop_stats"] = ctx.loop_stats()
    finally:
        _env(False)
        ctx.close()
    return r


def _same(a, b):
    assert a["iterations"] == b["iterations"]
    assert a["sum_class"] == b["sum_class"] and a["restarted"] == b["restarted"]
    assert a["inertia"] == b["inertia"]
    assert np.array_equal(a["labels"], b["labels"])
    assert np.array_equal(a["centroids"].view(np.uint32), b["centroids"].view(np.uint32))
    # passes that kept bounds (full + bounded); the pairs a bounded pass evaluates vary
    # from run to run, as the series' order inside a group comes from atomics
    assert sum(a["assign_stats"][:2]) == sum(b["assign_stats"][:2])


@pytest.mark.parametrize("mode,prec,n,m,k,init_chose,max_iter", [
    (0, 0, 6000, 128, 8, 0, 30),     # compat FP32, screened and bounded
    (0, 1, 6000, 128, 8, 0, 30),     # compat BF16 mixed, bounded
    (0, 0, 3000, 300, 6, 1, 30),     # raw-row start: assignment first (k_shape_tsl order)
    (0, 1, 8000, 512, 32, 0, 30),    # the precision configuration's shape, smaller n
    (0, 1, 8000, 512, 32, 1, 30),    # the same, assignment first
    (0, 1, 8000, 512, 32, 0, 6),     # the iteration cap reached inside the graph
    (1, 0, 3000, 200, 6, 0, 30),     # canonical (repeated squaring)
    (0, 0, 1500, 1300, 4, 0, 30),    # m > 1024: FFT assignment only, no bounds
])
def test_loop_graph_equals_host_loop(built, mode, prec, n, m, k, init_chose, max_iter):
    T, _ = built
    data, _ = T.generate(n, m, k, noise=0.3, seed=n + m + 11)
    kw = dict(mode=mode, precision=prec, init_chose=init_chose, seed=5, max_iter=max_iter)
    host = _run(T, data, k, False, **kw)
    dev = _run(T, data, k, True, **kw)
    d_it, h_it, builds = dev["loop_stats"]
    print("mode=%d prec=%d n=%d m=%d k=%d order=%d: %d iterations, %d in the loop graph (%d graphs built), "
          "bounds passes %s" % (mode, prec, n, m, k, init_chose, dev["iterations"], d_it, builds,
                                dev["assign_stats"]))
    _same(host, dev)
    assert host["loop_stats"][0] == 0  # all on the host
    assert d_it + h_it == dev["iterations"]
    if dev["iterations"] >= 10:  # the first iterations capture the stages on the host
        assert d_it >= 1 and builds >= 1


def test_loop_graph_regrouping_every_pass(built):
    """The loop graph's control kernel takes the regroup threshold it was given."""
    T, _ = built
    data, _ = T.generate(8000, 256, 16, noise=0.3, seed=17)
    os.environ["TIMESC_REGROUP_SHARE"] = "1000000"
    try:
        host = _run(T, data, 16, False, precision=1, seed=3, max_iter=25)
        dev = _run(T, data, 16, True, precision=1, seed=3, max_iter=25)
    finally:
        os.environ.pop("TIMESC_REGROUP_SHARE", None)
    _same(host, dev)


def test_loop_graph_with_restart(built):
    T, _ = built
    data, _ = T.generate(300, 128, 4, noise=0.3, seed=0)
    init = np.zeros(300, np.int32)  # one cluster -> sum_class 1 -> rerun with the full eigensolver
    host = _run(T, data, 4, False, init_labels=init, max_iter=10)
    dev = _run(T, data, 4, True, init_labels=init, max_iter=10)
    assert dev["restarted"] == 1
    _same(host, dev)


def test_loop_graph_on_repeated_runs(built):
    """Runs on one context reuse nothing stale: the second run of the same job gives
    the first one's results, as does a different job in between."""
    T, _ = built
    a_data, _ = T.generate(5000, 256, 8, noise=0.3, seed=3)
    b_data, _ = T.generate(4000, 200, 5, noise=0.3, seed=4)
    _env(True)
    ctx = T.Context(0)
    try:
        r1 = ctx.kshape_run(a_data, 8, precision=1, seed=5, max_iter=25)
        ctx.kshape_run(b_data, 5, precision=0, seed=5, max_iter=25)
        r2 = ctx.kshape_run(a_data, 8, precision=1, seed=5, max_iter=25)
        d_it, _, _ = ctx.loop_stats()
    finally:
        _env(False)
        ctx.close()
    assert d_it >= 1
    assert r1["iterations"] == r2["iterations"] and r1["inertia"] == r2["inertia"]
    assert np.array_equal(r1["labels"], r2["labels"])
    assert np.array_equal(r1["centroids"].view(np.uint32), r2["centroids"].view(np.uint32))
