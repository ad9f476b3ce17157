"""Assignments with distance bounds carried across iterations give exactly the
labels, distances and centroids of evaluating every pair.

On series kept fixed across calls (tc_prepare_series, and inside tc_kshape_run)
a full assignment leaves a lower bound on every (series, centroid) distance; the
next assignments lower each bound by its centroid's movement and evaluate only
the pairs the bounds do not rule out, per 128-row tile of series grouped by their
best centroid (in the FP32 form that bounded BF16 pass is the screen and the FFT
kernel evaluates its candidates).  TIMESC_NO_BOUNDS=1 turns that off: both runs
must agree bit for bit, on ordinary data, exact ties, a zero centroid and a
centroid that flips sign.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(ctx, data, k, mode, init_chose, seed, bounds, prec=0, cap=30):
    if bounds:
        os.environ.pop("TIMESC_NO_BOUNDS", None)
    else:
        os.environ["TIMESC_NO_BOUNDS"] = "1"
    try:
        return ctx.kshape_run(data, k, mode=mode, precision=prec, init_chose=init_chose, seed=seed, max_iter=cap)
    finally:
        os.environ.pop("TIMESC_NO_BOUNDS", None)


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("mode,n,m,k,init_chose", [
    (0, 3000, 128, 4, 0),      # compat, F = 128
    (0, 2000, 100, 5, 0),      # compat pad-with-2 (2m - 1 < 512)
    (0, 4000, 300, 8, 1),      # compat, raw-row start
    (1, 3000, 200, 6, 0),      # canonical, F = 512
    (1, 3000, 400, 6, 0),      # canonical, F = 1024
    (0, 8000, 512, 32, 0),     # the precision configuration's shape, smaller n
])
def test_loop_with_bounds_equals_dense(built, prec, mode, n, m, k, init_chose):
    T, _ = built
    data, _ = T.generate(n, m, k, noise=0.3, seed=n + m)
    ctx = T.Context(0)
    try:
        s0 = ctx.assign_stats()
        a = _run(ctx, data, k, mode, init_chose, 3, bounds=True, prec=prec)
        s1 = ctx.assign_stats()
        b = _run(ctx, data, k, mode, init_chose, 3, bounds=False, prec=prec)
    finally:
        ctx.close()
    bounded, pairs = s1[1] - s0[1], s1[2] - s0[2]
    print("prec=%d n=%d m=%d k=%d mode=%d: %d iterations, %d bounded passes, %.3f of their pairs evaluated"
          % (prec, n, m, k, mode, a["iterations"], bounded, pairs / max(1, bounded * n * k)))
    assert a["iterations"] == b["iterations"]
    assert a["sum_class"] == b["sum_class"] and a["restarted"] == b["restarted"]
    assert np.array_equal(a["labels"], b["labels"])
    assert np.array_equal(a["centroids"], b["centroids"])
    if a["iterations"] >= 3:
        assert bounded >= 1


@pytest.mark.parametrize("prec", [0, 1])
def test_loop_regrouping_every_pass_equals_dense(built, prec):
    """TIMESC_REGROUP_SHARE=1000000: every bounded pass after a moved series first
    groups the series anew (the path the default threshold takes less often)."""
    T, _ = built
    n, m, k = 8000, 256, 16
    data, _ = T.generate(n, m, k, noise=0.3, seed=17)
    ctx = T.Context(0)
    os.environ["TIMESC_REGROUP_SHARE"] = "1000000"
    try:
        a = _run(ctx, data, k, 0, 0, 3, bounds=True, prec=prec)
        b = _run(ctx, data, k, 0, 0, 3, bounds=False, prec=prec)
    finally:
        os.environ.pop("TIMESC_REGROUP_SHARE", None)
        ctx.close()
    assert a["iterations"] == b["iterations"] >= 3
    assert np.array_equal(a["labels"], b["labels"])
    assert np.array_equal(a["centroids"], b["centroids"])


@pytest.mark.parametrize("prec", [0, 1])
def test_stage_calls_with_bounds_ties_zero_and_flip(built, prec):
    """Stage calls on prepared series: each call with bounds against a context that
    evaluates every pair, over a sequence of centroid sets with small moves, an exact
    duplicate (ties go to the first index even when the labels passed in name the
    later one), a zero centroid appearing and disappearing, and a sign flip."""
    import torch
    T, O = built
    n, m, k = 6000, 256, 8
    data, truth = T.generate(n, m, k, noise=0.3, seed=11)
    X = O.znorm(data.astype(np.float64)).astype(np.float32)
    x = torch.from_numpy(X).cuda()
    rng = np.random.default_rng(5)
    base = np.stack([X[truth == j].mean(axis=0) for j in range(k)]).astype(np.float32)
    seq = [base]
    c = base + 0.01 * rng.standard_normal(base.shape).astype(np.float32)
    seq.append(c)
    c = c.copy()
    c[5] = c[2]  # exact duplicate of centroid 2
    seq.append(c)
    c = c.copy()
    c[3] = 0.0   # a zero centroid
    seq.append(c)
    c = c.copy()
    c[3] = base[3]
    c[6] = -c[6]  # back from zero; a sign flip
    seq.append(c)
    seq.append(c + 1e-4 * rng.standard_normal(c.shape).astype(np.float32))
    ctx_b, ctx_d = T.Context(0), T.Context(0)
    try:
        ctx_b.prepare_series(x)
        lab_b = torch.zeros(n, dtype=torch.int32, device="cuda")
        lab_d = torch.zeros(n, dtype=torch.int32, device="cuda")
        s0 = ctx_b.assign_stats()
        for step, C in enumerate(seq):
            cg = torch.from_numpy(np.ascontiguousarray(C)).cuda()
            if step == 2:
                lab_b.fill_(5)  # labels in naming the later duplicate: the first index must still win
            db = torch.zeros(n, dtype=torch.float32, device="cuda")
            dd = torch.zeros(n, dtype=torch.float32, device="cuda")
            ctx_b.sbd_assign(x, cg, mode=0, precision=prec, labels=lab_b, dist=db)
            os.environ["TIMESC_NO_BOUNDS"] = "1"
            try:
                ctx_d.sbd_assign(x, cg, mode=0, precision=prec, labels=lab_d, dist=dd)
            finally:
                os.environ.pop("TIMESC_NO_BOUNDS", None)
            torch.cuda.synchronize()
            assert np.array_equal(lab_b.cpu().numpy(), lab_d.cpu().numpy()), step
            assert np.array_equal(db.cpu().numpy(), dd.cpu().numpy()), step
            if step == 2:
                assert not np.any(lab_b.cpu().numpy() == 5)
        s1 = ctx_b.assign_stats()
    finally:
        ctx_b.close()
        ctx_d.close()
    print("prec=%d stage sequence: %d full, %d bounded, %d pairs evaluated by the bounded calls"
          % (prec, s1[0] - s0[0], s1[1] - s0[1], s1[2] - s0[2]))
    assert s1[1] - s0[1] >= 3
