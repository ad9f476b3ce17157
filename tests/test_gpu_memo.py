"""The extraction's memo of unchanged clusters gives exactly the centroids of
recomputing every cluster.

On series kept fixed across calls (tc_prepare_series, and the run's own copy
inside tc_kshape_run) a cluster whose members and input centroid equal those of
the previous extraction gets that extraction's output again instead of being
recomputed: every extraction stage is deterministic per cluster.
TIMESC_NO_MEMO=1 turns it off: both must agree bit for bit - whole runs, and
stage calls where labels or centroids change between calls.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _env(memo):
    if memo:
        os.environ.pop("TIMESC_NO_MEMO", None)
    else:
        os.environ["TIMESC_NO_MEMO"] = "1"


@pytest.mark.parametrize("mode,prec,n,m,k,init_chose", [
    (0, 0, 6000, 128, 8, 0),     # compat FP32 (F = 128)
    (0, 1, 6000, 128, 8, 0),     # compat BF16 mixed
    (0, 0, 3000, 300, 6, 1),     # compat, raw-row start (the alignment gate opens)
    (0, 0, 1500, 1300, 4, 0),    # m > 1024: row-major gather, transposed for the Gram; 16-CTA power clusters
    (1, 0, 3000, 200, 6, 0),     # canonical (repeated squaring where it fits: memo off there)
    (0, 0, 8000, 512, 32, 0),    # the precision configuration's shape, smaller n
])
def test_loop_with_memo_equals_recomputing(built, mode, prec, n, m, k, init_chose):
    T, _ = built
    data, _ = T.generate(n, m, k, noise=0.3, seed=n + m + 7)
    ctx = T.Context(0)
    try:
        s0 = ctx.extract_stats()
        _env(True)
        a = ctx.kshape_run(data, k, mode=mode, precision=prec, init_chose=init_chose, seed=5, max_iter=30)
        s1 = ctx.extract_stats()
        _env(False)
        b = ctx.kshape_run(data, k, mode=mode, precision=prec, init_chose=init_chose, seed=5, max_iter=30)
        s2 = ctx.extract_stats()
    finally:
        os.environ.pop("TIMESC_NO_MEMO", None)
        ctx.close()
    ext, clus, reused = (y - x for x, y in zip(s0, s1))
    print("mode=%d prec=%d n=%d m=%d k=%d: %d iterations, %d extractions with the memo, %d of %d clusters reused"
          % (mode, prec, n, m, k, a["iterations"], ext, reused, clus))
    assert s2 == s1  # nothing compared with the memo off
    assert a["iterations"] == b["iterations"]
    assert a["sum_class"] == b["sum_class"] and a["restarted"] == b["restarted"]
    assert np.array_equal(a["labels"], b["labels"])
    assert np.array_equal(a["centroids"].view(np.uint32), b["centroids"].view(np.uint32))
    if mode == 0:
        assert ext >= 1 and clus == ext * k


@pytest.mark.parametrize("prec", [0, 1])
def test_stage_calls_reuse_only_unchanged_clusters(built, prec):
    import torch
    T, _ = built
    n, m, k = 4000, 256, 8
    data, truth = T.generate(n, m, k, noise=0.3, seed=21)
    x = torch.from_numpy(data).cuda()
    ref = torch.from_numpy(data).cuda()
    ctx, plain = T.Context(0), T.Context(0)
    try:
        for c, t in ((ctx, x), (plain, ref)):
            c.znorm(t)
        ctx.prepare_series(x)
        lab = torch.from_numpy(truth.astype(np.int32)).cuda()
        C = torch.zeros((k, m), dtype=torch.float32, device="cuda")
        C0 = C.clone()

        def both(labels, Cin):
            """the memo context and a context without prepared series (no memo)"""
            a, b = Cin.clone(), Cin.clone()
            ctx.extract_shapes(x, labels, a, precision=prec)
            plain.extract_shapes(ref, labels, b, precision=prec)
            torch.cuda.synchronize()
            assert torch.equal(a.view(torch.int32), b.view(torch.int32))
            return a

        s0 = ctx.extract_stats()
        C1 = both(lab, C0)                   # first call: nothing to compare with
        s1 = ctx.extract_stats()
        C1b = both(lab, C0)                  # same labels and centroids: all reused
        s2 = ctx.extract_stats()
        assert torch.equal(C1.view(torch.int32), C1b.view(torch.int32))
        lab2 = lab.clone()
        lab2[17] = (int(lab2[17]) + 1) % k   # one series moves: two clusters recomputed
        both(lab2, C0)
        s3 = ctx.extract_stats()
        both(lab2, C1)                       # new input centroids
        C_in = C1.clone()                    # then another input centroid for one cluster
        C_in[3] *= 2.0
        s3b = ctx.extract_stats()
        both(lab2, C_in)
        s4 = ctx.extract_stats()
        both(lab2, C_in)                     # and again: all reused
        s5 = ctx.extract_stats()
        both(lab2, C_in)
        shift = torch.zeros(n, dtype=torch.int32, device="cuda")
        a = C_in.clone()
        ctx.extract_shapes(x, lab2, a, shift=shift, precision=prec)  # caller shifts: not compared
        s6 = ctx.extract_stats()
    finally:
        ctx.close()
        plain.close()
    reused = [s[2] for s in (s0, s1, s2, s3, s3b, s4, s5)]
    print("prec=%d reused per call:" % prec, np.diff(reused).tolist())
    assert s1[2] - s0[2] == 0 and s1[1] - s0[1] == k
    assert s2[2] - s1[2] == k
    assert s3[2] - s2[2] == k - 2
    assert s4[2] - s3b[2] == k - 1
    assert s5[2] - s4[2] == k
    assert s6[0] - s5[0] == 1  # the call before the shifted one compared; that one did not
