"""Many jobs on one GPU through the pool: a batch, continuous serving with
arrivals while other jobs run, and admission by device memory.  Each job's
result in the mix equals the same job run alone (labels identical, centroids
within 1e-6, same iteration count)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _specs(T, sizes, seed0=0, precision=0):
    out = []
    for i, (n, m, k, mode) in enumerate(sizes):
        data, _ = T.generate(n, m, k, noise=0.3, seed=seed0 + i)
        out.append(T.JobSpec(data, k, mode=mode, precision=precision, seed=seed0 + i, max_iter=12))
    return out


SIZES = [(3000, 512, 8, 0), (200, 64, 3, 1), (1500, 333, 5, 0), (64, 32, 2, 0), (5000, 128, 16, 1),
         (800, 1000, 4, 0), (2500, 256, 12, 1), (400, 2709, 3, 0), (1000, 96, 6, 0), (100, 700, 2, 1)]


def _alone(gpu_ctx, spec):
    j = spec.job
    return gpu_ctx.kshape_run(spec.data, spec.k, mode=j.mode, precision=j.precision, seed=j.seed,
                              max_iter=j.max_iter)


def _same(a, b, tag):
    assert a["iterations"] == b["iterations"], tag
    np.testing.assert_array_equal(a["labels"], b["labels"], err_msg=tag)
    np.testing.assert_allclose(a["centroids"], b["centroids"], atol=1e-6, err_msg=tag)


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_matches_alone(gpu_ctx, built, precision):
    T, _ = built
    specs = _specs(T, SIZES, seed0=10, precision=precision)
    alone = [_alone(gpu_ctx, s) for s in specs]
    pool = T.Pool(workers=4)
    try:
        st = pool.run_batch(specs)
    finally:
        pool.close()
    assert st == [T.OK] * len(specs)
    for i, (s, a) in enumerate(zip(specs, alone)):
        _same(s.result(), a, "job %d" % i)


def test_serving_arrivals_while_running(gpu_ctx, built):
    """Jobs submitted from another thread while earlier ones are on the GPU."""
    T, _ = built
    specs = _specs(T, SIZES + SIZES[:4], seed0=40)
    alone = [_alone(gpu_ctx, s) for s in specs]
    pool = T.Pool(workers=3)
    tickets = [None] * len(specs)
    seen_running = []

    def producer():
        for i, s in enumerate(specs):
            tickets[i] = pool.submit(s)
            seen_running.append(pool.stats()["running"])
            time.sleep(0.002)

    th = threading.Thread(target=producer)
    th.start()
    th.join()
    try:
        out = [pool.wait(t) for t in tickets]
    finally:
        pool.close()
    for i, (st, q, lat) in enumerate(out):
        assert st == T.OK and 0 <= q <= lat, (i, st, q, lat)
    assert max(seen_running) >= 1  # later jobs arrived while others ran
    for i, (s, a) in enumerate(zip(specs, alone)):
        _same(s.result(), a, "job %d" % i)


def test_admission_budget(gpu_ctx, built):
    T, _ = built
    specs = _specs(T, SIZES[:6], seed0=70)
    alone = [_alone(gpu_ctx, s) for s in specs]
    fp = [s.footprint() for s in specs]
    budget = int(max(fp) * 1.2)  # about one job in flight at a time
    pool = T.Pool(workers=4, hbm_budget_bytes=budget)
    try:
        big, _ = T.generate(20000, 1024, 4, noise=0.3, seed=1)
        with pytest.raises(T.TimescError) as e:
            pool.submit(T.JobSpec(big, 4))
        assert e.value.code == T.ERR_REJECTED
        tickets = [pool.submit(s) for s in specs]
        out = [pool.wait(t) for t in tickets]
        assert pool.stats()["held_bytes"] <= budget
    finally:
        pool.close()
    assert all(o[0] == T.OK for o in out)
    for i, (s, a) in enumerate(zip(specs, alone)):
        _same(s.result(), a, "job %d" % i)
