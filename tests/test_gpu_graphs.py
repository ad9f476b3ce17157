"""The whole loop with its stages replayed from CUDA graphs gives the same
results as the same stages launched one by one (TIMESC_NO_GRAPHS=1)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode,prec,init_chose", [(0, 0, 0), (1, 0, 1), (0, 1, 0), (1, 2, 0)])
def test_graph_replay_matches_direct_launches(gpu_ctx, built, mode, prec, init_chose):
    T, O = built
    data, _ = T.generate(3000, 200, 6, noise=0.3, seed=5)
    runs = []
    for no_graphs in (True, False):
        if no_graphs:
            os.environ["TIMESC_NO_GRAPHS"] = "1"
        else:
            os.environ.pop("TIMESC_NO_GRAPHS", None)
        try:
            runs.append(gpu_ctx.kshape_run(data, 6, mode=mode, precision=prec, init_chose=init_chose, seed=3,
                                           max_iter=30))
        finally:
            os.environ.pop("TIMESC_NO_GRAPHS", None)
    a, b = runs
    assert a["iterations"] == b["iterations"] and a["iterations"] >= 2
    np.testing.assert_array_equal(a["labels"], b["labels"])
    np.testing.assert_allclose(a["centroids"], b["centroids"], atol=1e-6)


def test_graph_replay_counts_kernels(gpu_ctx, built):
    """Replayed graphs still count their kernels in tc_launch_count."""
    T, _ = built
    data, _ = T.generate(2000, 128, 4, noise=0.3, seed=1)
    lib = T.lib()
    gpu_ctx.kshape_run(data, 4, max_iter=8, restart=False)  # one-time set-up launches (twiddle tables)
    counts = []
    for no_graphs in (True, False):
        if no_graphs:
            os.environ["TIMESC_NO_GRAPHS"] = "1"
        try:
            c0 = lib.tc_launch_count()
            r = gpu_ctx.kshape_run(data, 4, max_iter=8, restart=False)
            counts.append((lib.tc_launch_count() - c0, r["iterations"]))
        finally:
            os.environ.pop("TIMESC_NO_GRAPHS", None)
    assert counts[0] == counts[1]
