"""The oracle library's copy of the synthetic workloads (the same generator
source, times-c_gb300/csrc/gen_core.h, compiled without the engine) gives the
engine's series and labels bit for bit, so the CPU baseline runs on the
engine's inputs without loading the engine's library."""
import numpy as np
import pytest


@pytest.mark.parametrize("n,m,classes,noise,dirichlet,seed", [
    (300, 128, 4, 0.2, 0.0, 0),        # the labelled CPU-sized configuration
    (5000, 333, 7, 0.3, 2.0, 5),       # Dirichlet class sizes, threaded generation
    (20000, 64, 32, 0.3, 0.0, 0),      # many classes
    (1, 2, 1, 0.0, 0.0, 9),            # smallest series
])
def test_oracle_generator_matches_engine(built, n, m, classes, noise, dirichlet, seed):
    T, O = built
    a, la = T.generate(n, m, classes, noise=noise, dirichlet=dirichlet, seed=seed)
    b, lb = O.generate(n, m, classes, noise=noise, dirichlet=dirichlet, seed=seed)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(la, lb)
