import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "times-c_gb300")
for p in (ROOT, PKG):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a)")


def _load(path):
    import importlib.util
    spec = importlib.util.spec_from_file_location(os.path.basename(path)[:-3] + "_build", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


@pytest.fixture(scope="session")
def built():
    """Builds (if needed) the engine and the oracle; returns the binding modules."""
    _load(os.path.join(PKG, "build.py")).build()
    _load(os.path.join(ROOT, "oracle", "build.py")).build_oracle()
    import timesc
    from oracle import oracle
    return timesc, oracle


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


@pytest.fixture(scope="session")
def gpu_ctx(built):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    timesc, _ = built
    ctx = timesc.Context(0)
    yield ctx
    ctx.close()
