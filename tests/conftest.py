import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session")
def oracle():
    from oracle import pyoracle
    pyoracle.build()
    pyoracle.lib()
    return pyoracle


@pytest.fixture(scope="session")
def pumplib():
    from pump_gb300 import lib
    from pump_gb300.build import build as build_lib
    build_lib()
    return lib


@pytest.fixture(scope="session")
def goldens():
    out = {}
    for p in sorted(glob.glob(os.path.join(GOLDEN, "*.npz"))):
        out[os.path.basename(p)[:-4]] = dict(np.load(p))
    return out


@pytest.fixture(scope="session")
def gpu(pumplib):
    """(torch, Context, stream handle) on cuda:0."""
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test run without a CUDA device")
    ctx = pumplib.Context(0)
    yield torch, ctx
    ctx.close()
