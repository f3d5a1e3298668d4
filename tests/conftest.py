"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and run only on a CUDA machine."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libhgb.so")


@pytest.fixture(scope="session")
def eng():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from hala_gb300 import build
    build.build()
    from hala_gb300 import engine as E
    e = E.gpu_engine(0)
    # parity tests compare products bit for bit with the reference's separately rounded loop
    e.set_spmv_mode("exact")
    return e


@pytest.fixture(scope="session")
def eng_fused(eng):
    """An engine in the default SpMV mode (one fused multiply-add per entry)."""
    from hala_gb300 import engine as E
    e = E.gpu_engine(0)
    assert e.spmv_mode() == "fused"
    return e


@pytest.fixture
def rng():
    return np.random.default_rng(1234)
