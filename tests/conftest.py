import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.dirname(os.path.abspath(__file__))):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built engine library")
    config.addinivalue_line("markers", "slow: longer CPU runs")


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle bindings, built on first use."""
    from oracle import bindings

    bindings.build(ref=os.path.isdir(bindings.REF_SRC))
    return bindings


@pytest.fixture(scope="session")
def engine_lib():
    """The engine library, built on first use (nvcc cross-compiles without a GPU)."""
    from nmc_gb300 import build

    build.build()
    from nmc_gb300 import engine

    return engine


@pytest.fixture(scope="session")
def gpu(engine_lib):
    import ctypes

    try:
        import torch

        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    if not ok:
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return engine_lib
