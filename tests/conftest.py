import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
TESTS = os.path.dirname(os.path.abspath(__file__))
if TESTS not in sys.path:
    sys.path.insert(0, TESTS)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a engine)")


@pytest.fixture(scope="session")
def engine_built():
    """The engine library, compiled in-tree if a source changed (nvcc cross-compiles)."""
    from epirust_gb300 import build

    return build.build()


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle

    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def gpu(engine_built):
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected on a machine without a CUDA device")
    return torch.cuda.get_device_name(0)
