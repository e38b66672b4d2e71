import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU; run with -m gpu")


def has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:  # pragma: no cover
        return False


@pytest.fixture(scope="session")
def gpu():
    """GPU tests run only where a device exists; a missing device is a failure, not a skip."""
    if not has_gpu():
        pytest.fail("GPU test selected but no CUDA device is visible")
    from cuda_ndt_matcher_gb300 import capi
    capi.load()
    return True


@pytest.fixture(scope="session")
def oracle():
    from oracle import oracle as O
    O.lib()
    return O


@pytest.fixture(scope="session")
def single_cases():
    from cuda_ndt_matcher_gb300 import synth
    return [synth.single_case(seed) for seed in (1, 2, 3)]
