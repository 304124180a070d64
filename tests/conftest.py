import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libsbpgpu.so")


@pytest.fixture(scope="session")
def oracle():
    import oracle_bind
    oracle_bind.build()
    return oracle_bind


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "toy_example.json")) as f:
        return json.load(f)


def _cuda_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu():
    """The sbp_gb300 package with its CUDA library loaded; fails loudly without a GPU."""
    if not _cuda_available():
        pytest.fail("GPU test run without a CUDA device")
    from sbp_gb300 import build
    build.build()
    import sbp_gb300
    sbp_gb300.load()
    return sbp_gb300
