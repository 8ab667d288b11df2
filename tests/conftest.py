import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


@pytest.fixture(scope="session")
def gpu_lib():
    """Builds (if stale) and loads the CUDA library; GPU tests only."""
    if not HAS_GPU:
        pytest.skip("no CUDA device")
    from vulkanexp_gb300 import build, ddgi

    build.build()
    return ddgi.load_library()


@pytest.fixture(scope="session")
def room_workload():
    from vulkanexp_gb300 import scenes

    return scenes.workload(0)


@pytest.fixture(scope="session")
def room_oracle(room_workload):
    from oracle.oracle import Oracle

    return Oracle(room_workload.scene)


def rel_err(a, b, floor):
    """|a - b| / max(|b|, floor), elementwise."""
    return np.abs(a.astype(np.float64) - b.astype(np.float64)) / np.maximum(np.abs(b.astype(np.float64)), floor)
