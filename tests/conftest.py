import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")


def gpu_available():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built if needed; fails (never skips) when it cannot load."""
    from morpheus_gb300 import build as B, _native
    B.build()
    L = _native.lib()
    n = __import__("ctypes").c_int()
    assert L.cuda_get_device_count(__import__("ctypes").byref(n)) == 0 and n.value > 0, "no CUDA device visible"
    return L
