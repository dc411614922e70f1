import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests" / "golden"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built librawspec.so")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def cuda_device():
    """Skips on machines without a GPU; on a GPU machine the native library
    must load (a missing build is an error, not a skip)."""
    if not _cuda_available():
        pytest.skip("no CUDA device")
    from rawspec_gb300 import api
    api.load_library()
    return 0
