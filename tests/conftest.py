import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libgfe.so")


@pytest.fixture(scope="session")
def gfe_cuda():
    """Builds (if needed) and loads libgfe.so; the GPU tests call through its C ABI."""
    import torch

    if not torch.cuda.is_available():
        pytest.fail("GPU test collected without a CUDA device")
    from iron_gb300 import build as gb
    gb.build()
    from iron_gb300 import _lib
    _lib.load()
    return torch.device("cuda", 0)
