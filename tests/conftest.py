import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def _have_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def gpu_ctx():
    """One engine context for the GPU tests of the session."""
    if not _have_gpu():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import afquantumsim_gb300 as aq
    ctx = aq.Context(0)
    yield ctx
    ctx.close()
