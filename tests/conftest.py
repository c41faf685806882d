"""pytest set-up: the ``gpu`` marker, and GPU tests skipped where no CUDA device is visible."""

import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs the sm_103a kernels)")


def _cuda_available() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    gpu_items = [item for item in items if "gpu" in item.keywords]
    if gpu_items and not _cuda_available():
        skip = pytest.mark.skip(reason="no CUDA device")
        for item in gpu_items:
            item.add_marker(skip)


@pytest.fixture
def device():
    return "cuda:0"
