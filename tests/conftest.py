"""pytest set-up: the ``gpu`` marker, and GPU tests skipped where no CUDA device is visible."""

import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

# The reference's own package (mpm_core: the solver interface, the bake runner, the cache format), when an
# install of it sits in baseline/_ref (pip install --target). Tests then run against the real interface
# records and the unchanged runner; without it the data-only stand-ins are used and the runner tests skip.
# MPM_GB300_NO_MPM_CORE=1 runs the suite without it.
REF_INSTALL = ROOT / "baseline" / "_ref"
if (REF_INSTALL / "mpm_core").is_dir() and not os.environ.get("MPM_GB300_NO_MPM_CORE"):
    sys.path.append(str(REF_INSTALL))


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
