import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Builds libtpdsplat and the oracle in-tree when missing or stale (fast when up to date)."""
    from oracle import build as obuild
    from torpedo_gb300 import build as pbuild

    pbuild.build()
    obuild.build()
    yield


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def pytest_collection_modifyitems(config, items):
    # GPU tests run in file order; nothing else to reorder.
    os.environ.setdefault("OMP_NUM_THREADS", str(min(16, os.cpu_count() or 4)))
