"""Test configuration: repo root on sys.path, the ``gpu`` marker, shared fixtures."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built_lib():
    """The CUDA library, built in-tree if stale (nvcc cross-compiles without a GPU)."""
    from yatfhe_gb300 import build

    return build.build()
