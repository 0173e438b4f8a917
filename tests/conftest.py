import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); runs the product's kernels")
    config.addinivalue_line("markers", "slow: long CPU-only oracle runs")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds the CUDA library and the oracle once per session (cached by hash)."""
    from diaphane_gb300.build import build as build_product
    from oracle.build import build as build_oracle
    build_product()
    build_oracle()
    yield


@pytest.fixture(scope="session")
def threads():
    return max(1, min(16, os.cpu_count() or 1))
