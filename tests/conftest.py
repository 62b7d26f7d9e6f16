"""Test configuration: the `gpu` marker, and a session-wide build of the
libraries (a no-op when they are up to date)."""
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103)")


@pytest.fixture(scope="session", autouse=True)
def _built():
    from libcraw_gb300 import build
    return build.build()
