"""Shared fixtures.  GPU tests carry ``@pytest.mark.gpu``; everything else runs
on the CPU.  The oracle (``oracle/``) is imported here only as the checker."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")
    config.addinivalue_line("markers", "slow: takes more than a few seconds")


@pytest.fixture(scope="session")
def lib():
    """The built C-ABI library (built here if missing)."""
    from gturbo3d_gb300 import build, _lib
    if not _lib.LIB_PATH.exists():
        build.build()
    return _lib.load()
