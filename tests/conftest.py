"""pytest configuration: the `gpu` marker and shared fixtures."""
import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    return oracle.lib()


@pytest.fixture(scope="session")
def gpu_ctx():
    """One context per test session; fails loudly if the extension or the GPU is missing."""
    from bling_gb300 import build
    build.build()
    from bling_gb300.api import Context
    ctx = Context(device=int(os.environ.get("BLING_DEVICE", "0")))
    yield ctx
    ctx.close()
