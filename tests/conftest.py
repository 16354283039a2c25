import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built engine library")


@pytest.fixture(scope="session")
def oracle():
    """Build (if needed) and return the oracle module (C restatement)."""
    import oracle_lib
    oracle_lib.build_oracle()
    return oracle_lib


@pytest.fixture(scope="session")
def engine():
    """The engine package with its native library loaded (GPU tests only)."""
    import gpvmc_gb300
    from gpvmc_gb300 import build as b
    if not os.path.exists(b.LIB):
        b.build()
    gpvmc_gb300.lib()
    return gpvmc_gb300
