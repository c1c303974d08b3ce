import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(Path(__file__).resolve().parent))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103) and runs the engine")


@pytest.fixture(scope="session")
def engine():
    import myquantlib_gb300 as m
    from myquantlib_gb300 import build
    build.build()
    return m.default_engine()


@pytest.fixture(scope="session")
def oracle_lib():
    from oracle import oracle
    oracle.build(ref=False)
    return oracle
