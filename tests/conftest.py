import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def built_libraries():
    """Builds libbarnacle_gb300.so and the oracle in-tree when they are missing or stale."""
    from barnacle_gb300 import build as lib_build
    from oracle import build as oracle_build

    lib_build.build()
    oracle_build.build()
    yield


@pytest.fixture(scope="session")
def ctx():
    from barnacle_gb300 import Context

    c = Context(int(os.environ.get("BN_DEVICE", "0")))
    yield c
    c.close()
