"""Shared fixtures: put the package and the oracle on sys.path, register
the gpu marker, build the CUDA library and the oracle once per session."""
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
PKG = REPO / "skyfall-viewer_gb300"
for p in (str(REPO), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def orc():
    from oracle import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def sky():
    from skyfall import build
    build.build()
    import skyfall
    return skyfall
