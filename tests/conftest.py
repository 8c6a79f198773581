import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(REPO, "incidence-system-enumeration_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, os.path.join(REPO, "oracle"))
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (runs the CUDA path)")


def build_native():
    subprocess.run(["make", "-s", "-j4", "-C", PKG], check=True)


@pytest.fixture(scope="session")
def ctx():
    import ise_gb300
    build_native()
    c = ise_gb300.Context(max_items=1 << 17, aut_cap=64, max_trials=1 << 24)
    yield c
    c.close()
