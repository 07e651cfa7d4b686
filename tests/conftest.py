"""pytest configuration: the `gpu` marker and build-on-demand of the engine
and the oracle (both builds are incremental)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

REPO = Path(__file__).resolve().parents[1]
for p in (REPO / "tests", REPO / "deac-cpp_gb300", REPO):
    if str(p) not in sys.path:
        sys.path.insert(0, str(p))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103) GPU")


@pytest.fixture(scope="session")
def oracle():
    subprocess.run(["make", "-s", "-C", str(REPO / "oracle"), "all"], check=True)
    from deac_testlib import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def engine_built():
    import build as engine_build  # deac-cpp_gb300/build.py
    engine_build.build()
    return engine_build


@pytest.fixture(scope="session")
def engine(engine_built):
    import deac_gb300
    deac_gb300.load_library()
    return deac_gb300
