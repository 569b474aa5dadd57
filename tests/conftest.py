import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    from oracle.oracle import load_oracle
    return load_oracle()


@pytest.fixture(scope="session")
def gpulib():
    """Build (if stale) and load libnbody_gb300.so; fails loudly when absent."""
    from nbody_gb300 import build as nb_build
    from nbody_gb300 import _lib
    nb_build.build()
    return _lib.load()


@pytest.fixture()
def make_engine(gpulib):
    from nbody_gb300.engine import create_engine
    made = []

    def _make(**param):
        param.setdefault("engine", "gb300")
        e = create_engine(param)
        assert e is not None, f"engine not created for {param}"
        made.append(e)
        return e

    yield _make
    for e in made:
        e.close()
