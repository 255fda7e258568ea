import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def pytest_sessionstart(session):
    # libmgr.so is built in-tree when it is missing (nvcc cross-compiles for
    # sm_103a without a GPU), as the oracle's library is on first use
    from mia_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from mia_gb300 import build
        build.build()


@pytest.fixture(scope="session")
def goldens():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "reference_goldens.json")) as f:
        return json.load(f)["cases"]
