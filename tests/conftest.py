import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: test needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running test")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    # the engine library and the oracle are compiled in-tree (no-ops when up to date)
    from oracle import build as obuild
    from parafrost_gb300 import build as ebuild
    ebuild.build()
    obuild.build()
    yield
