import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU test")


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def gpu_lib():
    """The in-tree CUDA library; GPU tests fail (not skip) when it is missing."""
    from qudrip_gb300 import _capi
    return _capi.lib()


@pytest.fixture(scope="session")
def ctx(gpu_lib):
    import qudrip_gb300 as q
    return q.default_context()
