import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session", autouse=True)
def _built_libraries():
    """Build the oracle (test infrastructure) and the native library once."""
    from tests import oracle_binding
    oracle_binding.build()
    from turns2d_urans_git_gb300 import build as nbuild
    from turns2d_urans_git_gb300.abi import lib_path
    if not os.path.exists(lib_path()):
        nbuild.build()
    yield
