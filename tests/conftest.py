import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Build the native libraries and the oracle port once per session."""
    from first_repo_gb300 import build
    import pyoracle
    build.build_gen()
    pyoracle.build_port()
    return True


@pytest.fixture(scope="session")
def built_cuda(built):
    from first_repo_gb300 import build
    build.build_cuda()
    return True
