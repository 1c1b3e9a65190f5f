import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "products.json")) as f:
        return json.load(f)["products"]


@pytest.fixture(scope="session")
def gpu():
    """The native library, initialised on device 0 (GPU tests only)."""
    from preclib_gb300 import native
    native.init(0)
    return native
