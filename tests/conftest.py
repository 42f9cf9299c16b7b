import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")
# The reference checkout, present only where the golden files were made;
# FLOCK_REFERENCE overrides the default location.
REFERENCE = os.environ.get("FLOCK_REFERENCE", "/root/reference")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built native library")


@pytest.fixture(scope="session")
def flock_lib():
    import flock_gb300
    return flock_gb300.lib()


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.orc()
    return oracle
