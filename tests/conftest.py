import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

# Location of a checkout of the reference (its fixture files are read by a few
# CPU-only pins): the environment variable ATOMISTICA_REFERENCE, else a
# directory named "reference" beside this repository; tests that need it are
# skipped when neither exists.
REFERENCE = os.environ.get("ATOMISTICA_REFERENCE",
                           os.path.join(os.path.dirname(ROOT), "reference"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")
    config.addinivalue_line("markers", "slow: full-size workloads")


@pytest.fixture(scope="session")
def reference_tests_dir():
    d = os.path.join(REFERENCE, "tests")
    if not os.path.isdir(d):
        pytest.skip("reference fixtures not available")
    return d


@pytest.fixture(scope="session")
def gpu():
    from atomistica_gb300 import _lib
    _lib.load()
    if _lib.device_count() < 1:
        pytest.fail("no CUDA device visible for a gpu-marked test")
    return True
