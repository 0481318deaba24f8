import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def golden():
    """Fixtures written by tests/golden/make_golden.py from the reference."""
    from tests.golden_cases import load_cases
    return load_cases()
