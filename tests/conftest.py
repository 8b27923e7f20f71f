"""Shared pytest configuration: the ``gpu`` marker and import paths."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in (ROOT, os.path.join(ROOT, "oracle")):
    if sub not in sys.path:
        sys.path.insert(0, sub)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running CPU oracle case")


@pytest.fixture(scope="session")
def oracle():
    import tnr_oracle
    return tnr_oracle
