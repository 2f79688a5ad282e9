"""Shared test setup: repo on sys.path, the `gpu` marker, oracle libraries."""
import os
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if REPO not in sys.path:
    sys.path.insert(0, REPO)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (runs on the GB300 box)")


@pytest.fixture(scope="session")
def oracle_mod():
    """The oracle package with both libraries built (builds them on first use)."""
    import oracle
    if not (os.path.exists(os.path.join(oracle.OUT, "libcport.so")) and oracle.ref_available()):
        oracle.build()
    return oracle
