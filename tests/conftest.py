"""Shared test setup: markers, paths, and the oracle / library handles."""
import importlib
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


@pytest.fixture(scope="session")
def instances():
    return importlib.import_module("acd-alm_gb300.instances")


@pytest.fixture(scope="session")
def oracle_lib():
    import oracle as O
    if not O.available("oracle"):
        O.build(ref=False)
    return O.Lib("oracle")


@pytest.fixture(scope="session")
def ref_lib():
    import oracle as O
    if not O.available("ref"):
        # builds the reference only where its sources are (oracle/Makefile)
        O.build(ref=True)
    if not O.available("ref"):
        pytest.skip("reference sources not present on this machine")
    return O.Lib("ref")
