"""Shared test setup.

- registers the ``gpu`` marker (tests that need a CUDA device);
- makes the product binding (``ufo-ir_gb300/ufoir``) and the oracle binding
  (``oracle/pyoracle.py``, test infrastructure) importable;
- builds the oracle on first use.
"""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "ufo-ir_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 device")


@pytest.fixture(scope="session")
def oracle():
    import pyoracle
    pyoracle.build()
    return pyoracle


@pytest.fixture(scope="session")
def ufoir_lib():
    import ufoir
    ufoir.lib()          # raises if libufoir.so is missing: no fallback
    return ufoir


@pytest.fixture(scope="session")
def gpu_ctx(ufoir_lib):
    ctx = ufoir_lib.Context(0)
    yield ctx
    ctx.close()
