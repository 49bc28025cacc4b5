"""Shared test setup: import paths for the package and the oracle, the
`gpu` marker, and session fixtures that build the libraries once."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "tiny-path-tracer_gb300")
ORACLE = os.path.join(ROOT, "oracle")
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (PKG, ORACLE):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def built():
    """Builds libtpt.so and the oracle if needed."""
    import build as tpt_build
    import pyoracle

    tpt_build.build()
    pyoracle.build()
    return True


@pytest.fixture(scope="session")
def ctx(built):
    import tpt

    c = tpt.Context(0)
    yield c
    c.close()
