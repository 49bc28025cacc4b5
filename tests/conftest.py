"""Shared test setup: import paths for the package and the oracle, the
`gpu` marker, and session fixtures that build the libraries once."""
import os
import sys

import numpy as np
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


def zcheck(a, b):
    """a, b: (K, H, W, 3) independent render sets of the same estimator.

    Per pixel and channel, z = (difference of the K-run means) / (its
    standard error) follows Student's t with about 2K - 2 degrees of freedom
    when both sides estimate the same image, so its spread is
    sqrt(nu / (nu - 2)) (1.08 for K = 8, 1.12 for K = 6).  Measured between
    two sets of reference renders (and of oracle renders) of the same scene
    the spread is 1.05-1.15; a spread outside [0.9, 1.15 x the t value]
    or a mean shift beyond 0.12 fails.  The pixels of one reference run are
    correlated (its row streams are shifted copies of one mt19937 sequence),
    which is what widens the mean's band beyond iid noise."""
    k = a.shape[0]
    ma, mb = a.mean(axis=(1, 2, 3)), b.mean(axis=(1, 2, 3))
    se = np.sqrt(ma.var(ddof=1) / k + mb.var(ddof=1) / len(mb))
    assert abs(ma.mean() - mb.mean()) < 4 * se + 1e-7, (ma.mean(), mb.mean(), se)
    d = a.mean(0) - b.mean(0)
    s = np.sqrt(a.var(0, ddof=1) / k + b.var(0, ddof=1) / b.shape[0])
    ok = s > 0
    z = d[ok] / s[ok]
    nu = k + b.shape[0] - 2
    hi = 1.15 * np.sqrt(nu / (nu - 2.0))
    assert abs(z.mean()) < 0.12 and 0.9 < z.std() < hi, (z.mean(), z.std(), hi)
    assert np.mean(np.abs(z) > 5) < 0.005, np.mean(np.abs(z) > 5)
