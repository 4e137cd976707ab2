import os
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300 / sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    return dict(np.load(GOLDEN))


def c0_field(g):
    """Rebuild the 41^3 scalar field rows from the stored value column."""
    from arbinterp_gb300 import synth
    f = synth.gaussian_field3(seed=0).numpy()
    assert np.array_equal(f[:, 3], g["c0_U"]), "synthetic generator drifted from the fixture"
    return f


def normwise(a, b):
    """max |a-b| / max |b| over finite entries, per column."""
    a = np.atleast_2d(np.asarray(a, float).reshape(len(a), -1))
    b = np.atleast_2d(np.asarray(b, float).reshape(len(b), -1))
    m = np.isfinite(b).all(axis=1)
    d = np.abs(a[m] - b[m]).max(axis=0)
    s = np.abs(b[m]).max(axis=0)
    return d / np.where(s == 0, 1, s)
