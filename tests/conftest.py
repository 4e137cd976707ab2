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
    """Rebuild the 41^3 scalar field rows (meshgrid 'ij' order) from the
    stored axes and value column: the synthetic generator itself is not
    bit-stable across CPU architectures."""
    X, Y, Z = np.meshgrid(g["c0_ax0"], g["c0_ax1"], g["c0_ax2"], indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel(), g["c0_U"]], 1)


def normwise(a, b):
    """max |a-b| / max |b| over finite entries, per column."""
    a = np.atleast_2d(np.asarray(a, float).reshape(len(a), -1))
    b = np.atleast_2d(np.asarray(b, float).reshape(len(b), -1))
    m = np.isfinite(b).all(axis=1)
    d = np.abs(a[m] - b[m]).max(axis=0)
    s = np.abs(b[m]).max(axis=0)
    return d / np.where(s == 0, 1, s)


GOLDEN_SCALE = os.path.join(ROOT, "tests", "golden", "golden_scale.npz")


@pytest.fixture(scope="session")
def golden_scale():
    """Reference outputs on a 48^3 dipole field ('both', 'norm', 'vector')
    and a 16^3 x 12 4D scalar field, 49,500 queries each (tests/golden/
    make_golden.py --scale)."""
    return dict(np.load(GOLDEN_SCALE))


def grid_rows(axes, values):
    """Field rows in meshgrid(indexing='ij') order from stored axes and value
    columns (the generators are not bit-stable across CPU architectures)."""
    G = np.meshgrid(*axes, indexing="ij")
    vals = np.asarray(values).reshape(len(G[0].ravel()), -1)
    return np.hstack([np.stack([g.ravel() for g in G], 1), vals])


def c1s_field(g):
    return grid_rows([g[f"c1_ax{a}"] for a in range(3)], g["c1_B"])


def c2s_field(g):
    return grid_rows([g[f"c2_ax{a}"] for a in range(4)], g["c2_U"])
