"""Boundary conditions (ghost layer per face): the interpolation volume
becomes the whole input grid; Neumann gives zero normal derivative at
boundary nodes, Dirichlet the odd reflection about the boundary sample; both
equal the oracle built on the same ghost-padded rows."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _pad_np(f, bc):
    """The same ghost layer built independently in NumPy (x fastest rows)."""
    xs, ys, zs = (np.unique(f[:, a]) for a in range(3))
    n = (len(xs), len(ys), len(zs))
    order = np.lexsort((f[:, 0], f[:, 1], f[:, 2]))
    v = f[order, 3].reshape(n[2], n[1], n[0])
    for axis in (2, 1, 0):                        # x, y, z in array order (z, y, x)
        v = np.moveaxis(v, axis, 0)
        if bc == "neumann":
            lo, hi = v[1:2], v[-2:-1]
        else:
            lo, hi = 2 * v[0:1] - v[1:2], 2 * v[-1:] - v[-2:-1]
        v = np.moveaxis(np.concatenate([lo, v, hi], 0), 0, axis)
    ax = [np.concatenate([[a[0] - (a[1] - a[0])], a, [a[-1] + (a[-1] - a[-2])]]) for a in (xs, ys, zs)]
    Z, Y, X = np.meshgrid(ax[2], ax[1], ax[0], indexing="ij")
    return np.stack([X.ravel(), Y.ravel(), Z.ravel(), v.ravel()], 1)


@pytest.mark.parametrize("bc", ["neumann", "dirichlet"])
def test_boundary_padding(bc):
    from arbinterp_gb300 import tricubic, synth
    from oracle.arb_oracle import OracleTricubic
    f = synth.gaussian_field3(n=(12, 11, 10), h=(0.1, 0.12, 0.08), seed=21).numpy()
    plain = tricubic(f, "quiet")
    g = tricubic(f, "quiet", boundary=bc)
    xs, ys, zs = (np.unique(f[:, a]) for a in range(3))
    assert (g.xIntMin, g.xIntMax) == (xs[0], xs[-1]) and (plain.xIntMin, plain.xIntMax) == (xs[1], xs[-2])
    o = OracleTricubic(_pad_np(f, bc))
    rng = np.random.default_rng(1)
    q = np.stack([rng.uniform(xs[0], xs[-1], 3000), rng.uniform(ys[0], ys[-1], 3000),
                  rng.uniform(zs[0], zs[-1], 3000)], 1)
    ref = o.query(q.copy())
    n_, g_ = g.Query(q.copy())
    assert np.isfinite(n_).all()
    assert np.abs(n_ - ref["norms"]).max() <= 1e-12 * np.abs(ref["norms"]).max()
    assert np.abs(g_ - ref["grads"]).max() <= 1e-12 * np.abs(ref["grads"]).max()
    # at a boundary node: the sample itself, and the boundary-condition slope
    node = np.array([[xs[0], ys[4], zs[5]]])
    nv, gv = g.Query(node.copy())
    fv = f[(f[:, 0] == xs[0]) & (f[:, 1] == ys[4]) & (f[:, 2] == zs[5]), 3][0]
    f1 = f[(f[:, 0] == xs[1]) & (f[:, 1] == ys[4]) & (f[:, 2] == zs[5]), 3][0]
    assert abs(nv[0, 0] - fv) <= 1e-12 * max(1.0, abs(fv))
    hx = xs[1] - xs[0]
    want = 0.0 if bc == "neumann" else (f1 - fv) / hx
    assert abs(gv[0, 0] - want) <= 1e-9 * max(1.0, abs(want))
