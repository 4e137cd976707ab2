"""Fused RK4 particle trajectories (arb_rk4_trajectories) against a
fourth-order Runge-Kutta written here on top of the CPU oracle's queries."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _oracle_rk4(o, x, v, dt, nsteps, coef, grav, record_every):
    """x' = v, v' = coef * grad f + grav with the oracle's gradient; rows whose
    stage leaves the volume become NaN from then on."""
    grav = np.asarray(grav, float)

    def acc(p):
        r = o.query(p.copy())
        return coef * r["grads"] + grav

    x, v = x.copy(), v.copy()
    path = []
    for s in range(nsteps):
        k1 = acc(x)
        k2 = acc(x + 0.5 * dt * v)
        k3 = acc(x + 0.5 * dt * (v + 0.5 * dt * k1))
        k4 = acc(x + dt * (v + 0.5 * dt * k2))
        dx = v + 2 * (v + 0.5 * dt * k1) + 2 * (v + 0.5 * dt * k2) + (v + dt * k3)
        x = x + dt / 6 * dx
        v = v + dt / 6 * (k1 + 2 * k2 + 2 * k3 + k4)
        bad = ~(np.isfinite(k1).all(1) & np.isfinite(k2).all(1) & np.isfinite(k3).all(1) & np.isfinite(k4).all(1))
        x[bad] = np.nan
        v[bad] = np.nan
        if record_every and (s + 1) % record_every == 0:
            path.append(np.hstack([x, v]))
    return x, v, np.array(path)


def _setup(kind):
    from arbinterp_gb300 import synth
    if kind == "scalar":
        f = synth.gaussian_field3(n=(22, 20, 18), h=(0.1, 0.12, 0.08), seed=11).numpy()
        return f, {}
    f = synth.dipole_field3(n=(24, 24, 24), seed=12).numpy()
    return f, {"mode": "both"}


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["scalar", "both"])
def test_trajectories_match_oracle_rk4(prec, kind):
    from arbinterp_gb300 import tricubic
    from oracle.arb_oracle import OracleTricubic
    f, kw = _setup(kind)
    o = OracleTricubic(f, **kw)
    rng = np.random.default_rng(3)
    lo, hi = np.array(o.lo), np.array(o.hi)
    n = 96
    x0 = lo + (hi - lo) * rng.uniform(0.3, 0.7, (n, 3))
    v0 = (hi - lo) * rng.uniform(-0.05, 0.05, (n, 3))
    # one particle aimed out through the lower x face
    x0[0] = lo + (hi - lo) * np.array([0.02, 0.5, 0.5])
    v0[0] = [-(hi - lo)[0], 0.0, 0.0]
    dt, nsteps, coef, grav = 0.05, 24, -1e-3, (0.0, 0.0, -0.01)
    g = tricubic(f, "quiet", precision=prec, **kw)
    x, v, path = g.trajectories(x0, v0, dt, nsteps, coef=coef, gravity=grav, record_every=6)
    rx, rv, rpath = _oracle_rk4(o, x0, v0, dt, nsteps, coef, grav, 6)
    assert path.shape == (4, n, 6)
    assert np.array_equal(np.isnan(x), np.isnan(rx))
    assert np.isnan(x[0]).all() and g.lost >= 1
    assert g.lost == int(np.isnan(rx).any(1).sum())
    m = np.isfinite(rx).all(1)
    scale = np.abs(hi - lo).max()
    tol = 1e-11 if prec == "fp64" else 1e-6
    assert np.abs(x[m] - rx[m]).max() <= tol * scale
    assert np.abs(v[m] - rv[m]).max() <= tol * scale
    assert np.array_equal(np.isnan(path), np.isnan(rpath))
    pm = np.isfinite(rpath)
    assert np.abs(path[pm] - rpath[pm]).max() <= tol * scale


def test_trajectories_device_tensors_and_vector_mode():
    import torch
    from arbinterp_gb300 import tricubic
    f, _ = _setup("both")
    g = tricubic(f, "quiet", mode="both", precision="mixed")
    lo, hi = np.array(g._lo, float), np.array(g._hi, float)
    x0 = torch.tensor(lo + (hi - lo) * 0.5, device="cuda").repeat(8, 1)
    v0 = torch.zeros_like(x0)
    x, v = g.trajectories(x0, v0, 0.01, 5)
    assert x.is_cuda and x.shape == (8, 3) and torch.isfinite(x).all()
    gv = tricubic(f, "quiet", mode="vector")
    with pytest.raises(ValueError):
        gv.trajectories(x0.cpu().numpy(), v0.cpu().numpy(), 0.01, 5)


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_spatial_sort_changes_nothing(prec):
    """Integrating in Z-order returns the very same states, path and lost
    count in the caller's order as integrating in the given order."""
    from arbinterp_gb300 import tricubic
    f, kw = _setup("both")
    g = tricubic(f, "quiet", precision=prec, **kw)
    rng = np.random.default_rng(9)
    lo, hi = np.array(g._lo, float), np.array(g._hi, float)
    x0 = lo + (hi - lo) * rng.uniform(0.05, 0.95, (3000, 3))
    v0 = (hi - lo) * rng.uniform(-0.2, 0.2, (3000, 3))
    x0[17] = np.nan
    a = g.trajectories(x0, v0, 0.05, 30, coef=-1e-3, record_every=10)
    la = g.lost
    b = g.trajectories(x0, v0, 0.05, 30, coef=-1e-3, record_every=10, spatial_sort=False)
    assert g.lost == la and la > 1
    for p, q in zip(a, b):
        assert np.array_equal(p, q, equal_nan=True)
