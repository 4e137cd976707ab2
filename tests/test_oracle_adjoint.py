"""The oracle's float64 adjoint is the exact transpose of its forward map
(values and gradients are linear in the grid samples): for any upstream
(dv, dg), <adjoint(dv, dg), f> == <dv, value(f)> + <dg, grad(f)>."""
import numpy as np

from oracle.arb_oracle import OracleTricubic
from arbinterp_gb300 import synth


def test_adjoint_is_transpose_of_forward():
    f = synth.gaussian_field3(n=(12, 11, 13), seed=5).numpy()
    o = OracleTricubic(f)
    rng = np.random.default_rng(0)
    lo, hi = np.array(o.lo), np.array(o.hi)
    q = lo + (hi - lo) * rng.uniform(0, 1, (500, 3))
    out = o.query(q.copy())
    dv = rng.standard_normal(500)
    dg = rng.standard_normal((500, 3))
    gg = o.adjoint(q, dv, dg)
    lhs = gg @ o.fields["n"]
    rhs = dv @ out["norms"][:, 0] + np.sum(dg * out["grads"])
    assert abs(lhs - rhs) <= 1e-11 * max(1.0, abs(rhs))
    # rows outside the volume contribute nothing
    q2 = q.copy()
    q2[:10, 0] = hi[0] + 1.0
    gg2 = o.adjoint(q2, dv, dg)
    gg3 = o.adjoint(q2[10:], dv[10:], dg[10:])
    assert np.array_equal(gg2, gg3)
