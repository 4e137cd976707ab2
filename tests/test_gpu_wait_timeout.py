"""The bounded device wait of the tensor-core coefficient solve runs out.

The 3D mixed-precision solve (coef3_tc) waits on an mbarrier for its MMAs
with a poll limit; if the limit runs out the kernel ORs ARB_ERR_TIMEOUT into
the caller's status word, waits with the full limit for the MMAs it issued,
releases its tensor memory and returns, so the context stays usable.  The
test lowers the limit of that wait to zero polls through the test hook
(arb_test_set_mma_wait_limit: nothing hangs and nothing faults, the wait
simply gives up before its first poll), checks that the timeout reaches the
host as an error, restores the limit and checks that the next solve on the
same device succeeds and matches the oracle."""
import numpy as np
import pytest

from conftest import normwise

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from arbinterp_gb300 import _lib
    _lib.lib()


def test_mma_wait_timeout_is_reported_and_recovered():
    import torch
    from arbinterp_gb300 import _lib, synth, tricubic
    from oracle.arb_oracle import OracleTricubic
    L = _lib.lib()
    f = synth.dipole_field3(n=(12, 12, 12), seed=21).numpy()
    o = tricubic(f, "quiet", mode="both", precision="mixed", strategy="table")
    assert L.arb_test_set_mma_wait_limit(0) == _lib.ARB_OK
    try:
        with pytest.raises(RuntimeError, match="device wait timed out"):
            o.allCoeffs()
    finally:
        assert L.arb_test_set_mma_wait_limit(-1) == _lib.ARB_OK
    torch.cuda.synchronize()          # the context is still usable
    assert not o._solved.any()
    # the same object solves normally once the limit is back
    o.allCoeffs()
    ref = OracleTricubic(f, mode="both")
    q = synth.uniform_queries(ref.lo, ref.hi, 3000, 30, ref.h, seed=22).numpy()
    want = ref.query(q.copy())
    comps, norms, grads = o.Query(q.copy())
    assert np.array_equal(o.queryInds, want["inds"])
    for name, got in (("comps", comps), ("norms", norms), ("grads", grads)):
        assert np.array_equal(np.isnan(got), np.isnan(want[name])), name
        assert (normwise(got, want[name]) <= 1e-6).all(), name
