"""The allocation-free entry point (arb_query_eval_sorted_noalloc).

Some callers cannot allocate device memory while they run (engines that own
every device byte through their own pool, plugin hosts that forbid
allocation inside callbacks, services that must not grow device memory
mid-run).  For them the library keeps a fixed scratch array of
ARB_NOALLOC_SCRATCH_BYTES per GPU.  This test calls that entry point through
the C ABI twice in a row, on different query sets, and checks each result
against the workspace entry point (arb_query_eval_sorted) on the same
inputs: identical cell indices, out-of-volume rows, NaN masks and values.
It covers 3D vector ('both'), 3D scalar and 4D scalar fields, evaluating on
the fly and from a coefficient table.

It sits in a file of its own, collected last, and works alone in a fresh
process as well as after the other tests."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from arbinterp_gb300 import _lib
    return torch, _lib, _lib.lib()


def _run(torch, _lib, L, o, q, entry, use_table):
    n, d = q.shape[0], o._dim
    f64 = dict(dtype=torch.float64, device="cuda")
    comps = torch.full((n, 3), -7.0, **f64)
    norms = torch.full((n, 1), -7.0, **f64)
    grads = torch.full((n, d), -7.0, **f64)
    inds = torch.full((n,), -7, dtype=torch.int64, device="cuda")
    oob = torch.full((n,), -1, dtype=torch.int64, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = _lib.ArbQueryOut(comps.data_ptr(), norms.data_ptr(), grads.data_ptr(), inds.data_ptr(),
                           oob.data_ptr(), cnt.data_ptr())
    prec = _lib.PREC_FP64 if o.precision == "fp64" else _lib.PREC_MIXED
    stream = torch.cuda.current_stream().cuda_stream
    qq = q.clone()
    if entry == "workspace":
        need = int(L.arb_query_sorted_work_bytes(o._g, prec, n))
        ws = torch.empty(need, dtype=torch.uint8, device="cuda")
        rc = L.arb_query_eval_sorted(o._g, prec, use_table, qq.data_ptr(), n, d, 1, out, ws.data_ptr(), need,
                                     status.data_ptr(), stream)
    else:
        rc = L.arb_query_eval_sorted_noalloc(o._g, prec, use_table, qq.data_ptr(), n, d, 1, out,
                                             status.data_ptr(), stream)
    assert rc == _lib.ARB_OK, (entry, rc)
    assert L.arb_status_fetch(status.data_ptr(), stream) == _lib.ARB_OK
    k = int(cnt.item())
    return {"comps": comps.cpu().numpy(), "norms": norms.cpu().numpy(), "grads": grads.cpu().numpy(),
            "inds": inds.cpu().numpy(), "oob": np.sort(oob[:k].cpu().numpy()),
            "q": qq.cpu().numpy()}


def _field(case):
    from arbinterp_gb300 import quadcubic, synth, tricubic
    kind, prec, table = case
    if kind == "both":
        o = tricubic(synth.dipole_field3(n=(40, 36, 44), seed=12).numpy(), "quiet", mode="both", precision=prec)
    elif kind == "scalar":
        o = tricubic(synth.gaussian_field3(n=(38, 41, 35), seed=14).numpy(), "quiet", precision=prec)
    else:
        o = quadcubic(synth.moving_gaussian_field4(n=(14, 13, 15, 11), seed=15).numpy(), "quiet", precision=prec)
    if table:
        o.allCoeffs()
    return o


# 3D 'both' (the 8-lane bin kernel in mixed precision), a 3D scalar field,
# a 4D scalar field and the coefficient-table strategy: each carves the
# shared array differently
CASES = [("both", "fp64", 0), ("both", "mixed", 0), ("both", "mixed", 1), ("scalar", "mixed", 0),
         ("scalar", "fp64", 1), ("quad", "mixed", 0), ("quad", "fp64", 1)]


@pytest.mark.parametrize("case", CASES, ids=["-".join(map(str, c)) for c in CASES])
def test_noalloc_matches_workspace_entry_point_twice(case):
    torch, _lib, L = _setup()
    from arbinterp_gb300 import synth
    o = _field(case)
    d = o._dim
    names = "xyzt"[:d]
    lo = [getattr(o, a + "IntMin") for a in names]
    hi = [getattr(o, a + "IntMax") for a in names]
    h = [getattr(o, "h" + a) for a in names]
    for call, n_in in enumerate((60000, 25000)):     # two calls in a row, different sizes
        q = synth.uniform_queries(lo, hi, n_in, n_in // 100, h, seed=70 + call, device="cuda")
        want = _run(torch, _lib, L, o, q, "workspace", case[2])
        got = _run(torch, _lib, L, o, q, "noalloc", case[2])
        assert np.array_equal(got["inds"], want["inds"])
        assert np.array_equal(got["oob"], want["oob"]) and len(got["oob"]) > 0
        assert np.array_equal(got["q"], want["q"], equal_nan=True)
        for k in ("comps", "norms", "grads"):
            assert np.array_equal(np.isnan(got[k]), np.isnan(want[k])), k
            assert np.array_equal(got[k], want[k], equal_nan=True), k


def test_noalloc_rejects_oversized_calls():
    torch, _lib, L = _setup()
    from arbinterp_gb300 import synth, tricubic
    f = synth.dipole_field3(n=(12, 12, 12), seed=13).numpy()
    o = tricubic(f, "quiet", mode="both")
    limit = 16 << 20
    n = 1
    while int(L.arb_query_sorted_work_bytes(o._g, _lib.PREC_FP64, n)) <= limit:
        n *= 2
    # valid arguments throughout: the size alone is refused, on the host,
    # before any device work (none of these buffers is touched)
    f64 = dict(dtype=torch.float64, device="cuda")
    q = torch.zeros((1, 3), **f64)
    comps, norms, grads = torch.zeros((1, 3), **f64), torch.zeros((1, 1), **f64), torch.zeros((1, 3), **f64)
    out = _lib.ArbQueryOut(comps.data_ptr(), norms.data_ptr(), grads.data_ptr(), None, None, None)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.arb_query_eval_sorted_noalloc(o._g, _lib.PREC_FP64, 0, q.data_ptr(), n, 3, 0, out,
                                         status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.ARB_ERR_CAPACITY
    # and a call with a bad argument is refused as invalid whatever its size
    rc = L.arb_query_eval_sorted_noalloc(o._g, _lib.PREC_FP64, 0, q.data_ptr(), n, 2, 0, out,
                                         status.data_ptr(), torch.cuda.current_stream().cuda_stream)
    assert rc == _lib.ARB_ERR_INVALID
