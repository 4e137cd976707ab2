"""GPU parity at the scale where the bin-grouped query path runs.

The fixtures come from the unmodified reference (tests/golden/make_golden.py
--scale): a 48^3 dipole vector field in 'both', 'norm' and 'vector' mode and a
16^3 x 12 4D scalar field, 49,500 queries each, including 1% out of volume,
rows exactly on cell faces, rows on the upper faces (the reference's aliasing
into the next row or plane of cells, ARBInterp.py:481-483), rows whose index
is the sentinel column nc, and rows with a NaN coordinate.

Every case runs bin-grouped (sort_threshold=0: bin count / scan / place, then
the shared-memory bin kernels or the table kernel) and ungrouped, in float64
and mixed precision, evaluating on the fly and from a full coefficient table.
Bars: cell indices, NaN masks and the in-place NaN rows bit-exact; values
<= 1e-12 normwise (max|got - ref| / max|ref| per column) in float64 and
<= 1e-6 in mixed precision."""
import numpy as np
import pytest

from conftest import c1s_field, c2s_field, normwise

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed": 1e-6}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from arbinterp_gb300 import _lib
    _lib.lib()


def _check(got, ref, tol, what):
    assert got.shape == ref.shape, what
    assert np.array_equal(np.isnan(got), np.isnan(ref)), what
    err = normwise(got, ref)
    assert (err <= tol).all(), (what, err)


@pytest.mark.parametrize("sort_threshold", [0, 1 << 30])
@pytest.mark.parametrize("strategy", ["otf", "table"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("mode", ["both", "norm", "vector"])
def test_tricubic48_modes(golden_scale, mode, prec, strategy, sort_threshold):
    from arbinterp_gb300 import tricubic
    g = golden_scale
    o = tricubic(c1s_field(g), "quiet", mode=mode, precision=prec, strategy=strategy,
                 sort_threshold=sort_threshold)
    assert np.array_equal(o.nPos, g["c1_p_nPos"]) and o.nc == int(g["c1_p_nc"])
    assert np.array_equal(np.array([o.xIntMax, o.yIntMax, o.zIntMax]), g["c1_p_hi"])
    q = g["c1_q"].copy()
    res = o.Query(q)
    assert np.array_equal(o.queryInds, g["c1_both_inds"].astype(np.int64))
    assert np.array_equal(np.isnan(q).all(axis=1), g["c1_both_nanrows"])
    # rows that are not out of volume keep their coordinates (NaN ones too)
    keep = ~g["c1_both_nanrows"]
    assert np.array_equal(q[keep], g["c1_q"][keep], equal_nan=True)
    if mode == "both":
        for k, got in zip(("comps", "norms", "grads"), res):
            _check(got, g["c1_both_" + k], TOL[prec], k)
    elif mode == "norm":
        for k, got in zip(("norms", "grads"), res):
            _check(got, g["c1_both_" + k], TOL[prec], k)
    else:
        _check(res, g["c1_vector_comps"], TOL[prec], "comps")


@pytest.mark.parametrize("sort_threshold", [0, 1 << 30])
@pytest.mark.parametrize("strategy", ["otf", "table"])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_quadcubic16_scalar(golden_scale, prec, strategy, sort_threshold):
    from arbinterp_gb300 import quadcubic
    g = golden_scale
    o = quadcubic(c2s_field(g), "quiet", precision=prec, strategy=strategy, sort_threshold=sort_threshold)
    assert o.nc == int(g["c2_p_nc"])
    q = g["c2_q"].copy()
    norms, grads = o.Query(q)
    assert np.array_equal(o.queryInds, g["c2_inds"].astype(np.int64))
    assert np.array_equal(np.isnan(q).all(axis=1), g["c2_nanrows"])
    _check(norms, g["c2_norms"], TOL[prec], "norms")
    _check(grads, g["c2_grads"], TOL[prec], "grads")


def test_neighbour_indices_against_reference(golden_scale):
    """neighbourInd of the first and last cells, the last cell of a row and
    of a plane, the first cell of the last plane and random cells (3D,
    ARBInterp.py:605-621; 4D, ARBInterp.py:1357-1381)."""
    from arbinterp_gb300 import quadcubic, tricubic
    g = golden_scale
    o = tricubic(c1s_field(g), "quiet", mode="both")
    for c, want in zip(g["c1_nb_cells"], g["c1_nb_inds"]):
        got = o.neighbourInd(o.basePointInds[c])
        assert got.dtype == want.dtype and np.array_equal(got, want), c
    o4 = quadcubic(c2s_field(g), "quiet")
    for c, want in zip(g["c2_nb_cells"], g["c2_nb_inds"]):
        got = o4.neighbourInd(o4.basePointInds[c])
        assert got.dtype == want.dtype and np.array_equal(got, want), c
