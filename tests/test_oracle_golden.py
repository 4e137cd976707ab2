"""Pin the CPU oracle to the reference: B-matrix CSV fixtures, the reference's
own A matrices, and golden outputs generated from the unmodified reference."""
import os

import numpy as np
import pytest

from conftest import c0_field, normwise
from oracle import arb_oracle as O

CSV_DIR = os.path.join(os.path.dirname(__file__), "golden")


def test_B3_matches_reference_formula_and_A3_is_kron(golden):
    B = O.build_B3()
    A = O.build_A3()
    assert np.array_equal(A, golden["A3"])
    A1 = O.catmull_rom_A1()
    assert np.array_equal(A, np.kron(np.kron(A1, A1), A1))
    # B is integral with small entries; inv(B) integral in [-27, 27]
    Bi = np.linalg.inv(B)
    assert np.abs(Bi - np.round(Bi)).max() == 0 and np.abs(Bi).max() == 27


def test_A4_exact(golden):
    A4 = O.build_A4()
    assert np.array_equal(A4, golden["A4"])
    # correct-math D would give the Kronecker product; the bug makes it differ
    A1 = O.catmull_rom_A1()
    K4 = np.kron(np.kron(np.kron(A1, A1), A1), A1)
    assert np.abs(A4 - K4).max() == 0.5
    D = O.build_D4(True)
    assert not D[240].any()


def test_B_matrices_equal_reference_csv_fixtures(golden):
    # examples/B_Matrix_3D.csv and examples/B_Matrix_4D.csv, read by make_golden.py
    assert np.array_equal(O.build_B3(), golden["B3_csv"])
    assert np.array_equal(O.build_B4(), golden["B4_csv"])


def _check_range(o, g, prefix, q, tol=1e-13):
    qq = q.copy()
    r = o.query(qq)
    assert np.array_equal(np.isnan(qq).all(axis=1), g[prefix + "nanrows"])
    assert np.array_equal(r["inds"], g[prefix + "inds"])
    for k in ("comps", "norms", "grads"):
        if prefix + k in g:
            ref = g[prefix + k]
            assert np.array_equal(np.isnan(r[k]), np.isnan(ref)), k
            assert (normwise(r[k], ref) <= tol).all(), (k, normwise(r[k], ref))


def test_c0_scalar(golden):
    g = golden
    o = O.OracleTricubic(c0_field(g))
    assert np.array_equal(o.nPos, g["c0_p_nPos"]) and o.nc == g["c0_p_nc"]
    assert np.array_equal(np.array(o.h), g["c0_p_h"])
    assert np.array_equal(np.array(o.lo), g["c0_p_lo"]) and np.array_equal(np.array(o.hi), g["c0_p_hi"])
    assert np.array_equal(o.basePointInds, g["c0_p_basePointInds"])
    _check_range(o, g, "c0_", g["c0_q"])
    cells = g["c0_alpha_cells"]
    assert normwise(o.alpha["n"][cells].T.ravel()[:, None], g["c0_alphan"].ravel()[:, None]).max() < 1e-13


@pytest.mark.parametrize("tag,mode", [("both", "both"), ("norm", "norm"), ("vector", "vector"),
                                      ("default", None), ("invalid", "sideways")])
def test_vector_modes(golden, tag, mode):
    g = golden
    o = O.OracleTricubic(g["vec_field"], mode=mode)
    _check_range(o, g, f"vec_{tag}_", g[f"vec_{tag}_q"])
    if tag == "both":
        assert np.array_equal(o.inputfield, g["vec_inputfield"])
        o.all_coeffs()
        for k, key in (("x", "vec_both_alphax"), ("n", "vec_both_alphan")):
            ref = g[key]
            mine = o.alpha_matrix(k)
            assert mine.shape == ref.shape
            assert np.array_equal(np.isnan(mine), np.isnan(ref))
            m = np.isfinite(ref)
            assert np.abs(mine[m] - ref[m]).max() <= 1e-13 * np.abs(ref[m]).max()
    if tag == "vector":
        o.all_coeffs()
        ref = g["vec_vector_alphay"]
        mine = o.alpha_matrix("y")
        assert mine.shape == ref.shape and np.isnan(mine[:, -1]).all() and not mine[:, -2].any()


@pytest.mark.parametrize("tag,mode", [("scalar", None), ("norm", "norm")])
def test_upper_face_aliasing(golden, tag, mode):
    g = golden
    fld = g["face_field"] if tag == "scalar" else np.hstack([g["face_field"][:, :3], g["face_norm_vals"]])
    o = O.OracleTricubic(fld, mode=mode)
    _check_range(o, g, f"face_{tag}_", g[f"face_{tag}_q"])
    assert str(g[f"face_{tag}_err_rQuery"]) == "IndexError"
    with pytest.raises(IndexError):
        o.query(g[f"face_{tag}_qerr"].copy())


def test_float32_field(golden):
    g = golden
    o = O.OracleTricubic(g["f32_field"])
    assert np.array_equal(np.array(o.h, dtype=np.float64), g["f32_p_h"])
    _check_range(o, g, "f32_", g["f32_q"])


def test_quadcubic_scalar(golden):
    g = golden
    o = O.OracleQuadcubic(g["q4_field"])
    assert np.array_equal(o.inputfield, g["q4_inputfield"])
    assert np.array_equal(o.basePointInds, g["q4_p_basePointInds"])
    _check_range(o, g, "q4_", g["q4_q"])


def test_quadcubic_vector(golden):
    g = golden
    o = O.OracleQuadcubic(g["q4v_field"], mode="both")
    _check_range(o, g, "q4v_", g["q4v_q"])
    o.all_coeffs()
    ref = g["q4v_alphan"]
    mine = o.alpha_matrix("n")
    m = np.isfinite(ref)
    assert np.array_equal(np.isnan(mine), np.isnan(ref))
    assert np.abs(mine[m] - ref[m]).max() <= 1e-13 * np.abs(ref[m]).max()
    o3 = O.OracleQuadcubic(g["q4v_field"], mode="vector")
    _check_range(o3, g, "q4vv_", g["q4v_q"])


def test_quadcubic_kat_fingerprint(golden):
    g = golden
    ax = [np.arange(6) * 0.5] * 4
    X, Y, Z, T = np.meshgrid(*ax, indexing="ij")
    fk = np.stack([X.ravel(), Y.ravel(), Z.ravel(), T.ravel(), (X * Y * Z * T).ravel()], 1)
    o = O.OracleQuadcubic(fk)
    q = g["kat4_q"].copy()
    r = o.query(q)
    assert np.allclose(r["norms"], g["kat4_norms"], rtol=0, atol=1e-13)
    exact = np.prod(g["kat4_q"], axis=1)
    err = np.abs(r["norms"][:, 0] - exact).max()
    assert err > 1e-9     # a correct quadcubic reproduces x*y*z*t; the row-240 D bug does not


def test_scale_both_norm_vector(golden_scale):
    """48^3 dipole field, 49,500 queries (faces, upper faces, sentinel rows,
    NaN coordinates): the oracle against the reference in every vector mode."""
    from conftest import c1s_field
    g = golden_scale
    f = c1s_field(g)
    o = O.OracleTricubic(f, mode="both")
    assert np.array_equal(o.nPos, g["c1_p_nPos"]) and o.nc == g["c1_p_nc"]
    assert np.array_equal(np.array(o.h), g["c1_p_h"])
    assert np.array_equal(o.basePointInds, g["c1_p_basePointInds"])
    _check_range(o, g, "c1_both_", g["c1_q"])
    r = O.OracleTricubic(f, mode="norm").query(g["c1_q"].copy())
    for k in ("norms", "grads"):
        assert (normwise(r[k], g["c1_both_" + k]) <= 1e-13).all()
    r = O.OracleTricubic(f, mode="vector").query(g["c1_q"].copy())
    ref = g["c1_vector_comps"]
    assert np.array_equal(np.isnan(r["comps"]), np.isnan(ref))
    assert (normwise(r["comps"], ref) <= 1e-13).all()


def test_scale_quadcubic(golden_scale):
    from conftest import c2s_field
    g = golden_scale
    o = O.OracleQuadcubic(c2s_field(g))
    assert o.nc == g["c2_p_nc"]
    # 256-term sums in another order than the reference's (ARBInterp.py:1180-1188):
    # gradients agree to ~2e-13 normwise on this grid, well inside the 1e-12 bar
    _check_range(o, g, "c2_", g["c2_q"], tol=5e-13)
