"""Generate the golden fixtures in this folder from the UNMODIFIED reference.

Run in a container that holds the reference sources (read-only):

    python tests/golden/make_golden.py /path/to/ARBInterp/src/ARBInterp/ARBInterp.py

The reference module is loaded by file path under a private name so it never
shadows the drop-in ``ARBInterp`` package of this repository.  Every case
stores its inputs (field rows, query rows) and the reference's outputs, so the
tests need neither the reference nor this script at run time.
"""
from __future__ import annotations

import contextlib
import importlib.util
import io
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, "..", "..")))

from arbinterp_gb300 import synth  # noqa: E402


def load_reference(path):
    spec = importlib.util.spec_from_file_location("_arb_reference", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def quiet_call(fn, *a, **k):
    with contextlib.redirect_stdout(io.StringIO()):
        return fn(*a, **k)


def run_range(obj, q):
    qq = q.copy()
    out = obj.Query(qq)
    # the reference writes NaN over whole out-of-volume rows in place
    nanrows = np.isnan(qq).all(axis=1)
    assert np.array_equal(qq[~nanrows], q[~nanrows], equal_nan=True)
    res = {"nanrows": nanrows, "inds": np.asarray(obj.queryInds)}
    if isinstance(out, tuple) and len(out) == 3:
        res.update(comps=out[0], norms=out[1], grads=out[2])
    elif isinstance(out, tuple):
        res.update(norms=out[0], grads=out[1])
    else:
        res.update(comps=out)
    return res


def single_points(obj, pts):
    """sQuery results for each point; errors recorded by type name."""
    rows = []
    for p in pts:
        try:
            r = obj.Query(p.copy())
            if isinstance(r, tuple):
                flat = np.concatenate([np.atleast_1d(np.asarray(v, dtype=float)) for v in r])
            else:
                flat = np.atleast_1d(np.asarray(r, dtype=float))
            rows.append(("ok", flat))
        except Exception as e:  # the reference's own error behaviour
            rows.append((type(e).__name__, np.zeros(0)))
    return rows


def pack(prefix, d, store):
    for k, v in d.items():
        store[f"{prefix}{k}"] = np.asarray(v)


def params3(obj):
    return dict(nPos=obj.nPos, h=np.array([obj.hx, obj.hy, obj.hz], dtype=np.float64),
                lo=np.array([obj.xIntMin, obj.yIntMin, obj.zIntMin], dtype=np.float64),
                hi=np.array([obj.xIntMax, obj.yIntMax, obj.zIntMax], dtype=np.float64),
                nc=np.array(obj.nc), basePointInds=obj.basePointInds)


def params4(obj):
    return dict(nPos=np.array([obj.nPosx, obj.nPosy, obj.nPosz, obj.nPost]),
                h=np.array([obj.hx, obj.hy, obj.hz, obj.ht], dtype=np.float64),
                lo=np.array([obj.xIntMin, obj.yIntMin, obj.zIntMin, obj.tIntMin], dtype=np.float64),
                hi=np.array([obj.xIntMax, obj.yIntMax, obj.zIntMax, obj.tIntMax], dtype=np.float64),
                nc=np.array(obj.nc), basePointInds=obj.basePointInds)


def main(ref_path):
    R = load_reference(ref_path)
    out = {}

    # -- the reference's matrices -------------------------------------------
    ex = os.path.join(os.path.dirname(ref_path), "..", "..", "examples")
    out["B3_csv"] = np.loadtxt(os.path.join(ex, "B_Matrix_3D.csv"), delimiter=",")
    out["B4_csv"] = np.loadtxt(os.path.join(ex, "B_Matrix_4D.csv"), delimiter=",")
    f_small = synth.gaussian_field3(n=(5, 5, 5), seed=11).numpy()
    t = quiet_call(R.tricubic, f_small, "quiet")
    out["A3"] = t.A
    f4_small = synth.moving_gaussian_field4(n=(5, 5, 5, 5), seed=12).numpy()
    t4 = quiet_call(R.quadcubic, f4_small, "quiet")
    out["A4"] = t4.A

    # -- 41^3 scalar workload (full grid), 10k queries incl. 1% outside -----
    f0 = synth.gaussian_field3(seed=0).numpy()
    o0 = quiet_call(R.tricubic, f0, "quiet")
    q0 = synth.uniform_queries([o0.xIntMin, o0.yIntMin, o0.zIntMin], [o0.xIntMax, o0.yIntMax, o0.zIntMax],
                               9900, 100, [o0.hx, o0.hy, o0.hz], seed=5).numpy()
    out["c0_U"] = f0[:, 3]
    # rows are meshgrid(indexing='ij') order; the axes rebuild them exactly
    for a in range(3):
        out[f"c0_ax{a}"] = np.unique(f0[:, a])
    out["c0_q"] = q0
    pack("c0_", run_range(o0, q0), out)
    pack("c0_p_", params3(o0), out)
    cells = np.random.default_rng(0).choice(o0.nc, 64, replace=False)
    cells = cells[o0.alphamask[cells, 0] == 1]
    out["c0_alpha_cells"] = cells
    out["c0_alphan"] = o0.alphan[:, cells]

    # -- small vector fields, every mode ------------------------------------
    fv = synth.dipole_field3(n=(9, 10, 11), seed=7).numpy()
    # shuffle the rows: the constructor must sort them
    fv = fv[np.random.default_rng(1).permutation(len(fv))]
    out["vec_field"] = fv
    for tag, kw in [("both", {"mode": "both"}), ("norm", {"mode": "norm"}),
                    ("vector", {"mode": "vector"}), ("default", {}),
                    ("invalid", {"mode": "sideways"})]:
        o = quiet_call(R.tricubic, fv, "quiet", **kw)
        q = synth.uniform_queries([o.xIntMin, o.yIntMin, o.zIntMin], [o.xIntMax, o.yIntMax, o.zIntMax],
                                  1500, 100, [o.hx, o.hy, o.hz], seed=9, ncols=5).numpy()
        out[f"vec_{tag}_q"] = q
        pack(f"vec_{tag}_", run_range(o, q), out)
        if tag == "both":
            pack("vec_p_", params3(o), out)
            out["vec_inputfield"] = o.inputfield
            o2 = quiet_call(R.tricubic, fv, "quiet", **kw)
            o2.allCoeffs()
            out["vec_both_alphax"] = o2.alphax
            out["vec_both_alphan"] = o2.alphan
            out["vec_both_mask"] = o2.alphamask[:, 0]
        if tag == "vector":
            o2 = quiet_call(R.tricubic, fv, "quiet", **kw)
            o2.allCoeffs()
            out["vec_vector_alphay"] = o2.alphay
        pts = np.vstack([q[:6, :3], [[o.xIntMax + o.hx, o.yIntMin, o.zIntMin]]])
        res = single_points(o, pts)
        out[f"vec_{tag}_sp_pts"] = pts
        out[f"vec_{tag}_sp_status"] = np.array([r[0] for r in res])
        out[f"vec_{tag}_sp_vals"] = np.array([np.pad(r[1], (0, 7 - len(r[1])), constant_values=np.nan)
                                              for r in res])

    # -- upper-face aliasing: integer grid so (IntMax-IntMin)/h == nPos ----
    xs = np.arange(7.0)
    ys = np.arange(6.0)
    zs = np.arange(8.0)
    X, Y, Z = np.meshgrid(xs, ys, zs, indexing="ij")
    U = np.sin(0.7 * X) + np.cos(0.4 * Y) * Z + 0.1 * X * Y
    fa = np.stack([X.ravel(), Y.ravel(), Z.ravel(), U.ravel()], 1)
    out["face_field"] = fa
    for tag, fld, kw in [("scalar", fa, {}),
                         ("norm", np.hstack([fa[:, :3], np.stack([U.ravel(), 2 * U.ravel(), -U.ravel()], 1)]),
                          {"mode": "norm"})]:
        o = quiet_call(R.tricubic, fld, "quiet", **kw)
        q = np.array([[5.0, 2.5, 3.25],        # x on the upper face -> aliases to cell (0, iy+1, iz)
                      [5.0, 4.0, 3.5],         # x and y on upper faces
                      [1.0, 1.0, 1.0],         # lower corner
                      [3.3, 1.7, 2.2]])
        pack(f"face_{tag}_", run_range(o, q), out)
        out[f"face_{tag}_q"] = q
        if tag == "norm":
            out["face_norm_vals"] = fld[:, 3:]
        # z on the top face: cell index > nc.  rQuery raises IndexError; Query
        # catches it, retries sQuery on the 2-D array and raises ValueError.
        qe = np.array([[2.5, 2.5, 6.0], [1.5, 1.5, 2.0]])
        for fn in ("Query", "rQuery"):
            try:
                getattr(o, fn)(qe.copy())
                out[f"face_{tag}_err_{fn}"] = np.array("none")
            except Exception as e:
                out[f"face_{tag}_err_{fn}"] = np.array(type(e).__name__)
        out[f"face_{tag}_qerr"] = qe

    # -- float32 scalar field ------------------------------------------------
    f32 = synth.gaussian_field3(n=(14, 13, 12), h=(0.11, 0.07, 0.13), seed=21).numpy().astype(np.float32)
    o = quiet_call(R.tricubic, f32, "quiet")
    q = synth.uniform_queries([float(o.xIntMin), float(o.yIntMin), float(o.zIntMin)],
                              [float(o.xIntMax), float(o.yIntMax), float(o.zIntMax)],
                              2000, 40, [float(o.hx), float(o.hy), float(o.hz)], seed=22).numpy()
    out["f32_field"] = f32
    out["f32_q"] = q
    pack("f32_", run_range(o, q), out)
    pack("f32_p_", params3(o), out)

    # -- 4D ----------------------------------------------------------------
    f4 = synth.moving_gaussian_field4(n=(8, 7, 6, 7), h=(0.2, 0.15, 0.25, 0.1), seed=31).numpy()
    f4 = f4[np.random.default_rng(2).permutation(len(f4))]
    o = quiet_call(R.quadcubic, f4, "quiet")
    q = synth.uniform_queries([o.xIntMin, o.yIntMin, o.zIntMin, o.tIntMin],
                              [o.xIntMax, o.yIntMax, o.zIntMax, o.tIntMax],
                              1500, 60, [o.hx, o.hy, o.hz, o.ht], seed=32).numpy()
    out["q4_field"] = f4
    out["q4_q"] = q
    pack("q4_", run_range(o, q), out)
    pack("q4_p_", params4(o), out)
    out["q4_inputfield"] = o.inputfield
    pts = np.vstack([q[:5, :4], [[o.xIntMin - 1, o.yIntMin, o.zIntMin, o.tIntMin]]])
    res = single_points(o, pts)
    out["q4_sp_pts"] = pts
    out["q4_sp_status"] = np.array([r[0] for r in res])
    out["q4_sp_vals"] = np.array([np.pad(r[1], (0, 7 - len(r[1])), constant_values=np.nan) for r in res])

    g = synth.moving_gaussian_field4(n=(6, 6, 7, 6), h=(0.3, 0.2, 0.25, 0.2), seed=33).numpy()
    rng = np.random.default_rng(3)
    vec = np.stack([g[:, 4], np.sin(g[:, 0]) * g[:, 3], g[:, 4] * 0.5 + g[:, 1]], 1)
    f4v = np.hstack([g[:, :4], vec])
    f4v = f4v[rng.permutation(len(f4v))]
    o = quiet_call(R.quadcubic, f4v, "quiet", mode="both")
    q = synth.uniform_queries([o.xIntMin, o.yIntMin, o.zIntMin, o.tIntMin],
                              [o.xIntMax, o.yIntMax, o.zIntMax, o.tIntMax],
                              800, 30, [o.hx, o.hy, o.hz, o.ht], seed=34).numpy()
    out["q4v_field"] = f4v
    out["q4v_q"] = q
    pack("q4v_", run_range(o, q), out)
    o2 = quiet_call(R.quadcubic, f4v, "quiet", mode="both")
    o2.allCoeffs()
    out["q4v_alphan"] = o2.alphan
    o3 = quiet_call(R.quadcubic, f4v, "quiet", mode="vector")
    pack("q4vv_", run_range(o3, q), out)

    # -- 4D known answer: x*y*z*t is NOT reproduced (row-240 fingerprint) ----
    ax = [np.arange(6) * 0.5, np.arange(6) * 0.5, np.arange(6) * 0.5, np.arange(6) * 0.5]
    X, Y, Z, T = np.meshgrid(*ax, indexing="ij")
    fk = np.stack([X.ravel(), Y.ravel(), Z.ravel(), T.ravel(), (X * Y * Z * T).ravel()], 1)
    o = quiet_call(R.quadcubic, fk, "quiet")
    qk = np.array([[1.1, 1.3, 0.7, 1.9], [0.6, 0.6, 0.6, 0.6], [1.75, 1.2, 1.6, 0.9]])
    out["kat4_q"] = qk
    pack("kat4_", run_range(o, qk), out)

    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    sz = os.path.getsize(os.path.join(HERE, "golden.npz"))
    print(f"wrote golden.npz ({sz / 1e6:.2f} MB, {len(out)} arrays)")


def ref_index(q, lo, hi, h, npos):
    """The reference's flat cell index of range-query rows (rQuery3,
    ARBInterp.py:463-485; 4D rQuery2, ARBInterp.py:1138-1160), computed with the
    same float64 operations (out-of-volume rows NaN), so candidate rows that
    would make it raise IndexError (index > nc) can be dropped before the
    reference runs."""
    q = q.copy()
    d = len(lo)
    for a in range(d):
        q[(q[:, a] < lo[a]) | (q[:, a] > hi[a])] = np.nan
    idx = np.zeros(len(q))
    stride = 1.0
    for a in range(d):
        ia = np.floor((q[:, a] - lo[a]) / h[a])
        idx = idx + ia * stride
        stride = stride * npos[a]
    return idx


def face_rows(rng, axes, lo, hi, h, npos, nc, n_faces, n_upper, n_nan):
    """Special query rows: coordinates exactly on grid planes (cell faces,
    IntMin and IntMax included), rows on each upper face (x = IntMax aliases
    to the next row of cells, ARBInterp.py:481-483), rows on the last axis'
    upper face inside the first cell column (index == nc: the sentinel
    column), and rows with one NaN coordinate."""
    d = len(lo)
    rows = []
    base = lambda m: lo + (hi - lo) * rng.random((m, d))  # noqa: E731
    q = base(n_faces)
    for r in q:
        for a in rng.choice(d, rng.integers(1, d + 1), replace=False):
            r[a] = axes[a][rng.integers(1, len(axes[a]) - 1)]
    rows.append(q)
    for a in range(d - 1):
        q = base(n_upper)
        q[:, a] = hi[a]
        rows.append(q)
    q = base(n_upper)
    q[:, 0] = hi[0]
    q[:, 1] = hi[1]
    rows.append(q)
    q = lo + rng.random((n_upper // 4, d)) * h * 0.999
    q[:, d - 1] = hi[d - 1]
    rows.append(q)
    q = base(n_nan)
    q[np.arange(n_nan), rng.integers(0, d, n_nan)] = np.nan
    rows.append(q)
    q = np.vstack(rows)
    idx = ref_index(q, lo, hi, h, npos)
    keep = ~(idx > nc)
    return q[keep]


def main_scale(ref_path):
    """Reduced-size versions of the 256^3 'both' workload and the 4D
    64^3 x 32 scalar workload, at sizes where the binned query path runs
    (5e4 queries, above the default sort threshold), written to
    golden_scale.npz."""
    R = load_reference(ref_path)
    out = {}
    rng = np.random.default_rng(77)

    # -- 48^3 dipole field, 'both' / 'norm' / 'vector' -----------------------
    n = (48, 48, 48)
    f = synth.dipole_field3(n=n, seed=1).numpy()
    axes = [np.unique(f[:, a]) for a in range(3)]
    out["c1_B"] = f[:, 3:]
    for a in range(3):
        out[f"c1_ax{a}"] = axes[a]
    ob = quiet_call(R.tricubic, f, "quiet", mode="both")
    lo = np.array([ob.xIntMin, ob.yIntMin, ob.zIntMin])
    hi = np.array([ob.xIntMax, ob.yIntMax, ob.zIntMax])
    h = np.array([ob.hx, ob.hy, ob.hz])
    q = synth.uniform_queries(lo, hi, 49000, 500, h, seed=41).numpy()
    special = face_rows(rng, axes, lo, hi, h, ob.nPos, ob.nc, 300, 60, 20)
    q[rng.choice(len(q), len(special), replace=False)] = special
    assert not (ref_index(q, lo, hi, h, ob.nPos) > ob.nc).any()
    out["c1_q"] = q
    res = run_range(ob, q)
    pack("c1_both_", res, out)
    out["c1_both_inds"] = res["inds"].astype(np.int32)
    pack("c1_p_", params3(ob), out)
    out["c1_p_basePointInds"] = ob.basePointInds.astype(np.int32)
    on = quiet_call(R.tricubic, f, "quiet", mode="norm")
    rn = run_range(on, q)
    # rQuery2 evaluates alphan exactly as rQuery3 does: the same bits
    assert np.array_equal(rn["norms"], res["norms"], equal_nan=True)
    assert np.array_equal(rn["grads"], res["grads"], equal_nan=True)
    ov = quiet_call(R.tricubic, f, "quiet", mode="vector")
    rv = run_range(ov, q)
    out["c1_vector_comps"] = rv["comps"]
    assert np.array_equal(rv["inds"], res["inds"])
    cells = [0, 1, ob.nPos[0] - 1, ob.nPos[0] * (ob.nPos[1] - 1), ob.nPos[0] * ob.nPos[1] - 1,
             ob.nc - ob.nPos[0] * ob.nPos[1], ob.nc - ob.nPos[0], ob.nc - 1]
    cells += list(rng.choice(ob.nc, 12, replace=False))
    out["c1_nb_cells"] = np.array(cells)
    out["c1_nb_inds"] = np.array([ob.neighbourInd(ob.basePointInds[c]) for c in cells])

    # -- 16^3 x 12 moving-Gaussian scalar field (4D) --------------------------
    n4 = (16, 16, 16, 12)
    f4 = synth.moving_gaussian_field4(n=n4, seed=2).numpy()
    axes4 = [np.unique(f4[:, a]) for a in range(4)]
    out["c2_U"] = f4[:, 4]
    for a in range(4):
        out[f"c2_ax{a}"] = axes4[a]
    o4 = quiet_call(R.quadcubic, f4, "quiet")
    lo4 = np.array([o4.xIntMin, o4.yIntMin, o4.zIntMin, o4.tIntMin])
    hi4 = np.array([o4.xIntMax, o4.yIntMax, o4.zIntMax, o4.tIntMax])
    h4 = np.array([o4.hx, o4.hy, o4.hz, o4.ht])
    np4 = np.array([o4.nPosx - 3, o4.nPosy - 3, o4.nPosz - 3, o4.nPost - 3])
    q4 = synth.uniform_queries(lo4, hi4, 49000, 500, h4, seed=42).numpy()
    special = face_rows(rng, axes4, lo4, hi4, h4, np4, o4.nc, 300, 60, 20)
    q4[rng.choice(len(q4), len(special), replace=False)] = special
    assert not (ref_index(q4, lo4, hi4, h4, np4) > o4.nc).any()
    out["c2_q"] = q4
    r4 = run_range(o4, q4)
    pack("c2_", r4, out)
    out["c2_inds"] = r4["inds"].astype(np.int32)
    pack("c2_p_", params4(o4), out)
    del out["c2_p_basePointInds"]
    cells = [0, 1, np4[0] - 1, o4.nc - 1, o4.nc - np4[0], o4.nc - np4[0] * np4[1] * np4[2]]
    cells += list(rng.choice(o4.nc, 10, replace=False))
    out["c2_nb_cells"] = np.array(cells)
    out["c2_nb_inds"] = np.array([o4.neighbourInd(o4.basePointInds[c]) for c in cells])

    path = os.path.join(HERE, "golden_scale.npz")
    np.savez_compressed(path, **out)
    print(f"wrote golden_scale.npz ({os.path.getsize(path) / 1e6:.2f} MB, {len(out)} arrays)")


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    path = args[0] if args else os.path.join(os.sep, "root", "reference", "src", "ARBInterp", "ARBInterp.py")
    if "--scale" in sys.argv:
        main_scale(path)
    else:
        main(path)
