"""GPU parity: the CUDA path through the C ABI against the reference's golden
outputs (small cases) and the CPU oracle (seeded synthetic fields).

Bars: cell indices, NaN masks and the in-place NaN rows of the caller's query
array bit-exact; values <= 1e-12 normwise in float64, <= 1e-6 in mixed
precision (normwise = max|got - ref| / max|ref| per output column)."""
import numpy as np
import pytest

from conftest import c0_field, normwise

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "mixed": 1e-6}


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from arbinterp_gb300 import _lib
    _lib.lib()


def _mods():
    from arbinterp_gb300 import tricubic, quadcubic
    return tricubic, quadcubic


def _check(res, g, prefix, qafter, inds, tol):
    assert np.array_equal(inds, g[prefix + "inds"])
    assert np.array_equal(np.isnan(qafter).all(axis=1), g[prefix + "nanrows"])
    names = [k for k in ("comps", "norms", "grads") if prefix + k in g]
    if len(names) == 1:
        res = (res,)
    for k, got in zip(names, res):
        ref = g[prefix + k]
        assert got.shape == ref.shape, k
        assert np.array_equal(np.isnan(got), np.isnan(ref)), k
        err = normwise(got, ref)
        assert (err <= tol).all(), (k, err)


@pytest.mark.parametrize("sort_threshold", [0, 1 << 30])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("strategy", ["otf", "table"])
def test_c0_scalar_golden(golden, prec, strategy, sort_threshold):
    tricubic, _ = _mods()
    g = golden
    o = tricubic(c0_field(g), "quiet", precision=prec, strategy=strategy, sort_threshold=sort_threshold)
    assert np.array_equal(o.nPos, g["c0_p_nPos"]) and o.nc == int(g["c0_p_nc"])
    assert np.array_equal(np.array([o.hx, o.hy, o.hz]), g["c0_p_h"])
    assert np.array_equal(np.array([o.xIntMin, o.yIntMin, o.zIntMin]), g["c0_p_lo"])
    assert np.array_equal(np.array([o.xIntMax, o.yIntMax, o.zIntMax]), g["c0_p_hi"])
    assert np.array_equal(o.basePointInds, g["c0_p_basePointInds"])
    q = g["c0_q"].copy()
    res = o.Query(q)
    _check(res, g, "c0_", q, o.queryInds, TOL[prec])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("tag,mode", [("both", "both"), ("norm", "norm"), ("vector", "vector"),
                                      ("default", None), ("invalid", "sideways")])
def test_vector_modes_golden(golden, prec, tag, mode):
    tricubic, _ = _mods()
    g = golden
    kw = {} if mode is None else {"mode": mode}
    o = tricubic(g["vec_field"], "quiet", precision=prec, **kw)
    q = g[f"vec_{tag}_q"].copy()
    res = o.Query(q)
    _check(res, g, f"vec_{tag}_", q, o.queryInds, TOL[prec])
    # single points: statuses and values as the reference returned them
    pts = g[f"vec_{tag}_sp_pts"]
    for p, st, vals in zip(pts, g[f"vec_{tag}_sp_status"], g[f"vec_{tag}_sp_vals"]):
        if st == "ok":
            r = o.Query(p.copy())
            flat = np.concatenate([np.atleast_1d(np.asarray(v, float)) for v in (r if isinstance(r, tuple) else (r,))])
            want = vals[:len(flat)]
            assert np.array_equal(np.isnan(flat), np.isnan(want))
            m = np.isfinite(want)
            if m.any():
                assert np.abs(flat[m] - want[m]).max() <= 10 * TOL[prec] * max(1.0, np.abs(want[m]).max())
        else:
            # out of volume: bare NaN; in norm/both mode the reference's
            # tuple-unpack of that NaN raises TypeError
            r = o.sQuery(p.copy())
            assert isinstance(r, float) and np.isnan(r)


def test_both_coefficients_and_attributes(golden):
    tricubic, _ = _mods()
    g = golden
    o = tricubic(g["vec_field"], "quiet", mode="both")
    assert np.array_equal(o.inputfield, g["vec_inputfield"])
    o.allCoeffs()
    for name in ("alphax", "alphan"):
        ref = g[f"vec_both_{name}"]
        mine = getattr(o, name)
        assert mine.shape == ref.shape
        assert np.array_equal(np.isnan(mine), np.isnan(ref))
        m = np.isfinite(ref)
        assert np.abs(mine[m] - ref[m]).max() <= 1e-12 * np.abs(ref[m]).max()
    assert np.array_equal(o.alphamask[:, 0], g["vec_both_mask"])
    ov = tricubic(g["vec_field"], "quiet", mode="vector")
    ov.allCoeffs()
    ref = g["vec_vector_alphay"]
    mine = ov.alphay
    assert mine.shape == ref.shape and np.array_equal(np.isnan(mine), np.isnan(ref))
    m = np.isfinite(ref)
    assert np.abs(mine[m] - ref[m]).max() <= 1e-12 * np.abs(ref[m]).max()


@pytest.mark.parametrize("sort_threshold", [0, 1 << 30])
@pytest.mark.parametrize("strategy", ["otf", "table"])
@pytest.mark.parametrize("tag,mode", [("scalar", None), ("norm", "norm")])
def test_upper_face_aliasing_and_errors(golden, strategy, tag, mode, sort_threshold):
    tricubic, _ = _mods()
    g = golden
    fld = g["face_field"] if tag == "scalar" else np.hstack([g["face_field"][:, :3], g["face_norm_vals"]])
    kw = {} if mode is None else {"mode": mode}
    o = tricubic(fld, "quiet", strategy=strategy, sort_threshold=sort_threshold, **kw)
    q = g[f"face_{tag}_q"].copy()
    res = o.Query(q)
    _check(res, g, f"face_{tag}_", q, o.queryInds, 1e-12)
    assert str(g[f"face_{tag}_err_rQuery"]) == "IndexError"
    assert str(g[f"face_{tag}_err_Query"]) == "ValueError"
    with pytest.raises(IndexError):
        o.rQuery(g[f"face_{tag}_qerr"].copy())
    with pytest.raises(ValueError):
        o.Query(g[f"face_{tag}_qerr"].copy())


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_float32_field_golden(golden, prec):
    tricubic, _ = _mods()
    g = golden
    o = tricubic(g["f32_field"], "quiet", precision=prec)
    assert o.hx.dtype == np.float32
    assert np.array_equal(np.array([o.hx, o.hy, o.hz], dtype=np.float64), g["f32_p_h"])
    q = g["f32_q"].copy()
    res = o.Query(q)
    _check(res, g, "f32_", q, o.queryInds, TOL[prec])


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("strategy", ["otf", "table"])
def test_quadcubic_golden(golden, prec, strategy):
    _, quadcubic = _mods()
    g = golden
    o = quadcubic(g["q4_field"], "quiet", precision=prec, strategy=strategy, sort_threshold=0)
    assert np.array_equal(o.inputfield, g["q4_inputfield"])
    assert np.array_equal(o.basePointInds, g["q4_p_basePointInds"])
    q = g["q4_q"].copy()
    res = o.Query(q)
    _check(res, g, "q4_", q, o.queryInds, TOL[prec])
    o2 = quadcubic(g["q4v_field"], "quiet", mode="both", precision=prec, strategy=strategy)
    q = g["q4v_q"].copy()
    _check(o2.Query(q), g, "q4v_", q, o2.queryInds, TOL[prec])
    o3 = quadcubic(g["q4v_field"], "quiet", mode="vector", precision=prec, strategy=strategy)
    q = g["q4v_q"].copy()
    _check(o3.Query(q), g, "q4vv_", q, o3.queryInds, TOL[prec])


def test_quadcubic_alpha_and_kat(golden):
    _, quadcubic = _mods()
    g = golden
    o = quadcubic(g["q4v_field"], "quiet", mode="both")
    o.allCoeffs()
    ref = g["q4v_alphan"]
    mine = o.alphan
    assert np.array_equal(np.isnan(mine), np.isnan(ref))
    m = np.isfinite(ref)
    assert np.abs(mine[m] - ref[m]).max() <= 1e-12 * np.abs(ref[m]).max()
    ax = [np.arange(6) * 0.5] * 4
    X, Y, Z, T = np.meshgrid(*ax, indexing="ij")
    fk = np.stack([X.ravel(), Y.ravel(), Z.ravel(), T.ravel(), (X * Y * Z * T).ravel()], 1)
    n, _ = quadcubic(fk, "quiet").Query(g["kat4_q"].copy())
    assert np.abs(n - g["kat4_norms"]).max() <= 1e-12


def test_quadcubic_single_points(golden):
    _, quadcubic = _mods()
    g = golden
    o = quadcubic(g["q4_field"], "quiet")
    for p, st, vals in zip(g["q4_sp_pts"], g["q4_sp_status"], g["q4_sp_vals"]):
        if st == "ok":
            nv, gv = o.Query(p.copy())
            flat = np.concatenate([[nv], gv])
            assert np.abs(flat - vals[:5]).max() <= 1e-12 * max(1, np.abs(vals[:5]).max())
        else:
            assert np.isnan(o.sQuery(p.copy()))


def test_irregular_grid_rejected():
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth
    f = synth.gaussian_field3(n=(6, 6, 6), seed=1).numpy()
    with pytest.raises(ValueError):
        tricubic(f[:-1], "quiet")          # a missing point
    f2 = f.copy()
    f2[5, 0] += 1e-9                        # a coordinate off its axis
    with pytest.raises(ValueError):
        tricubic(f2, "quiet")
    with pytest.raises(SystemExit):
        tricubic(np.hstack([f, f[:, 3:]]), "quiet")      # N x 5


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_random_both_vs_oracle(prec):
    """64^3 dipole field, 'both' mode, 2e5 queries against the CPU oracle."""
    import torch
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth
    from oracle.arb_oracle import OracleTricubic
    f = synth.dipole_field3(n=(40, 48, 44), seed=3).numpy()
    ref = OracleTricubic(f, mode="both")
    q = synth.uniform_queries(ref.lo, ref.hi, 200000, 2000, ref.h, seed=4).numpy()
    want = ref.query(q.copy())
    for strategy in ("otf", "table"):
        o = tricubic(f, "quiet", mode="both", precision=prec, strategy=strategy)
        qq = q.copy()
        comps, norms, grads = o.Query(qq)
        assert np.array_equal(o.queryInds, want["inds"])
        for got, k in ((comps, "comps"), (norms, "norms"), (grads, "grads")):
            assert np.array_equal(np.isnan(got), np.isnan(want[k]))
            assert (normwise(got, want[k]) <= TOL[prec]).all(), (strategy, k, normwise(got, want[k]))
        # device-tensor queries: outputs stay on the device, OOB rows NaN'd in place
        qd = torch.from_numpy(q.copy()).cuda()
        c2, n2, g2 = o.Query(qd)
        assert np.array_equal(torch.isnan(qd).all(1).cpu().numpy(), np.isnan(qq).all(1))
        assert np.array_equal(c2.cpu().numpy(), comps, equal_nan=True)


def test_fd_planes_match_D_matrix():
    """arb_fd_planes equals the reference's D-matrix stencils at cell corners."""
    import torch
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth, _lib
    from oracle import arb_oracle as O
    f = synth.gaussian_field3(n=(7, 8, 9), seed=2).numpy()
    o = tricubic(f, "quiet")
    npts = o._npts
    planes = torch.empty(8 * npts, dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().arb_fd_planes(o._g, planes.data_ptr(), torch.cuda.current_stream().cuda_stream),
               "arb_fd_planes")
    P = planes.view(8, npts).cpu().numpy()
    ref = O.OracleTricubic(f)
    D = O.build_D3()
    vals = ref.fields["n"]
    for cell in (0, 5, ref.nc - 1):
        block = vals[ref.basePointInds[cell] + ref.block_offsets]
        b = D @ block                       # b[8r + k]: kind r at corner k
        for k in range(8):
            p = ref.basePointInds[cell] + (k & 1) + ref.nx * ((k >> 1) & 1) + ref.nx * ref.ny * (k >> 2)
            assert np.allclose(P[:, p], b[k::8], rtol=0, atol=1e-13)


@pytest.mark.parametrize("mode", ["both", "vector", "norm"])
def test_tensor_core_table_matches_fp64(mode):
    """Mixed-precision table (FP16 fixed-point tcgen05 GEMM, float32 rows)
    against the float64 table; single-cell solves (partial tiles, cell
    offsets) included."""
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth
    f = synth.dipole_field3(n=(23, 19, 21), seed=8).numpy()
    o64 = tricubic(f, "quiet", mode=mode)
    o64.allCoeffs()
    omx = tricubic(f, "quiet", mode=mode, precision="mixed")
    omx.allCoeffs()
    names = {"both": ("alphax", "alphay", "alphaz", "alphan"), "vector": ("alphax", "alphay", "alphaz"),
             "norm": ("alphan",)}[mode]
    ex = np.arange(64) & 3
    for name in names:
        a64 = getattr(o64, name)[:, :o64.nc]
        amx = getattr(omx, name)[:, :o64.nc]
        d = np.abs(amx - a64)
        # monomials are <= 1 on the unit cell: sum_i |d alpha_i| bounds the
        # value error, sum_i ex_i |d alpha_i| the (cell-unit) x-gradient error
        val_err = d.sum(axis=0).max() / np.abs(a64[0]).max()
        grad_err = (ex[:, None] * d).sum(axis=0).max() / (ex[:, None] * np.abs(a64)).sum(axis=0).max()
        # triangle bounds over the 64 float32-rounded coefficients (float32
        # deltas, vector components without a lo word): ~1.5e-5 on this
        # coarse, fast-varying grid even for exactly computed coefficients;
        # the GEMM itself adds no accumulation error (next test)
        assert val_err <= 3e-5 and grad_err <= 3e-5, (name, val_err, grad_err)
    one = tricubic(f, "quiet", mode=mode, precision="mixed")
    for cell in (0, 7, one.nc - 1):
        one.calcCoefficients(cell)
    a = getattr(one, names[0])
    ref = getattr(o64, names[0])
    for cell in (0, 7, one.nc - 1):
        assert np.abs(a[:, cell] - ref[:, cell]).max() <= 1e-6 * np.abs(ref[:, :o64.nc]).max()
    assert not a[:, 3].any()      # unsolved cells stay zero


@pytest.mark.parametrize("shape", [(23, 19, 21), (136, 11, 9)])
@pytest.mark.parametrize("mode", ["both", "vector", "norm", None])
def test_tensor_core_table_exact_from_deltas(mode, shape):
    """The tcgen05 solve adds no accumulation error: every float32
    coefficient equals alpha = A d computed exactly from the kernel's float32
    deltas d = (hi - hi_ref) + (lo - lo_ref), up to its own float32 rounding
    and the fixed-point truncation of d (2^-33 of the row's power-of-two
    scale, times the largest row abs-sum 216 of A).  Coarse, fast-varying
    dipole field; scalar field too.  The 23-point x axis takes the gather
    kernel (coef3_tc); the 136-point one (a multiple of 4) the warp-
    specialised TMA kernel, with full and partial tiles for every field
    count (133 cells per x-row: 4 x 32 + 5, 3 x 42 + 7, 128 + 5)."""
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth
    from oracle.arb_oracle import OracleTricubic
    f = synth.dipole_field3(n=shape, seed=8).numpy()
    if mode is None:
        f = np.hstack([f[:, :3], f[:, 3:4] * f[:, 4:5] + 3.0])
    kw = {} if mode is None else {"mode": mode}
    omx = tricubic(f, "quiet", precision="mixed", **kw)
    omx.allCoeffs()
    o = OracleTricubic(f, **kw)
    blocks = o.basePointInds[:, None] + o.block_offsets[None, :]
    corner = 1 + 4 + 16
    for key in o.fields:
        v = o.fields[key]
        hi = v.astype(np.float32)
        lo = (v - hi).astype(np.float32) if key == "n" else np.zeros_like(hi)
        rhi, rlo = hi[blocks[:, corner]], lo[blocks[:, corner]]
        d = (hi[blocks] - rhi[:, None]) + (lo[blocks] - rlo[:, None])      # float32, as the kernel
        want = d.astype(np.float64) @ o.A.T
        want[:, 0] = (rhi + (rlo + np.float32(0))).astype(np.float64)
        got = getattr(omx, "alpha" + key)[:, :o.nc].T.astype(np.float64)
        amax = np.abs(d).max(axis=1).astype(np.float64)
        scale = 2.0 ** np.ceil(np.log2(np.maximum(amax, 1e-300)) + 1e-12)
        bound = 2.0 ** -23 * np.abs(want) + (2.0 ** -24 + 216 * 2.0 ** -33) * 2 * scale[:, None]
        err = np.abs(got - want)
        assert (err <= bound).all(), (key, (err / np.maximum(bound, 1e-300)).max())


@pytest.mark.parametrize("mode", [None, "both"])
def test_tensor_core_table_exact_from_deltas_4d(mode):
    """4D tensor-core solve: every float32 coefficient equals alpha = A4 d
    computed exactly from the kernel's float32 deltas, up to its own float32
    rounding, the rounding of its three-part recombination, and the
    fixed-point truncation of d (2^-30 of the row's power-of-two scale,
    times the largest row abs-sum 1296.25 of A4)."""
    _, quadcubic = _mods()
    from arbinterp_gb300 import synth
    from oracle.arb_oracle import OracleQuadcubic
    f = synth.moving_gaussian_field4(n=(9, 8, 8, 7), h=(0.1, 0.12, 0.08, 0.1), seed=5).numpy()
    if mode == "both":
        f = np.hstack([f[:, :4], f[:, 4:5], np.sin(f[:, 4:5] + f[:, :1]), f[:, 4:5] * f[:, 1:2] + 0.5])
    kw = {} if mode is None else {"mode": mode}
    omx = quadcubic(f, "quiet", precision="mixed", **kw)
    omx.allCoeffs()
    o = OracleQuadcubic(f, **kw)
    blocks = o.basePointInds[:, None] + o.block_offsets[None, :]
    corner = 1 + 4 + 16 + 64
    for key in o.fields:
        v = o.fields[key]
        hi = v.astype(np.float32)
        lo = (v - hi).astype(np.float32) if key == "n" else np.zeros_like(hi)
        rhi, rlo = hi[blocks[:, corner]], lo[blocks[:, corner]]
        d = (hi[blocks] - rhi[:, None]) + (lo[blocks] - rlo[:, None])
        want = d.astype(np.float64) @ o.A.T
        want[:, 0] = (rhi + (rlo + np.float32(0))).astype(np.float64)
        got = getattr(omx, "alpha" + key)[:, :o.nc].T.astype(np.float64)
        amax = np.abs(d).max(axis=1).astype(np.float64)
        scale = 2.0 ** np.ceil(np.log2(np.maximum(amax, 1e-300)) + 1e-12)
        bound = 2.0 ** -23 * np.abs(want) + (2.0 ** -23 + 1296.25 * 2.0 ** -30) * 2 * scale[:, None]
        err = np.abs(got - want)
        assert (err <= bound).all(), (key, (err / np.maximum(bound, 1e-300)).max())


def test_quadcubic_mixed_gradient_with_strong_time_variation():
    """4D mixed on-the-fly gradients against the float64 path on a field that
    varies far more along t than in space (moving Gaussians with a fast
    cos(w t) amplitude): float32 deltas taken along one axis at a time keep
    every component within 6e-7 normwise."""
    _, quadcubic = _mods()
    from arbinterp_gb300 import synth
    f = synth.moving_gaussian_field4(n=(28, 26, 24, 20), h=(0.1, 0.1, 0.1, 0.1), seed=11)
    o64 = quadcubic(f, "quiet", precision="fp64", strategy="otf")
    omx = quadcubic(f, "quiet", precision="mixed", strategy="otf")
    q = synth.uniform_queries([float(v) for v in o64._lo], [float(v) for v in o64._hi], 300_000, 0,
                              [float(v) for v in o64._h], seed=12)
    v64, g64 = o64.Query(q.numpy().copy())
    vmx, gmx = omx.Query(q.numpy().copy())
    assert (normwise(vmx, v64) <= 2e-7).all()
    err = normwise(gmx, g64)
    assert (err <= 6e-7).all(), err


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_bin_once_evaluate_twice(prec):
    """arb_query_bin + arb_query_eval_binned equal the one-call sorted path,
    and the records are reusable on a second field of the same geometry."""
    import torch
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth, _lib
    L = _lib.lib()
    fa = synth.dipole_field3(n=(30, 34, 28), seed=21).numpy()
    fb = fa.copy()
    fb[:, 3:] = synth.dipole_field3(n=(30, 34, 28), seed=22).numpy()[:, 3:]
    oa = tricubic(fa, "quiet", mode="both", precision=prec, sort_threshold=0)
    ob = tricubic(fb, "quiet", mode="both", precision=prec, sort_threshold=0)
    q = synth.uniform_queries([oa.xIntMin, oa.yIntMin, oa.zIntMin], [oa.xIntMax, oa.yIntMax, oa.zIntMax],
                              40000, 400, [oa.hx, oa.hy, oa.hz], seed=23, device="cuda")
    n = q.shape[0]
    pc = _lib.PREC_FP64 if prec == "fp64" else _lib.PREC_MIXED
    need = int(L.arb_query_sorted_work_bytes(oa._g, pc, n))
    ws = torch.empty(need, dtype=torch.uint8, device="cuda")
    f64 = dict(dtype=torch.float64, device="cuda")
    c, nn, g = torch.empty((n, 3), **f64), torch.empty((n, 1), **f64), torch.empty((n, 3), **f64)
    inds = torch.empty(n, dtype=torch.int64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    out = _lib.ArbQueryOut(c.data_ptr(), nn.data_ptr(), g.data_ptr(), inds.data_ptr(), None, None)
    s = torch.cuda.current_stream().cuda_stream
    assert L.arb_query_bin(oa._g, pc, q.clone().data_ptr(), n, 3, 0, out, ws.data_ptr(), need,
                           st.data_ptr(), s) == 0
    for o in (oa, ob):
        assert L.arb_query_eval_binned(o._g, pc, 0, n, out, ws.data_ptr(), need, s) == 0
        want = o.Query(q.clone())
        for got, ref in zip((c, nn, g), want):
            assert torch.equal(torch.isnan(got), torch.isnan(ref))
            assert torch.equal(torch.nan_to_num(got), torch.nan_to_num(ref))


def test_autotuner_plans_and_caches(tmp_path, monkeypatch):
    """The autotuner times strategies / bin sizes on the caller's rows, caches
    the winner on disk, and every candidate gives identical results."""
    import json
    import torch
    monkeypatch.setenv("ARBINTERP_TUNE_DIR", str(tmp_path))
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth, autotune
    autotune._MEM.clear()
    f = synth.dipole_field3(n=(48, 40, 44), seed=31).numpy()
    o = tricubic(f, "quiet", mode="both", precision="mixed")
    q = synth.uniform_queries([o.xIntMin, o.yIntMin, o.zIntMin], [o.xIntMax, o.yIntMax, o.zIntMax],
                              300000, 3000, [o.hx, o.hy, o.hz], seed=32, device="cuda")
    got = o.Query(q.clone())
    plan = o.last_plan
    assert plan is not None and "ms" in plan
    cache = json.load(open(tmp_path / "autotune.json"))
    assert list(cache.values())[0]["bin_shift"] == plan["bin_shift"]
    ref = tricubic(f, "quiet", mode="both", precision="mixed", strategy="otf", sort_threshold=1 << 40)
    want = ref.Query(q.clone())
    for a, b in zip(got, want):
        assert torch.equal(torch.isnan(a), torch.isnan(b))
        assert (torch.nan_to_num(a) - torch.nan_to_num(b)).abs().max() <= 1e-6 * torch.nan_to_num(b).abs().max()
    n = q.shape[0]
    for cand in autotune._candidates(o):
        if cand["table"] and not o._table_complete:
            o.allCoeffs()
        res = o._launch(q.clone(), n, 3, False, False, cand)
        for a, b in zip(res[:3], want):
            assert torch.equal(torch.isnan(a), torch.isnan(b))
            assert (torch.nan_to_num(a) - torch.nan_to_num(b)).abs().max() <= 1e-6 * torch.nan_to_num(b).abs().max()
    autotune._MEM.clear()
    o2 = tricubic(f, "quiet", mode="both", precision="mixed")
    o2.Query(q.clone())
    assert o2.last_plan == plan


@pytest.mark.parametrize("prec,binned", [("fp64", False), ("mixed", False), ("mixed", True)])
def test_adjoint_gradients(prec, binned):
    """Backward kernel: dL/d(grid values) against the float64 reference
    adjoint (dense A^T scatter of the reference's monomial form) and against
    central finite differences; dL/d(query) against finite differences.
    binned: the bin-grouped adjoint (shared-memory scatter per bin)."""
    import torch
    from arbinterp_gb300 import synth
    from arbinterp_gb300.autograd import TricubicField
    from oracle.arb_oracle import OracleTricubic
    dt = torch.float64 if prec == "fp64" else torch.float32
    f = synth.gaussian_field3(n=(18, 16, 20), h=(0.1, 0.12, 0.08), seed=41).numpy()
    if prec == "mixed":
        f = f.astype(np.float32)
    fld = TricubicField(f, precision=prec, binned_adjoint=binned)
    ref = OracleTricubic(f.astype(np.float64))
    vals = fld.initial_values().to(dt).cuda().requires_grad_()
    lo, hi = np.array(ref.lo), np.array(ref.hi)
    rng = np.random.default_rng(42)
    qn = lo + (hi - lo) * rng.uniform(0.01, 0.99, (3000, 3))
    q = torch.tensor(qn, device="cuda", dtype=torch.float64, requires_grad=True)
    target = torch.tensor(rng.standard_normal(3000) * 0.1, device="cuda", dtype=dt)
    value, grad = fld(vals, q)
    loss = ((value - target) ** 2).sum() + 0.01 * (grad ** 2).sum()
    loss.backward()
    dv = (2 * (value - target)).detach().double().cpu().numpy()
    dg = (0.02 * grad).detach().double().cpu().numpy()
    gg_ref = ref.adjoint(qn, dv, dg)
    gg = vals.grad.double().cpu().numpy()
    tol = 1e-12 if prec == "fp64" else 2e-5
    assert np.abs(gg - gg_ref).max() <= tol * np.abs(gg_ref).max()

    # central finite differences in float64 through the float64 forward
    fd = TricubicField(f.astype(np.float64), precision="fp64")
    v64 = fd.initial_values().cuda()
    q64 = q.detach().clone()
    t64 = target.double()

    def L64(v, qq):
        a, b = fd(v, qq)
        return float((((a - t64) ** 2).sum() + 0.01 * (b ** 2).sum()).item())

    for p in rng.choice(v64.numel(), 40, replace=False):
        e = 1e-4
        vp, vm = v64.clone(), v64.clone()
        vp[p] += e
        vm[p] -= e
        fdv = (L64(vp, q64) - L64(vm, q64)) / (2 * e)
        assert abs(fdv - gg[p]) <= 1e-6 * max(1.0, np.abs(gg).max()) + 3e-5 * abs(fdv), (p, fdv, gg[p])
    qg = q.grad.cpu().numpy()
    for r in rng.choice(3000, 20, replace=False):
        for a in range(3):
            e = 1e-6 * ref.h[a]
            qp, qm = q64.clone(), q64.clone()
            qp[r, a] += e
            qm[r, a] -= e
            fdq = (L64(v64, qp) - L64(v64, qm)) / (2 * e)
            assert abs(fdq - qg[r, a]) <= 1e-4 * max(1.0, abs(fdq)), (r, a, fdq, qg[r, a])


def test_quadcubic_bin_tiles_equal_global_gathers():
    """4D mixed on the fly: the bin-staged kernel (4^4-cell bins, blocks read
    from shared memory) returns the same bits as the kernel gathering from
    global memory (8^4-cell bins), on a grid whose cell counts are not
    multiples of 4, with queries outside the volume and in the last cells."""
    import torch
    _, quadcubic = _mods()
    from arbinterp_gb300 import synth
    f = synth.moving_gaussian_field4(n=(23, 18, 21, 14), h=(0.1, 0.12, 0.08, 0.1), seed=31)
    o = quadcubic(f, "quiet", precision="mixed", strategy="otf")
    lo, hi = np.array([float(v) for v in o._lo]), np.array([float(v) for v in o._hi])
    rng = np.random.default_rng(32)
    q = lo + (hi - lo) * rng.uniform(-0.02, 1.0, (200_000, 4))
    q[:500] = hi - (hi - lo) * rng.uniform(0, 1e-3, (500, 4))
    qd = torch.tensor(q, device="cuda", dtype=torch.float64)
    outs = []
    for shift in (2, 3):
        plan = {"table": False, "binned": True, "bin_shift": shift}
        res = o._launch(qd.clone(), qd.shape[0], 4, False, False, plan)
        outs.append([None if t is None else t.clone() for t in res[:4]])
    for a, b in zip(*outs):
        if a is None:
            assert b is None
            continue
        assert torch.equal(torch.isnan(a), torch.isnan(b))
        assert torch.equal(torch.nan_to_num(a), torch.nan_to_num(b))
    assert torch.isnan(outs[0][1]).any() and not torch.isnan(outs[0][1]).all()


@pytest.mark.parametrize("mode", [None, "norm", "vector", "both"])
def test_tricubic_scalar_bin_tiles_equal_global_gathers(mode):
    """3D mixed on the fly, one field (a scalar field, or |B| in norm mode),
    the three components (vector mode) or both: the bin-staged kernel (8^3-cell
    bins in bank-class order, blocks read from shared memory) returns the same
    bits as the kernel gathering from global memory (4^3-cell bins), on a grid
    whose cell counts are not multiples of 8, with queries outside the volume
    and in the last cells."""
    import torch
    tricubic, _ = _mods()
    from arbinterp_gb300 import synth
    if mode is None:
        f = synth.gaussian_field3(n=(45, 38, 29), h=(0.1, 0.12, 0.08), seed=33)
        kw = {}
    else:
        f = synth.dipole_field3(n=(37, 30, 42), seed=34)
        kw = {"mode": mode}
    o = tricubic(f, "quiet", precision="mixed", strategy="otf", **kw)
    lo, hi = np.array([float(v) for v in o._lo]), np.array([float(v) for v in o._hi])
    rng = np.random.default_rng(35)
    q = lo + (hi - lo) * rng.uniform(-0.02, 1.0, (300_000, 3))
    q[:500] = hi - (hi - lo) * rng.uniform(0, 1e-3, (500, 3))
    qd = torch.tensor(q, device="cuda", dtype=torch.float64)
    outs = []
    for shift in (3, 2):
        plan = {"table": False, "binned": True, "bin_shift": shift}
        res = o._launch(qd.clone(), qd.shape[0], 3, False, False, plan)
        outs.append([None if t is None else t.clone() for t in res[:4]])
    for a, b in zip(*outs):
        if a is None:
            assert b is None
            continue
        assert torch.equal(torch.isnan(a), torch.isnan(b))
        assert torch.equal(torch.nan_to_num(a), torch.nan_to_num(b))
    first = next(t for t in outs[0][:3] if t is not None)
    assert torch.isnan(first).any() and not torch.isnan(first).all()
