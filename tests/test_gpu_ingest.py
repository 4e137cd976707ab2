"""Single-pass ingest of rows in meshgrid order (arb_ingest_ordered) against
the general two-step ingest (arb_ingest_axes + arb_ingest_scatter): same
axes, same grids, same query results, for every axis order and direction;
rows in any other order fall back to the general path."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _field(dim, order, flip, seed=0, vector=False, dtype=np.float64):
    """Rows of a regular grid listed lexicographically with axis order
    `order` (slowest first) and the axes in `flip` descending."""
    rng = np.random.default_rng(seed)
    n = [7, 6, 5, 4][:dim]
    h = rng.uniform(0.05, 0.2, dim)
    ax = [rng.uniform(-1, 1) + h[a] * np.arange(n[a]) for a in range(dim)]
    ax = [a[::-1] if i in flip else a for i, a in enumerate(ax)]
    mesh = np.meshgrid(*[ax[a] for a in order], indexing="ij")
    cols = [None] * dim
    for k, a in enumerate(order):
        cols[a] = mesh[k].ravel()
    X = np.stack(cols, 1)
    vals = np.sin(X @ rng.uniform(0.5, 2.0, dim))[:, None] * (rng.uniform(0.5, 2.0, 3 if vector else 1))
    return np.hstack([X, vals]).astype(dtype)


def _both_paths(make, field, monkeypatch):
    from arbinterp_gb300 import interp
    a = make(field)
    monkeypatch.setattr(interp, "_ORDERED_INGEST", False)
    b = make(field)
    monkeypatch.setattr(interp, "_ORDERED_INGEST", True)
    return a, b


def _same(a, b, q):
    import torch
    assert a._n == b._n
    for x, y in zip(a._axes_dev, b._axes_dev):
        assert torch.equal(x, y)
    assert torch.equal(a._grid64, b._grid64)
    if a._grid32 is not None:
        assert torch.equal(a._grid32, b._grid32)
    if a._raw is not None:
        assert torch.equal(a._raw, b._raw)
    ra, rb = a.Query(q.copy()), b.Query(q.copy())
    ra = ra if isinstance(ra, tuple) else (ra,)
    rb = rb if isinstance(rb, tuple) else (rb,)
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y, equal_nan=True)


@pytest.mark.parametrize("order,flip", [((0, 1, 2), ()), ((2, 1, 0), ()), ((1, 2, 0), (1,)),
                                        ((0, 2, 1), (0, 2)), ((2, 1, 0), (0, 1, 2))])
@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_tricubic_meshgrid_orders(order, flip, prec, monkeypatch):
    from arbinterp_gb300 import tricubic
    f = _field(3, order, flip, vector=True)
    q = np.random.default_rng(1).uniform(f[:, :3].min(0), f[:, :3].max(0), (500, 3))
    for mode in ("both", "norm"):
        a, b = _both_paths(lambda x: tricubic(x, "quiet", mode=mode, precision=prec), f, monkeypatch)
        assert a.ingest_path == "ordered" and b.ingest_path == "general"
        _same(a, b, q)
        assert np.array_equal(a.inputfield, b.inputfield)


@pytest.mark.parametrize("order,flip", [((3, 2, 1, 0), ()), ((0, 1, 2, 3), (3,)), ((1, 3, 0, 2), (0,))])
def test_quadcubic_meshgrid_orders(order, flip, monkeypatch):
    from arbinterp_gb300 import quadcubic
    f = _field(4, order, flip)
    q = np.random.default_rng(2).uniform(f[:, :4].min(0), f[:, :4].max(0), (300, 4))
    a, b = _both_paths(lambda x: quadcubic(x, "quiet"), f, monkeypatch)
    assert a.ingest_path == "ordered"
    _same(a, b, q)


def test_float32_field_ordered(monkeypatch):
    from arbinterp_gb300 import tricubic
    f = _field(3, (2, 1, 0), (), dtype=np.float32)
    q = np.random.default_rng(3).uniform(f[:, :3].min(0), f[:, :3].max(0), (200, 3))
    a, b = _both_paths(lambda x: tricubic(x, "quiet", precision="mixed"), f, monkeypatch)
    assert a.ingest_path == "ordered"
    _same(a, b, q)


def test_other_orders_fall_back():
    from arbinterp_gb300 import tricubic
    f = _field(3, (2, 1, 0), ())
    q = np.random.default_rng(4).uniform(f[:, :3].min(0), f[:, :3].max(0), (300, 3))
    ref = tricubic(f, "quiet")
    rng = np.random.default_rng(5)
    swapped = f.copy()
    swapped[[10, 57]] = swapped[[57, 10]]               # meshgrid order but two rows exchanged
    shuffled = f[rng.permutation(len(f))]
    for g in (swapped, shuffled):
        o = tricubic(g, "quiet")
        assert o.ingest_path == "general"
        assert np.array_equal(o.Query(q.copy())[0], ref.Query(q.copy())[0], equal_nan=True)
    # a field that is no full regular grid raises ValueError: at construction
    # when the axis probe sees it, else at the first use of the grid
    off = f.copy()
    off[33, 1] += 1e-3                                  # a point off its axis (not on the probed lines)
    with pytest.raises(ValueError):
        tricubic(off, "quiet").Query(q.copy())
    dup = f.copy()
    dup[5] = dup[6]                                     # duplicate point, one slot empty
    with pytest.raises(ValueError):
        tricubic(dup, "quiet").Query(q.copy())


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("binned", [False, True])
def test_single_pass_check_read_at_first_query(prec, binned):
    """The constructor waits for the axis probe only; the pass that writes the
    grid is checked at the first synchronisation.  Rows that pass the probe
    (the lines through row 0 form a meshgrid) but are out of order elsewhere
    make the first device query rewrite the grid with the general ingest and
    evaluate again: the same outputs, write-back and indices as an
    interpolant built from the rows in order; a point off its axis raises
    ValueError there."""
    import torch
    from arbinterp_gb300 import tricubic
    f = _field(3, (2, 1, 0), (), vector=True)
    g = f.copy()
    g[[10, 57]] = g[[57, 10]]
    q = np.random.default_rng(6).uniform(f[:, :3].min(0) - 0.05, f[:, :3].max(0) + 0.05, (500, 3))
    kw = dict(mode="both", precision=prec, sort_threshold=0 if binned else 1 << 30)
    ref = tricubic(torch.from_numpy(f).cuda(), "quiet", **kw)
    o = tricubic(torch.from_numpy(g).cuda(), "quiet", **kw)
    assert o._fill_pending
    qa, qb = torch.from_numpy(q).cuda(), torch.from_numpy(q).cuda()
    ra, rb = ref.Query(qa), o.Query(qb)
    assert not o._fill_pending and o._ingest_path == "general" and ref.ingest_path == "ordered"
    assert torch.equal(qa.isnan(), qb.isnan())
    assert np.array_equal(ref.queryInds, o.queryInds)
    for x, y in zip(ra, rb):
        assert torch.equal(x.isnan(), y.isnan())
        assert torch.equal(torch.nan_to_num(x), torch.nan_to_num(y))
    off = f.copy()
    off[33, 1] += 1e-3
    o = tricubic(torch.from_numpy(off).cuda(), "quiet", **kw)
    with pytest.raises(ValueError):
        o.Query(torch.from_numpy(q).cuda())


@pytest.mark.parametrize("mode", ["both", "norm"])
def test_mixed_device_field_float64_grid_on_first_use(mode):
    """Mixed precision on a CUDA field tensor skips the float64 grid at
    construction; it is produced from the (unmodified) tensor when first
    needed and equals the eagerly built one."""
    import torch
    from arbinterp_gb300 import tricubic
    f = torch.from_numpy(_field(3, (2, 1, 0), (), vector=True)).cuda()
    eager = tricubic(f.cpu().numpy(), "quiet", mode=mode, precision="mixed")   # NumPy input: eager
    lazy = tricubic(f, "quiet", mode=mode, precision="mixed")
    assert eager._grid64_t is not None and lazy._grid64_t is None
    q = np.random.default_rng(6).uniform(f[:, :3].min(0).values.cpu().numpy(),
                                         f[:, :3].max(0).values.cpu().numpy(), (300, 3))
    for x, y in zip(lazy.Query(q.copy()), eager.Query(q.copy())):
        assert np.array_equal(x, y, equal_nan=True)
    assert lazy._grid64_t is None                   # queries never needed it
    assert np.array_equal(lazy.inputfield, eager.inputfield)
    assert lazy._grid64_t is not None
    for name in ("Bx", "By", "Bz", "Bn") if mode == "both" else ("Bn",):
        a, b = getattr(lazy, name), getattr(eager, name)
        assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max(), name   # double-float |B| vs float64
    again = tricubic(f, "quiet", mode=mode, precision="mixed")
    f[0, 3] += 1.0                                   # the caller changes the field in place
    with pytest.raises(RuntimeError):
        again.inputfield


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_single_pass_check_read_after_pipelined_host_query(prec):
    """A large host query starts its uploads without waiting for the grid
    fill and reads the fill's row check with the status at the end: rows out
    of meshgrid order (past the probe) make it rewrite the grid and evaluate
    again, with the outputs, in-place NaN rows and indices of an interpolant
    built from the rows in order; a point off its axis raises ValueError."""
    from arbinterp_gb300 import interp, tricubic
    f = _field(3, (2, 1, 0), (), vector=True)
    g = f.copy()
    g[[10, 57]] = g[[57, 10]]
    n = interp.PIPELINE_MIN_ROWS + 777
    q = np.random.default_rng(8).uniform(f[:, :3].min(0) - 0.05, f[:, :3].max(0) + 0.05, (n, 3))
    kw = dict(mode="both", precision=prec, strategy="otf")
    ref = tricubic(f, "quiet", **kw)
    o = tricubic(g, "quiet", **kw)
    assert o._fill_pending
    qa, qb = q.copy(), q.copy()
    ra, rb = ref.Query(qa), o.Query(qb)
    assert not o._fill_pending and o._ingest_path == "general" and ref.ingest_path == "ordered"
    assert np.array_equal(np.isnan(qa), np.isnan(qb)) and np.isnan(qb).any()
    assert np.array_equal(ref.queryInds, o.queryInds)
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y, equal_nan=True)
    off = f.copy()
    off[33, 1] += 1e-3
    o = tricubic(off, "quiet", **kw)
    with pytest.raises(ValueError):
        o.Query(q.copy())
