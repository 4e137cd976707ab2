"""Batched persistent evaluation (arb_batched_launch) and its CUDA graph:
every field's rows match the single-field path; per-field strategy and tile
size come from the batch tuner."""
import numpy as np
import pytest

from conftest import normwise

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _batch(seed=0, nfields=7):
    import torch
    from arbinterp_gb300 import synth
    rng = np.random.default_rng(seed)
    fields, qs, counts = [], [], []
    for i in range(nfields):
        e = int(rng.integers(6, 24))
        h = tuple(rng.uniform(0.05, 0.2, 3))
        f = synth.gaussian_field3(n=(e, e + 1, e + 2), h=h, seed=100 + i).numpy()
        n = int(rng.choice([5, 300, 5000, 40000]))
        from oracle.arb_oracle import OracleTricubic
        o = OracleTricubic(f)
        q = synth.uniform_queries(o.lo, o.hi, n, max(1, n // 50), o.h, seed=200 + i)
        fields.append(f)
        qs.append(q)
        counts.append(q.shape[0])
    return fields, torch.cat(qs).cuda(), counts


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
def test_batched_matches_single_field(prec, tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("ARBINTERP_TUNE_DIR", str(tmp_path))
    from arbinterp_gb300 import tricubic
    from arbinterp_gb300.batched import BatchedTricubic
    fields, q, counts = _batch()
    b = BatchedTricubic(fields, precision=prec)
    norms, grads = b.query(q.clone(), counts)
    assert b.tile_rows in (256, 512, 1024, 2048)
    off = np.concatenate([[0], np.cumsum(counts)])
    tol = 1e-12 if prec == "fp64" else 1e-6
    for k, f in enumerate(fields):
        ref = tricubic(f, "quiet")                       # float64 single-field path
        rn, rg = ref.Query(q[off[k]:off[k + 1]].clone())
        gn, gg = norms[off[k]:off[k + 1]], grads[off[k]:off[k + 1]]
        assert torch.equal(torch.isnan(gn), torch.isnan(rn))
        a, r = gn.cpu().numpy(), rn.cpu().numpy()
        assert (normwise(a, r) <= tol).all(), (k, normwise(a, r))
        assert (normwise(gg.cpu().numpy(), rg.cpu().numpy()) <= tol).all()


def test_batched_graph_replay(tmp_path, monkeypatch):
    import torch
    monkeypatch.setenv("ARBINTERP_TUNE_DIR", str(tmp_path))
    from arbinterp_gb300.batched import BatchedTricubic
    fields, q, counts = _batch(seed=1)
    b = BatchedTricubic(fields, precision="mixed")
    qbuf = q.clone()
    graph, (gn, gg) = b.capture(qbuf, counts)
    graph.replay()
    torch.cuda.synchronize()
    want_n, want_g = b.query(q.clone(), counts)
    assert torch.equal(torch.nan_to_num(gn), torch.nan_to_num(want_n))
    # new query contents, same shape: replay re-evaluates them
    fields2, q2, counts2 = _batch(seed=2)
    q2 = q2[:q.shape[0]] if q2.shape[0] >= q.shape[0] else torch.cat([q2, q[q2.shape[0]:]])
    qbuf.copy_(q2)
    graph.replay()
    torch.cuda.synchronize()
    w2n, _ = b.query(q2.clone(), counts)
    assert torch.equal(torch.nan_to_num(gn), torch.nan_to_num(w2n))
    assert not torch.equal(torch.nan_to_num(want_n), torch.nan_to_num(w2n))


@pytest.mark.parametrize("prec", ["fp64", "mixed"])
@pytest.mark.parametrize("ratio", [None, 1.0])
def test_batched_c3_shaped_fields_vs_oracle(prec, ratio):
    """Fields shaped like the 512-field batched workload: cubes with edges
    log-uniform in [16, 128], anisotropic spacings in [0.05, 0.2],
    Gaussian-sum values, 1e3-1e5 queries each (1% outside the volume).  Each
    field's rows in the persistent launch against the CPU oracle: NaN masks
    bit-exact, values <= 1e-12 normwise in float64 and <= 1e-6 in mixed
    precision.  ratio None evaluates every field on the fly; 1.0 switches
    the fields with at least one query per cell to coefficient tables."""
    import torch
    from arbinterp_gb300 import synth
    from arbinterp_gb300.batched import BatchedTricubic
    from oracle.arb_oracle import OracleTricubic
    fields, qs, counts, refs = [], [], [], []
    for f, nq, seed in synth.batched_fields(n_fields=24, seed=7, q_range=(1e3, 1e5)):
        f = f.numpy()
        o = OracleTricubic(f)
        q = synth.uniform_queries(o.lo, o.hi, nq, max(1, nq // 100), o.h, seed=seed % (1 << 30))
        fields.append(f)
        qs.append(q)
        counts.append(q.shape[0])
        refs.append(o.query(q.numpy().copy()))
    edges = [int(round(len(f) ** (1 / 3))) for f in fields]
    assert min(edges) < 24 and max(edges) > 90
    b = BatchedTricubic(fields, precision=prec)
    b.tile_rows = 1024
    b.table_ratio = ratio
    b._apply_strategy(counts, ratio)
    if ratio is not None:
        assert any(o._table_complete for o in b.interps) and not all(o._table_complete for o in b.interps)
    norms, grads = b.query(torch.cat(qs).cuda(), counts)
    off = np.concatenate([[0], np.cumsum(counts)])
    tol = 1e-12 if prec == "fp64" else 1e-6
    for k, ref in enumerate(refs):
        gn = norms[off[k]:off[k + 1]].cpu().numpy()
        gg = grads[off[k]:off[k + 1]].cpu().numpy()
        assert np.array_equal(np.isnan(gn), np.isnan(ref["norms"])), k
        assert np.array_equal(np.isnan(gg), np.isnan(ref["grads"])), k
        assert (normwise(gn, ref["norms"]) <= tol).all(), (k, normwise(gn, ref["norms"]))
        assert (normwise(gg, ref["grads"]) <= tol).all(), (k, normwise(gg, ref["grads"]))
