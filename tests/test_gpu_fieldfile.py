"""GPU field-file reader (arb_csv_* through arbinterp_gb300.genfromtxt)
against np.genfromtxt: values bit-identical (NaN payloads and signs
included), shapes, warnings and error messages equal; per-line value counts
equal to the oracle's restatement of genfromtxt's line handling."""
import os
import warnings

import numpy as np
import pytest

from csv_corpus import STRUCT_CASES, long_line_case, savetxt_bytes, tokens
from oracle import csv_oracle as co

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _gpu(data, **kw):
    from arbinterp_gb300 import genfromtxt
    stats = {}
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        out = genfromtxt(data, stats=stats, **kw)
    assert out.is_cuda and str(out.dtype) == "torch.float64"
    return out.cpu().numpy(), [str(x.message) for x in w], stats


def _same_bits(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    assert a.shape == b.shape, (a.shape, b.shape)
    assert np.array_equal(a.reshape(-1).view(np.uint64), b.reshape(-1).view(np.uint64))


@pytest.mark.parametrize("case", range(len(STRUCT_CASES)))
def test_line_structure_cases(case):
    data, kw = STRUCT_CASES[case]
    try:
        ref, rw = co.reference(data, **kw)
    except ValueError as e:
        with pytest.raises(ValueError) as got:
            _gpu(data, **kw)
        assert str(got.value) == str(e)
        return
    got, gw, _ = _gpu(data, **kw)
    _same_bits(got, ref)
    assert any("Empty input file" in w for w in gw) == any("Empty input file" in w for w in rw)


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_token_corpus_bit_exact(seed):
    """Every token's double equals float()'s, including exact midpoints,
    subnormals, overflow edges and 700-900 digit mantissas; the exact
    big-integer pass is exercised."""
    toks = tokens(seed, 20000)
    data = "".join(f"{i},{t}\n" for i, t in enumerate(toks)).encode()
    got, _, stats = _gpu(data)
    want = np.array([co.token_bits(t.encode()) for t in toks], dtype=np.uint64)
    assert got.shape == (len(toks), 2)
    bad = np.flatnonzero(got[:, 1].view(np.uint64) != want)
    assert bad.size == 0, [(toks[i], hex(int(got[i, 1].view(np.uint64))), hex(int(want[i]))) for i in bad[:5]]
    assert np.array_equal(got[:, 0], np.arange(len(toks), dtype=np.float64))
    assert stats["nexact"] > 0 and stats["nrows"] == len(toks)


def test_field_file_round_trip_and_interpolant(tmp_path):
    """A 'both' field written as the reference's example files are
    (savetxt '%.18e'), read from disk: equal to np.genfromtxt bit for bit,
    and an interpolant built from the device tensor answers exactly as one
    built from numpy's array."""
    from arbinterp_gb300 import genfromtxt, synth, tricubic
    f = synth.dipole_field3(n=(20, 18, 16), seed=4).numpy()
    path = os.path.join(tmp_path, "Example3DVectorField.csv")
    with open(path, "wb") as fh:
        fh.write(savetxt_bytes(f))
    ref = np.genfromtxt(path, delimiter=",")
    dev = genfromtxt(path, delimiter=",")
    _same_bits(dev.cpu().numpy(), ref)
    q = np.random.default_rng(0).uniform(f[:, :3].min(0), f[:, :3].max(0), (2000, 3))
    a = tricubic(ref, "quiet", mode="both").Query(q.copy())
    b = tricubic(dev, "quiet", mode="both").Query(q.copy())
    for x, y in zip(a, b):
        assert np.array_equal(x, y, equal_nan=True)


def test_long_lines_leave_the_shared_memory_stage():
    data = long_line_case(5000)
    got, _, _ = _gpu(data)
    ref, _ = co.reference(data)
    _same_bits(got, ref)


def test_many_rows_with_blank_comment_and_crlf_lines():
    """Row compaction across CTAs: 100k lines with skipped lines spread
    through them, CRLF endings, ragged whitespace."""
    rng = np.random.default_rng(7)
    a = rng.standard_normal((100_000, 4)) * 10.0 ** rng.integers(-20, 20, (100_000, 4))
    lines = savetxt_bytes(a).split(b"\n")[:-1]
    out = []
    for k, l in enumerate(lines):
        if k % 97 == 0:
            out.append(b"# comment line")
        if k % 131 == 0:
            out.append(b"   ")
        out.append(b" " + l.replace(b",", b" ,", 1) + (b"  # trailing" if k % 3 == 0 else b""))
    data = b"\r\n".join(out) + b"\r\n"
    got, _, stats = _gpu(data)
    ref, _ = co.reference(data)
    _same_bits(got, ref)
    assert stats["nlines"] == len(out)


def test_nvals_match_oracle_line_counts():
    import torch
    from arbinterp_gb300 import _lib
    from arbinterp_gb300.fieldfile import bytes_to_device
    data = b"\n".join([b"1,2,3", b"", b"#x", b"4,5", b"  ", b"6,7,8 # c", b",,", b"9"]) + b"\r"
    text, n = bytes_to_device(data)
    L = _lib.lib()
    s = torch.cuda.current_stream().cuda_stream
    info = torch.zeros(9, dtype=torch.int64, device="cuda")
    cw = torch.empty(L.arb_csv_count_work_bytes(n), dtype=torch.uint8, device="cuda")
    _lib.check(L.arb_csv_count(text.data_ptr(), n, cw.data_ptr(), cw.numel(), info.data_ptr(), s), "count")
    nlines = int(info[0])
    lw = torch.empty(L.arb_csv_lines_work_bytes(nlines), dtype=torch.uint8, device="cuda")
    nv = torch.empty(nlines, dtype=torch.int32, device="cuda")
    _lib.check(L.arb_csv_split(text.data_ptr(), n, nlines, ord(","), ord("#"), 0, cw.data_ptr(), lw.data_ptr(),
                               lw.numel(), nv.data_ptr(), info.data_ptr(), s), "split")
    assert np.array_equal(nv.cpu().numpy(), co.values_per_line(data))
    h = info.cpu().numpy()
    assert h[2] == 0 and h[3] == 3 and h[4] == 3 and h[5] == 2    # first line, ncols, nrows, ninvalid


def test_non_ascii_and_unsupported_inputs_are_refused(tmp_path):
    from arbinterp_gb300 import genfromtxt
    with pytest.raises(ValueError, match="not ASCII"):
        genfromtxt("1,2\n3,é\n".encode("utf-8"))
    with pytest.raises(NotImplementedError):
        genfromtxt(b"1 2\n", delimiter=None)
    with pytest.raises(NotImplementedError):
        genfromtxt(os.path.join(tmp_path, "f.csv.gz"))


def test_concurrent_readers():
    """Two threads reading texts longer than one staging chunk at the same
    time get the same tables as reading from device-resident text."""
    import threading
    from arbinterp_gb300 import fieldfile, genfromtxt, synth
    texts = [synth.field_csv_text((128, 128, 34), 3, seed=s, device="cuda") for s in (21, 22)]
    assert all(t.numel() > fieldfile.CHUNK for t in texts)
    host = [t.cpu().numpy().tobytes() for t in texts]
    want = [fieldfile.parse_device_text(t, t.numel()).cpu().numpy() for t in texts]
    got = [None, None]

    def run(k):
        got[k] = genfromtxt(host[k]).cpu().numpy()
    th = [threading.Thread(target=run, args=(k,)) for k in range(2)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for g, w in zip(got, want):
        _same_bits(g, w)
