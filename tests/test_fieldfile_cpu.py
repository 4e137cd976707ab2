"""Field-file reader, CPU side: the oracle's restatement of genfromtxt's
line handling and the host's error message agree with np.genfromtxt itself,
and every corpus token's expected bits are what genfromtxt produces."""
import struct

import numpy as np
import pytest

from csv_corpus import STRUCT_CASES, long_line_case, tokens
from oracle import csv_oracle as co


def _expected(data, kw):
    d = kw.get("delimiter", ",").encode()
    c = kw.get("comments", "#")
    c = None if c is None else c.encode()
    return co.values_per_line(data, d, c, kw.get("skip_header", 0))


@pytest.mark.parametrize("case", range(len(STRUCT_CASES)))
def test_line_structure_matches_genfromtxt(case):
    from arbinterp_gb300.fieldfile import _invalid_message
    data, kw = STRUCT_CASES[case]
    nv = _expected(data, kw)
    data_lines = np.flatnonzero(nv > 0)
    try:
        ref, warns = co.reference(data, **kw)
    except ValueError as e:
        first = int(data_lines[0])
        assert str(e) == _invalid_message(nv, first, int(nv[first]), kw.get("skip_header", 0))
        return
    if data_lines.size == 0:
        assert ref.size == 0 and any("Empty input file" in w for w in warns)
        return
    ncols = int(nv[data_lines[0]])
    assert (nv[data_lines] == ncols).all()
    shape = tuple(s for s in (data_lines.size, ncols) if s != 1)
    assert ref.shape == shape
    # every value is float() of its token (NaN when float() rejects it)
    lines = co.split_lines(data)
    toks = [t for l in data_lines for t in co.line_values(lines[l], kw.get("delimiter", ",").encode(),
                                                          None if kw.get("comments", "#") is None
                                                          else kw.get("comments", "#").encode())]
    want = np.array([co.token_bits(t) for t in toks], dtype=np.uint64)
    assert np.array_equal(np.atleast_1d(ref).reshape(-1).view(np.uint64), want)


def test_token_corpus_bits_are_genfromtxts():
    toks = tokens(1, 3000)
    data = "".join(f"0,{t}\n" for t in toks).encode()
    ref, _ = co.reference(data)
    want = np.array([co.token_bits(t.encode()) for t in toks], dtype=np.uint64)
    assert np.array_equal(ref[:, 1].view(np.uint64), want)
    # the corpus reaches the edges it is meant to
    vals = np.array([struct.unpack("<d", struct.pack("<Q", int(b)))[0] for b in want])
    fin = vals[np.isfinite(vals)]
    assert (np.abs(fin[fin != 0]) < 2.2250738585072014e-308).any()     # subnormals
    assert np.isinf(vals).sum() > 5 and np.isnan(vals).sum() > 20


def test_long_line_case_parses():
    data = long_line_case(300)
    ref, _ = co.reference(data)
    assert ref.shape == (2, 300) and np.isfinite(ref).all()
