"""CPU oracle for the GPU field-file reader (test infrastructure only).

The reference loads its fields with ``np.genfromtxt(path, delimiter=',')``
(examples/3D_ARBInterpExample.py:14,37, examples/4D_ARBInterpExample.py:14,38),
so numpy itself is the oracle for values: ``reference(data, ...)`` runs
``np.genfromtxt`` on the bytes opened in text mode (universal newlines, as
for a path).  For the line structure (which lines carry how many values)
this module restates genfromtxt's line handling in plain Python, following
numpy/lib/_npyio_impl.py (genfromtxt: skip_header, the first-values loop,
the per-line column check) and numpy/lib/_iotools.py
(LineSplitter._delimited_splitter: comment cut, strip(" \\r\\n"), split),
pinned against ``np.genfromtxt`` by tests/test_fieldfile_cpu.py.  Token
values are Python's ``float()`` (genfromtxt's float converter, with NaN for
a token float() rejects: StringConverter._loose_call).
"""
from __future__ import annotations

import io
import struct
import warnings

import numpy as np

NAN_BITS = 0x7FF8000000000000


def split_lines(data: bytes) -> list[bytes]:
    """Lines of a text-mode file: "\\n", "\\r\\n" and a lone "\\r" end a
    line; an unterminated last line counts, an empty tail does not."""
    out, start, i, n = [], 0, 0, len(data)
    while i < n:
        c = data[i]
        if c == 10 or c == 13:
            out.append(data[start:i])
            i += 2 if (c == 13 and i + 1 < n and data[i + 1] == 10) else 1
            start = i
        else:
            i += 1
    if start < n:
        out.append(data[start:])
    return out


def line_values(line: bytes, delimiter: bytes = b",", comments: bytes | None = b"#") -> list[bytes]:
    """LineSplitter._delimited_splitter on one line (autostrip off)."""
    if comments is not None:
        line = line.split(comments)[0]
    line = line.strip(b" \r\n")
    if not line:
        return []
    return line.split(delimiter)


def values_per_line(data: bytes, delimiter: bytes = b",", comments: bytes | None = b"#",
                    skip_header: int = 0) -> np.ndarray:
    """int32 count of values on each physical line (0: skipped line)."""
    lines = split_lines(data)
    nv = np.array([len(line_values(l, delimiter, comments)) for l in lines], dtype=np.int32)
    nv[:skip_header] = 0
    return nv


def token_bits(tok: bytes) -> int:
    """float(tok) as IEEE bits; NaN (0x7ff8...) when float() rejects it."""
    try:
        v = float(tok.decode("ascii"))
    except ValueError:
        return NAN_BITS
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def reference(data: bytes, delimiter: str = ",", comments: str | None = "#", skip_header: int = 0):
    """np.genfromtxt on the bytes as a text-mode file; returns (array,
    warnings list) or raises what genfromtxt raises."""
    f = io.StringIO(data.decode("ascii"), newline=None)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        a = np.genfromtxt(f, delimiter=delimiter, comments=comments, skip_header=skip_header)
    return a, [str(x.message) for x in w]
