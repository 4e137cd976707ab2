"""Field files on the device.

``genfromtxt(path, delimiter=',')`` replaces the reference's way of loading
its N x 4..7 field tables, ``np.genfromtxt(path, delimiter=',')``
(examples/3D_ARBInterpExample.py:14,37, examples/4D_ARBInterpExample.py:14,38),
and returns the table as a CUDA float64 tensor that ``tricubic`` /
``quadcubic`` take directly.  The file is read into a small ring of pinned
host buffers by several threads while earlier chunks are copied to the
device; lines, values per line and every number are then found and
converted on the GPU (``csrc/csv.cu``, C ABI ``arb_csv_*``), with results
bit-identical to numpy's:

* universal newlines; text from the comment character on dropped; lines
  stripped of spaces and skipped when empty; ``skip_header`` lines skipped;
* the first line with values fixes the column count, and any other count
  raises numpy's ``ValueError`` ("Some errors were detected !" with its
  line numbering);
* each token converted exactly as Python's ``float()`` (correctly rounded;
  ``inf``/``nan`` spellings, underscores between digits); an empty or
  malformed token reads as NaN;
* an input without any value warns "genfromtxt: Empty input file" and gives
  an empty array; the result is squeezed (one row or one column -> 1-D).

Not covered, and refused loudly: non-ASCII text (the reader checks every
byte), compressed files, ``delimiter=None`` (whitespace splitting), and the
other ``genfromtxt`` keywords.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import threading
import warnings

import numpy as np
import torch

from . import _lib

CHUNK = 64 << 20          # pinned staging buffer size (bytes)
RING = 3                  # staging buffers per device
READERS = 8               # threads reading one chunk
_INFO_WORDS = 9           # arb_csv_info: 8 int64 + 2 int32

_rings: dict = {}
_ring_lock = threading.Lock()
_pool = None


def _readers():
    global _pool
    if _pool is None:
        _pool = cf.ThreadPoolExecutor(max_workers=READERS, thread_name_prefix="arb-csv-read")
    return _pool


def _ring(device: torch.device):
    """(buffers, events, lock) of a device's staging ring; the lock is held
    for a whole transfer so concurrent callers do not share buffers."""
    key = device.index
    with _ring_lock:
        if key not in _rings:
            bufs = [torch.empty(CHUNK, dtype=torch.uint8, pin_memory=True) for _ in range(RING)]
            _rings[key] = (bufs, [torch.cuda.Event() for _ in range(RING)], threading.Lock())
        return _rings[key]


def _pread_into(fd: int, mv: memoryview, offset: int) -> None:
    done = 0
    while done < len(mv):
        n = os.preadv(fd, [mv[done:]], offset + done)
        if n <= 0:
            raise OSError(f"short read at offset {offset + done}")
        done += n


def _padded(n: int) -> int:
    return max(16, (n + 15) & ~15)


def _to_device(size: int, fill, device, stream):
    """A CUDA uint8 tensor (16-byte padded) holding ``size`` bytes that
    ``fill(view, offset)`` writes into pinned staging buffers, chunk by chunk
    on several threads; each chunk's host-to-device copy runs on ``stream``
    while the next chunk is filled."""
    device = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    stream = torch.cuda.current_stream(device) if stream is None else stream
    text = torch.empty(_padded(size), dtype=torch.uint8, device=device)
    if size == 0:
        return text, 0
    bufs, evs, lock = _ring(device)
    pool = _readers()
    with lock:
        for k, off in enumerate(range(0, size, CHUNK)):
            n = min(CHUNK, size - off)
            slot = k % RING
            evs[slot].synchronize()           # the copy that last used this buffer is done
            mv = memoryview(bufs[slot].numpy())[:n]
            step = max(4 << 20, -(-n // READERS))
            list(pool.map(lambda a: fill(mv[a:a + step], off + a), range(0, n, step)))
            with torch.cuda.stream(stream):
                text[off:off + n].copy_(bufs[slot][:n], non_blocking=True)
                evs[slot].record(stream)
        for e in evs:                         # buffers idle before another caller takes the ring
            e.synchronize()
    return text, size


def file_to_device(path, device=None, stream=None):
    """Bytes of the file at ``path`` in a CUDA uint8 tensor (16-byte padded)
    and the file size; reads overlap the copies."""
    size = os.path.getsize(path)
    fd = os.open(path, os.O_RDONLY)
    try:
        return _to_device(size, lambda mv, off: _pread_into(fd, mv, off), device, stream)
    finally:
        os.close(fd)


def bytes_to_device(data, device=None, stream=None):
    """A bytes-like object's contents in a CUDA uint8 tensor (16-byte padded)."""
    src = np.frombuffer(memoryview(data).cast("B"), dtype=np.uint8)

    def fill(mv, off):
        np.copyto(np.frombuffer(mv, dtype=np.uint8), src[off:off + len(mv)])
    return _to_device(int(src.size), fill, device, stream)


def _char(v, what: str) -> int:
    if v is None:
        return -1
    if isinstance(v, bytes):
        v = v.decode("latin1")
    if not isinstance(v, str) or len(v) != 1 or ord(v) > 127 or v in "\r\n":
        raise NotImplementedError(f"{what} must be one ASCII character other than CR/LF (got {v!r})")
    return ord(v)


def _info(t: torch.Tensor) -> dict:
    h = t.cpu().numpy()
    names = ("nlines", "first_nonascii", "first_data_line", "ncols", "nrows", "ninvalid", "nexact", "nqueued")
    d = {k: int(h[i]) for i, k in enumerate(names)}
    d["error"] = int(h[8] & 0xFFFFFFFF)
    return d


def parse_device_text(text: torch.Tensor, nbytes: int, delimiter=",", comments="#", skip_header: int = 0,
                      name: str = "<bytes>", stream=None, stats: dict | None = None,
                      timing: dict | None = None) -> torch.Tensor:
    """Parse ``nbytes`` of CSV text already on the device (a 16-byte aligned
    uint8 CUDA tensor) into a float64 table, as ``genfromtxt`` does.
    ``timing``, when given, receives each phase's device time in ms (CUDA
    events around the count, split and parse calls)."""
    L = _lib.lib()
    delim = _char(delimiter, "delimiter")
    if delim == -1:
        raise NotImplementedError("delimiter=None (whitespace splitting) is not supported by the GPU reader")
    comment = _char(comments, "comments")
    if comment == delim:
        raise ValueError("the comment character equals the delimiter")
    skip_header = int(skip_header)
    if skip_header < 0:
        raise ValueError("skip_header must be >= 0")
    device = text.device
    stream = torch.cuda.current_stream(device) if stream is None else stream
    s = stream.cuda_stream
    if text.data_ptr() % 16 or text.numel() < nbytes:
        raise ValueError("text must be a 16-byte aligned uint8 tensor holding nbytes bytes")
    info = torch.zeros(_INFO_WORDS, dtype=torch.int64, device=device)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(6)] if timing is not None else None

    def mark(k):
        if ev is not None:
            ev[k].record(stream)
    with torch.cuda.stream(stream):
        cw = torch.empty(L.arb_csv_count_work_bytes(nbytes), dtype=torch.uint8, device=device)
        mark(0)
        _lib.check(L.arb_csv_count(text.data_ptr(), nbytes, cw.data_ptr(), cw.numel(), info.data_ptr(), s),
                   "arb_csv_count")
        mark(1)
        h = _info(info)
        if h["first_nonascii"] >= 0:
            off = h["first_nonascii"]
            raise ValueError(f"{name}: byte 0x{int(text[off]):02x} at offset {off} is not ASCII; "
                             "the GPU reader accepts ASCII text only")
        nlines = h["nlines"]
        if nlines == 0:
            return _empty(name, device)
        lw = torch.empty(L.arb_csv_lines_work_bytes(nlines), dtype=torch.uint8, device=device)
        nvals = torch.empty(nlines, dtype=torch.int32, device=device)
        mark(2)
        _lib.check(L.arb_csv_split(text.data_ptr(), nbytes, nlines, delim, comment, skip_header, cw.data_ptr(),
                                   lw.data_ptr(), lw.numel(), nvals.data_ptr(), info.data_ptr(), s),
                   "arb_csv_split")
        mark(3)
        h = _info(info)
        if h["first_data_line"] < 0:
            return _empty(name, device)
        ncols, nrows = h["ncols"], h["nrows"]
        if h["ninvalid"]:
            raise ValueError(_invalid_message(nvals.cpu().numpy(), h["first_data_line"], ncols, skip_header))
        out = torch.empty((nrows, ncols), dtype=torch.float64, device=device)
        mark(4)
        _lib.check(L.arb_csv_parse(text.data_ptr(), nbytes, nlines, delim, comment, lw.data_ptr(), lw.numel(),
                                   nvals.data_ptr(), out.data_ptr(), nrows, ncols, info.data_ptr(), s),
                   "arb_csv_parse")
        mark(5)
        h = _info(info)
    if ev is not None:
        timing.update(count_ms=ev[0].elapsed_time(ev[1]), split_ms=ev[2].elapsed_time(ev[3]),
                      parse_ms=ev[4].elapsed_time(ev[5]))
    if h["error"]:
        raise RuntimeError(f"arb_csv_parse: exact conversion ran out of big-integer capacity ({h['error']})")
    if stats is not None:
        stats.update(h)
    return _squeeze(out)


def _empty(name, device):
    warnings.warn(f'genfromtxt: Empty input file: "{name}"', stacklevel=3)
    return torch.empty(0, dtype=torch.float64, device=device)


def _squeeze(out: torch.Tensor) -> torch.Tensor:
    # numpy's ndmin=0: every length-1 dimension is dropped
    return out.squeeze() if 1 in out.shape else out


def _invalid_message(nvals: np.ndarray, first: int, ncols: int, skip_header: int) -> str:
    bad = np.flatnonzero((nvals > 0) & (nvals != ncols))
    lines = [f"    Line #{int(l) - first + skip_header + 1} (got {int(nvals[l])} columns instead of {ncols})"
             for l in bad]
    return "\n".join(["Some errors were detected !", *lines])


def genfromtxt(fname, delimiter=",", comments="#", skip_header: int = 0, *, device=None,
               stats: dict | None = None) -> torch.Tensor:
    """``np.genfromtxt(fname, delimiter=..., comments=..., skip_header=...)``
    computed on the GPU; returns a CUDA float64 tensor.

    ``fname``: a path (str / PathLike), a bytes-like object holding the
    file's contents, a file object (read whole), or the text already on the
    device as a 1-D uint8 CUDA tensor.  ``stats``, when given,
    receives the reader's counters (lines, rows, tokens settled by the exact
    big-integer pass)."""
    if isinstance(fname, os.PathLike):
        fname = os.fspath(fname)
    if isinstance(fname, str):
        if fname.endswith((".gz", ".bz2", ".xz", ".zip", ".zst")):
            raise NotImplementedError(f"{fname}: compressed files are not read by the GPU reader")
        text, n = file_to_device(fname, device)
        name = fname
    elif isinstance(fname, torch.Tensor):
        if not (fname.is_cuda and fname.dtype == torch.uint8 and fname.dim() == 1):
            raise TypeError("a tensor input must be 1-D uint8 text on a CUDA device")
        n = fname.numel()
        text = fname if fname.data_ptr() % 16 == 0 else fname.clone()
        name = "<device text>"
    elif isinstance(fname, (bytes, bytearray, memoryview)):
        text, n = bytes_to_device(fname, device)
        name = "<bytes>"
    elif hasattr(fname, "read"):
        data = fname.read()
        if isinstance(data, str):
            data = data.encode("utf-8")       # non-ASCII text is then refused by the byte check
        text, n = bytes_to_device(data, device)
        name = getattr(fname, "name", "<file>")
    else:
        raise TypeError(f"fname must be a path, a bytes-like object or a file object, not {type(fname)}")
    return parse_device_text(text, n, delimiter, comments, skip_header, name=str(name), stats=stats)
