"""Many independent 3D interpolants evaluated in one persistent launch.

The reference builds one Python object per field and queries them one by
one.  `BatchedTricubic` ingests every field once, keeps their descriptors in
device memory, and evaluates the concatenated query sets of all fields with
`arb_batched_launch`: a persistent kernel whose CTAs take tiles of rows
from an atomic work counter, so fields of very different sizes share the GPU
without per-field launches.  `capture()` records the launch in a CUDA graph
for repeated evaluation with fixed buffers.

Tuning (`tune()`, run on first query unless given explicitly): the tile
size and, per field, the strategy — evaluate on the fly from the grid, or
build the field's coefficient table first and evaluate from it (worth it
when a field has many queries per cell).  Candidates are timed on the
caller's batch with CUDA events; a table's build is charged once per
`expected_reuse` evaluations.  The choice is cached like the single-field
autotuner's (same cache file).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib, autotune
from ._lib import ArbGrid, ArbQueryOut, lib, check
from .interp import _stream, tricubic

__all__ = ["BatchedTricubic"]

TILE_CHOICES = (256, 512, 1024, 2048)
TABLE_RATIOS = (None, 64.0, 8.0, 1.0)      # table when rows >= ratio * cells; None: never




class BatchedTricubic:
    """fields: sequence of N x 4 (scalar) or N x 6 rows (3D); kwargs as for
    `tricubic` (precision, mode, device)."""

    def __init__(self, fields, precision="mixed", mode=None, device=None):
        kw = {} if mode is None else {"mode": mode}
        self.precision = precision
        self.interps = [tricubic(f, "quiet", precision=precision, strategy="otf", device=device, **kw)
                        for f in fields]
        F = {o._F for o in self.interps}
        if len(F) != 1:
            raise ValueError("all fields of a batch must have the same kind (mode and column count)")
        self.F = F.pop()
        self.kind = self.interps[0]._kind
        self.device = self.interps[0].device
        self.tile_rows = None
        self.table_ratio = None
        self._desc = None
        self._status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self._counter = torch.zeros(1, dtype=torch.int64, device=self.device)

    # ---------------------------------------------------------------- plan
    def _upload(self):
        n = len(self.interps)
        arr = (ArbGrid * n)(*[o._g for o in self.interps])
        raw = bytes(memoryview(arr).cast("B"))
        self._desc = torch.frombuffer(bytearray(raw), dtype=torch.uint8).to(self.device)

    def _apply_strategy(self, counts, ratio):
        for o, n in zip(self.interps, counts):
            want = ratio is not None and n >= ratio * o.nc
            if want and not o._table_complete:
                o.allCoeffs()
            elif not want and o._table is not None:
                o._drop_table()
        self._upload()

    def _offsets(self, counts, tile_rows):
        counts = np.asarray(counts, dtype=np.int64)
        q_off = np.concatenate([[0], np.cumsum(counts)])
        tiles = (counts + tile_rows - 1) // tile_rows
        t_off = np.concatenate([[0], np.cumsum(tiles)])
        dev = self.device
        return (torch.tensor(q_off, device=dev), torch.tensor(t_off, device=dev), int(t_off[-1]))

    def _outputs(self, total):
        f64 = dict(dtype=torch.float64, device=self.device)
        comps = torch.empty((total, 3), **f64) if self.F >= 3 else None
        norms = torch.empty((total, 1), **f64) if self.F != 3 else None
        grads = torch.empty((total, 3), **f64) if self.F != 3 else None
        return comps, norms, grads

    def _launch(self, q, counts, tile_rows, outs, offsets=None):
        q_off, t_off, ntiles = offsets if offsets is not None else self._offsets(counts, tile_rows)
        comps, norms, grads = outs
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        out = ArbQueryOut(p(comps), p(norms), p(grads), None, None, None)
        prec = _lib.PREC_MIXED if self.precision == "mixed" else _lib.PREC_FP64
        check(lib().arb_batched_launch(self._desc.data_ptr(), len(self.interps), self.F, q_off.data_ptr(),
                                       t_off.data_ptr(), ntiles, tile_rows, prec, q.data_ptr(), q.shape[1],
                                       0, out, self._counter.data_ptr(), self._status.data_ptr(), _stream()),
              "arb_batched_launch")
        return (q_off, t_off, ntiles)

    def tune(self, q, counts, expected_reuse=1):
        """Pick the tile size and table threshold for this batch by timing."""
        key = (f"batched|{torch.cuda.get_device_name(self.device)}|{self.precision}|F{self.F}|"
               f"n{len(self.interps)}|rows2^{int(np.log2(max(int(np.sum(counts)), 1)))}|reuse{expected_reuse}")
        cached = autotune._MEM.get(key) or autotune._load().get(key)
        if cached:
            self.tile_rows, self.table_ratio = cached["tile_rows"], cached["table_ratio"]
            self._apply_strategy(counts, self.table_ratio)
            return cached
        total = int(np.sum(counts))
        outs = self._outputs(total)
        best = None
        for ratio in TABLE_RATIOS:
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            self._apply_strategy(counts, ratio)
            e.record()
            torch.cuda.synchronize()
            build_ms = s.elapsed_time(e)
            for tr in TILE_CHOICES:
                offs = self._offsets(counts, tr)
                self._launch(q, counts, tr, outs, offs)
                s.record()
                for _ in range(2):
                    self._launch(q, counts, tr, outs, offs)
                e.record()
                torch.cuda.synchronize()
                t = s.elapsed_time(e) / 2 + build_ms / max(expected_reuse, 1)
                if best is None or t < best["ms"]:
                    best = {"tile_rows": tr, "table_ratio": ratio, "ms": round(t, 4)}
        self.tile_rows, self.table_ratio = best["tile_rows"], best["table_ratio"]
        self._apply_strategy(counts, self.table_ratio)
        autotune._MEM[key] = best
        autotune._store(key, best)
        return best

    # ---------------------------------------------------------------- query
    def query(self, q, counts):
        """q: (sum(counts), >=3) float64 CUDA tensor, field f's rows after
        field f-1's.  Returns concatenated device outputs: comps (vector,
        both), norms and grads (scalar, norm, both)."""
        if q.dtype != torch.float64 or not q.is_cuda:
            q = q.to(device=self.device, dtype=torch.float64)
        q = q.contiguous()
        if self.tile_rows is None:
            self.tune(q, counts)
        if self._desc is None:
            self._upload()
        outs = self._outputs(q.shape[0])
        self._launch(q, counts, self.tile_rows, outs)
        st = lib().arb_status_fetch(self._status.data_ptr(), _stream())
        if st & _lib.ARB_ERR_CELL_INDEX:
            raise IndexError("cell index beyond the coefficient table (query on an upper face)")
        return tuple(t for t in outs if t is not None)

    def capture(self, q, counts):
        """Record one batched evaluation of q in a CUDA graph.  Returns
        (graph, outputs): graph.replay() re-evaluates the current contents of
        q (same shape) into the same output tensors."""
        q = q.contiguous()
        if self.tile_rows is None:
            self.tune(q, counts)
        if self._desc is None:
            self._upload()
        outs = self._outputs(q.shape[0])
        offs = self._offsets(counts, self.tile_rows)
        self._launch(q, counts, self.tile_rows, outs, offs)            # warm-up outside capture
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self._launch(q, counts, self.tile_rows, outs, offs)
        self._graph_keep = (q, outs, offs)
        return g, tuple(t for t in outs if t is not None)
