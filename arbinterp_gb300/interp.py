"""GB300-native drop-in for ``ARBInterp.tricubic`` / ``ARBInterp.quadcubic``.

Mirrors the reference class API (src/ARBInterp/ARBInterp.py:8-621 and
627-1381): constructor ``cls(field, *args, **kwargs)`` on an N x 4/6 (3D) or
N x 5/7 (4D) row array in any row order, ``'quiet'`` among the positional
args, ``mode='vector'|'norm'|'both'``; ``Query``/``rQuery``/``sQuery``,
``allCoeffs``, ``calcCoefficients``, ``neighbourInd`` and the public
attributes.  All arithmetic runs in CUDA kernels of ``libarbinterp.so``;
torch is used only for device memory and streams.

Extra keyword arguments (reference-compatible defaults):
  precision  'fp64' (default; matches the reference to <=1e-12) or 'mixed'
             (split-precision tensor-core / float32 evaluation, <=1e-6)
  strategy   'auto' (default), 'otf' (evaluate from the grid) or 'table'
             (evaluate from the full coefficient table)
  device     CUDA device (default: the current one)
  check      True (default): synchronise after each query to raise the
             reference's errors; False: fully asynchronous device queries
  sort_threshold
             row count from which queries are grouped by spatial bin before
             evaluation (default 32768)

Inputs may be NumPy arrays (outputs are NumPy, as in the reference) or torch
CUDA tensors (outputs stay on the device).  Differences from the reference on
inputs it does not handle: rows that are not a full regular grid raise
ValueError instead of producing undefined results.
"""
from __future__ import annotations

import ctypes
import sys
import threading

import numpy as np
import torch

from . import _lib
from . import autotune
from . import matrices
from ._lib import ArbGrid, ArbQueryOut, lib, check

__version__ = "1.8"

_F = {_lib.KIND_SCALAR: 1, _lib.KIND_VECTOR: 3, _lib.KIND_NORM: 1, _lib.KIND_BOTH: 4}
_AXIS_CAP = 1 << 17
_ORDERED_INGEST = True      # try the single-pass ingest for rows in meshgrid order first
# host (NumPy) range queries of at least this many rows are uploaded, evaluated
# and downloaded chunk by chunk on overlapping streams
PIPELINE_MIN_ROWS = 1 << 21
PIPELINE_MIN_CHUNK_ROWS = 1 << 20
PIPELINE_MAX_CHUNKS = 8
_COPY_STREAMS: dict = {}
_PER_THREAD = threading.local()


def _probe_summary_slot(device):
    """(pinned host buffer of the 17-double ingest summary, event) for this
    thread and device, made once: the summary kernel writes the buffer in
    place (pinned host memory is addressable from the device), so
    construction needs no device buffer and no copy, and waits on the event."""
    key = torch.device(device).index
    slots = getattr(_PER_THREAD, "summary", None)
    if slots is None:
        slots = _PER_THREAD.summary = {}
    if key not in slots:
        slots[key] = (torch.empty(17, dtype=torch.float64, pin_memory=True), torch.cuda.Event())
    return slots[key]


def _copy_streams(device):
    """(copy-in, copy-out) side streams of a device, created once."""
    key = torch.device(device).index
    if key not in _COPY_STREAMS:
        _COPY_STREAMS[key] = (torch.cuda.Stream(device), torch.cuda.Stream(device))
    return _COPY_STREAMS[key]

_BANNERS = {
    "scalar": "--- Scalar field, ignoring switches, interpolating for magnitude and gradient --- \n",
    "vector": "--- Vector field, interpolating for vector components --- \n",
    "norm": "--- Vector field, interpolating for magnitude and gradient --- \n",
    "both": "--- Vector field, interpolating vector components plus magnitude and gradient --- \n",
    "invalid": "--- Vector field, invalid option, defaulting to interpolating for vector components --- \n",
    "none": "--- Vector field, no option selected, defaulting to interpolating for vector components --- \n",
}


def _ptr(t):
    return None if t is None else t.data_ptr()


def _nan_rows(qa, rows):
    """qa[rows] = NaN for a host array qa and a CPU int64 tensor of row
    indices: through torch's multithreaded index_fill_ on a view of qa when
    it is a C-contiguous float array (numpy's row-wise fancy assignment is
    about five times slower for 1e5 scattered rows), else by numpy."""
    if qa.dtype in (np.float32, np.float64) and qa.flags.c_contiguous and qa.flags.writeable:
        torch.from_numpy(qa).index_fill_(0, rows, float("nan"))
    else:
        qa[rows.numpy()] = np.nan


if hasattr(torch._C, "_cuda_getCurrentRawStream") and hasattr(torch._C, "_cuda_getDevice"):
    def _stream():
        """The current CUDA stream of the current device, as a raw handle
        (one C call: torch.cuda.current_stream() costs ~15 us of Python per
        call, several times per query)."""
        return torch._C._cuda_getCurrentRawStream(torch._C._cuda_getDevice())
else:  # pragma: no cover
    def _stream():
        return torch.cuda.current_stream().cuda_stream


class _Interpolant:
    __version__ = "1.8"
    _dim = 3

    def __init__(self, field, *args, **kwargs):
        self.eps = 10 * np.finfo(float).eps
        quiet = "quiet" in args
        dim = self._dim
        prec = kwargs.get("precision", "fp64")
        if prec not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = prec
        self.strategy = kwargs.get("strategy", "auto")
        if self.strategy not in ("auto", "otf", "table"):
            raise ValueError("strategy must be 'auto', 'otf' or 'table'")
        self.check = bool(kwargs.get("check", True))
        self.sort_threshold = int(kwargs.get("sort_threshold", 1 << 15))
        self._ws = None
        ncol = int(field.shape[1])
        # mode dispatch (ARB:24-104, 641-723)
        extra_col = False
        sentinel_nan = True
        if ncol == dim + 1:
            kind, banner = _lib.KIND_SCALAR, "scalar"
            sentinel_nan = False
        elif ncol == dim + 3:
            if "mode" in kwargs:
                m = kwargs["mode"]
                if m == "vector":
                    kind, banner, extra_col, sentinel_nan = _lib.KIND_VECTOR, "vector", True, False
                elif m == "norm":
                    kind, banner = _lib.KIND_NORM, "norm"
                elif m == "both":
                    kind, banner = _lib.KIND_BOTH, "both"
                else:
                    kind, banner = _lib.KIND_VECTOR, "invalid"
            else:
                kind, banner = _lib.KIND_VECTOR, "none"
        else:
            lo, hi = (4, 6) if dim == 3 else (5, 7)
            sys.exit(f"--- Input not shaped as expected - should be N x {lo} or N x {hi} ---")
        dev = kwargs.get("device", None)
        self.device = torch.device("cuda", torch.cuda.current_device()) if dev is None else torch.device(dev)
        self._kind = kind
        self._F = _F[kind]
        self._extra_col = extra_col
        self._sentinel_nan = sentinel_nan
        bc = kwargs.get("boundary", None)
        if bc is not None:
            if bc not in ("neumann", "dirichlet"):
                raise ValueError("boundary must be None, 'neumann' or 'dirichlet'")
            field = self._pad_field(field, bc)
        self.boundary = bc
        self._ingest(field)
        if not quiet:
            print(_BANNERS[banner])
        self._table = None
        self._table_prec = None
        self._solved = None          # host bool mask of solved cells (partial solves)
        self._last_inds = None
        self._last_ind = None
        self.last_plan = None

    # ------------------------------------------------------------------ ingest
    def _pad_field(self, field, bc):
        """Field rows extended by one ghost layer on every face, so that the
        interpolation volume becomes the whole input grid (the reference
        loses one cell layer per face; README.md "Further work will implement
        boundary conditions of the Neumann or Dirichlet types").
        'neumann': zero normal derivative at the boundary node, ghost = mirror
        image of the first interior node (f[-1] = f[1]); 'dirichlet': the
        boundary samples are the prescribed values, continued by odd
        reflection (f[-1] = 2 f[0] - f[1], zero second difference at the
        boundary node).  Ghost coordinates continue the axis spacing."""
        dim = self._dim
        dev = self.device
        ft = field if isinstance(field, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(np.asarray(field)))
        dtype = ft.dtype if ft.dtype in (torch.float32, torch.float64) else torch.float64
        ncol = int(ft.shape[1])
        nval = ncol - dim
        # sorted samples and axes from a float64 interpolant of the raw value columns
        kw = {} if nval == 1 else {"mode": "vector"}
        base = type(self)(ft.to(dev, torch.float64), "quiet", precision="fp64", **kw)
        n = base._n
        vals = base._grid64.view(*reversed(n), nval)          # (t,) z, y, x, value
        axes = [base._axes_dev[a].to(torch.float64) for a in range(dim)]
        for a in range(dim):                                    # pad axis a (tensor dim dim-1-a)
            d = dim - 1 - a
            lo_i, hi_i = vals.narrow(d, 1, 1), vals.narrow(d, n[a] - 2, 1)
            if bc == "neumann":
                g_lo, g_hi = lo_i, hi_i
            else:
                g_lo = 2.0 * vals.narrow(d, 0, 1) - lo_i
                g_hi = 2.0 * vals.narrow(d, n[a] - 1, 1) - hi_i
            vals = torch.cat([g_lo, vals, g_hi], d)
            ax = axes[a]
            h = ax[1] - ax[0]
            axes[a] = torch.cat([ax[:1] - h, ax, ax[-1:] + (ax[-1] - ax[-2])])
        mesh = torch.meshgrid(*reversed(axes), indexing="ij")   # slowest first, x fastest
        cols = [mesh[dim - 1 - a].reshape(-1) for a in range(dim)]
        rows = torch.cat([torch.stack(cols, 1), vals.reshape(-1, nval)], 1).to(dtype)
        del base
        return rows if isinstance(field, torch.Tensor) else rows.cpu().numpy()

    def _ingest(self, field):
        L = lib()
        dim = self._dim
        dev = self.device
        if isinstance(field, torch.Tensor):
            ft = field.to(dev)
        else:
            fa = np.asarray(field)
            if fa.dtype not in (np.float32, np.float64):
                fa = fa.astype(np.float64)
            ft = torch.from_numpy(np.ascontiguousarray(fa)).to(dev, non_blocking=True)
        if ft.dtype not in (torch.float32, torch.float64):
            ft = ft.to(torch.float64)
        ft = ft.contiguous()
        self._field_dtype = np.float32 if ft.dtype == torch.float32 else np.float64
        npts, ncol = int(ft.shape[0]), int(ft.shape[1])
        is32 = int(ft.dtype == torch.float32)
        cap = max(4, min(npts, _AXIS_CAP))
        axes = torch.empty(2 * dim * cap, dtype=torch.float64, device=dev)
        counts = torch.empty(dim, dtype=torch.int64, device=dev)   # written by the probe or the axis pass
        wb = L.arb_ingest_axes_work_bytes(dim)
        work = torch.empty(int(wb), dtype=torch.uint8, device=dev)
        status = torch.empty(1, dtype=torch.int32, device=dev)
        s = _stream()
        check(L.arb_status_clear(status.data_ptr(), s), "arb_status_clear")
        kind, F = self._kind, self._F
        # Mixed precision with the caller's own CUDA tensor: the float64 grid is
        # not needed by the float32 query path and is produced on first use from
        # that tensor (if it is still unmodified) instead of on every construction.
        lazy64 = (self.precision == "mixed" and isinstance(field, torch.Tensor)
                  and ft.data_ptr() == field.data_ptr())
        self._src = (ft, ft._version, is32, ncol) if lazy64 else None

        def grids():
            # allocated once the probe is queued (the GPU starts on it meanwhile)
            g64 = None if lazy64 else torch.empty(npts * F, dtype=torch.float64, device=dev)
            # mixed-precision grid: F=1 (hi, lo); F=3 float4 of hi; F=4 float4 of hi + lo of |B|
            g32 = (torch.empty(npts * {1: 2, 3: 4, 4: 5}[F], dtype=torch.float32, device=dev)
                   if self.precision == "mixed" else None)
            r = (torch.empty(npts * 3, dtype=torch.float64, device=dev)
                 if kind == _lib.KIND_NORM and not lazy64 else None)
            return g64, g32, r

        grid64 = grid32 = raw = None
        self._status = status
        self._fill_pending = False
        self._fill_src = None
        done = False
        if _ORDERED_INGEST and npts < 0xFFFFFFFF:
            # rows in meshgrid order (the common case): one pass, no sort.  The
            # host waits for the single-block axis probe only (its summary
            # arrives in pinned memory behind an event); the pass that writes
            # the grid runs while the host sets up and the first query is
            # queued, and its row check is read at the next synchronisation
            # (_settle), before any result derived from the grid is returned.
            check(L.arb_ingest_ordered_probe(ft.data_ptr(), is32, npts, ncol, dim, kind, cap, axes.data_ptr(),
                                             counts.data_ptr(), work.data_ptr(), wb, status.data_ptr(), s),
                  "arb_ingest_ordered_probe")
            summ_h, ev = _probe_summary_slot(dev)
            check(L.arb_ingest_summary(axes.data_ptr(), cap, counts.data_ptr(), dim, status.data_ptr(),
                                       summ_h.data_ptr(), s), "arb_ingest_summary")
            ev.record()
            grid64, grid32, raw = grids()
            check(L.arb_ingest_ordered_fill(ft.data_ptr(), is32, npts, ncol, dim, kind, cap, axes.data_ptr(),
                                            work.data_ptr(), wb, _ptr(grid64), _ptr(grid32), _ptr(raw),
                                            status.data_ptr(), s), "arb_ingest_ordered_fill")
            ev.synchronize()
            sm = summ_h.numpy().copy()
            done = int(sm[0]) == 0
            if done:
                self._fill_pending = True
                self._fill_src = (ft, is32, npts, ncol, cap, axes, counts, work, wb, grid64, grid32, raw)
        if not done:
            if grid32 is None and grid64 is None:
                grid64, grid32, raw = grids()
            sm = self._ingest_general(ft, is32, npts, ncol, cap, axes, counts, work, wb, grid64, grid32, raw)
        n = [int(sm[1 + a]) for a in range(dim)]
        ax64 = axes[: dim * cap].view(dim, cap)
        self._axes_dev = [ax64[a, : n[a]] for a in range(dim)]
        self._n = n
        self._npts = npts
        self._ingest_path = "ordered" if done else "general"
        self._grid64_t, self._grid32_t, self._raw_t = grid64, grid32, raw
        self._ingest_ordered = done
        # reference attributes, computed in the field's own dtype (ARB:541-568)
        dt = self._field_dtype
        h = [np.abs(dt(sm[5 + 3 * a]) - dt(sm[6 + 3 * a])) for a in range(dim)]
        lo = [dt(sm[6 + 3 * a]) for a in range(dim)]
        hi = [dt(sm[7 + 3 * a]) for a in range(dim)]
        self._h, self._lo, self._hi = h, lo, hi
        names = "xyzt"
        for a in range(dim):
            setattr(self, "h" + names[a], h[a])
            setattr(self, names[a] + "IntMin", lo[a])
            setattr(self, names[a] + "IntMax", hi[a])
        self.nc = int(np.prod([v - 3 for v in n]))
        self._set_counts(n)
        g = ArbGrid()
        g.dim = dim
        g.kind = kind
        g.nfield = F
        g.sentinel_nan = int(self._sentinel_nan)
        for a in range(4):
            g.n[a] = n[a] if a < dim else 1
            g.lo[a] = float(lo[a]) if a < dim else 0.0
            g.hi[a] = float(hi[a]) if a < dim else 0.0
            g.h[a] = float(h[a]) if a < dim else 1.0
        g.nc = self.nc
        g.grid64 = _ptr(grid64)
        g.grid32 = _ptr(grid32)
        g.table = None
        g.table_prec = 0
        self._gs = g

    def _ingest_general(self, ft, is32, npts, ncol, cap, axes, counts, work, wb, grid64, grid32, raw):
        """Rows in any order: axis scan, rank sort and scatter (ARB:528-568);
        returns the ingest summary, raises ValueError for a field that is not
        a full regular grid."""
        L = lib()
        dim, dev, kind, s = self._dim, self.device, self._kind, _stream()
        status = self._status
        summ = torch.empty(17, dtype=torch.float64, device=dev)
        ax64 = axes[: dim * cap].view(dim, cap)
        check(L.arb_ingest_axes(ft.data_ptr(), is32, npts, ncol, dim, cap, axes.data_ptr(),
                                counts.data_ptr(), work.data_ptr(), wb, status.data_ptr(), s),
              "arb_ingest_axes")
        st = L.arb_status_fetch(status.data_ptr(), s)
        n = [int(v) for v in counts.cpu()]
        if st & _lib.ARB_ERR_CAPACITY:
            raise ValueError(f"an axis has more than {cap} grid samples")
        if st:
            raise ValueError("field rows are not a regular grid (NaN coordinates or duplicate points)")
        if any(v < 4 for v in n):
            raise ValueError("every axis needs at least 4 grid points")
        if int(np.prod(n)) != npts:
            raise ValueError(f"field rows do not form a full regular grid: {npts} rows, axes {n}")
        claim = torch.empty(npts, dtype=torch.int32, device=dev)
        n_c = (ctypes.c_int64 * 4)(*(n + [1] * (4 - dim)))
        check(L.arb_ingest_scatter(ft.data_ptr(), is32, npts, ncol, dim, ax64.data_ptr(), cap,
                                   n_c, kind, _ptr(grid64), _ptr(grid32), _ptr(raw),
                                   claim.data_ptr(), status.data_ptr(), s), "arb_ingest_scatter")
        check(L.arb_ingest_summary(axes.data_ptr(), cap, counts.data_ptr(), dim, status.data_ptr(),
                                   summ.data_ptr(), s), "arb_ingest_summary")
        sm = summ.cpu().numpy()
        if self.check and int(sm[0]):
            raise ValueError("field rows are not a full regular grid (duplicate or off-axis points)")
        return sm

    def _settle(self):
        """Wait for a single-pass grid fill still in flight and read its row
        check (see _settle_status)."""
        if self._fill_pending:
            self._settle_status(lib().arb_status_fetch(self._status.data_ptr(), _stream()))

    def _settle_status(self, st):
        """Close the single-pass fill given the status word read after it.
        If a row was not where meshgrid order puts it, the general ingest
        rewrites the grid (or raises ValueError for a field that is no full
        regular grid).  The geometry stays: when the probe's lines through
        row 0 hold n_a strictly monotone samples per axis with prod n_a rows,
        a full grid's axes hold exactly those samples.  Returns True when the
        grid was rewritten (results computed from it before are void)."""
        self._fill_pending = False
        src, self._fill_src = self._fill_src, None
        if not st & _lib.ARB_ERR_IRREGULAR_GRID:
            return False
        n_probe = list(self._n)
        sm = self._ingest_general(*src)
        if [int(sm[1 + a]) for a in range(self._dim)] != n_probe:
            raise RuntimeError("the general ingest found other axes than the single-pass probe")
        self._ingest_ordered = False
        self._ingest_path = "general"
        return True

    @property
    def _g(self):
        """The arb_grid descriptor, once the grid is written and checked."""
        if self._fill_pending:
            self._settle()
        return self._gs

    @property
    def _grid32(self):
        if self._fill_pending:
            self._settle()
        return self._grid32_t

    @property
    def ingest_path(self):
        """'ordered' (rows in meshgrid order, single pass) or 'general'."""
        if self._fill_pending:
            self._settle()
        return self._ingest_path

    @property
    def _grid64(self):
        """[npts*F] float64 grid values (produced on first use in the lazy case)."""
        if self._fill_pending:
            self._settle()
        if self._grid64_t is None:
            self._materialise_grid64()
        return self._grid64_t

    @property
    def _raw(self):
        if self._fill_pending:
            self._settle()
        if self._grid64_t is None and self._src is not None:
            self._materialise_grid64()
        return self._raw_t

    def _materialise_grid64(self):
        ft, version, is32, ncol = self._src
        if ft._version != version:
            raise RuntimeError("the field tensor was modified in place after this mixed-precision interpolant "
                               "was built; its float64 grid values are no longer available")
        L = lib()
        dim, npts, F, dev = self._dim, self._npts, self._F, self.device
        s = _stream()
        grid64 = torch.empty(npts * F, dtype=torch.float64, device=dev)
        raw = torch.empty(npts * 3, dtype=torch.float64, device=dev) if self._kind == _lib.KIND_NORM else None
        cap = max(4, min(npts, _AXIS_CAP))
        axes = torch.empty(2 * dim * cap, dtype=torch.float64, device=dev)
        counts = torch.zeros(dim, dtype=torch.int64, device=dev)
        wb = L.arb_ingest_axes_work_bytes(dim)
        work = torch.empty(int(wb), dtype=torch.uint8, device=dev)
        if self._ingest_ordered:
            check(L.arb_ingest_ordered(ft.data_ptr(), is32, npts, ncol, dim, self._kind, cap, axes.data_ptr(),
                                       counts.data_ptr(), grid64.data_ptr(), None, _ptr(raw), work.data_ptr(),
                                       wb, self._status.data_ptr(), s), "arb_ingest_ordered")
        else:
            check(L.arb_ingest_axes(ft.data_ptr(), is32, npts, ncol, dim, cap, axes.data_ptr(),
                                    counts.data_ptr(), work.data_ptr(), wb, self._status.data_ptr(), s),
                  "arb_ingest_axes")
            claim = torch.empty(npts, dtype=torch.int32, device=dev)
            n_c = (ctypes.c_int64 * 4)(*(self._n + [1] * (4 - dim)))
            check(L.arb_ingest_scatter(ft.data_ptr(), is32, npts, ncol, dim, axes.data_ptr(), cap, n_c,
                                       self._kind, grid64.data_ptr(), None, _ptr(raw), claim.data_ptr(),
                                       self._status.data_ptr(), s), "arb_ingest_scatter")
        if L.arb_status_fetch(self._status.data_ptr(), s):
            raise RuntimeError("re-reading the field for its float64 grid values failed")
        self._grid64_t, self._raw_t = grid64, raw
        self._g.grid64 = grid64.data_ptr()

    def _set_counts(self, n):
        raise NotImplementedError

    # ------------------------------------------------------------ coefficients
    @property
    def _M(self):
        return 4 ** self._dim

    def _ensure_table(self):
        if self._table is None:
            dt = torch.float64 if self.precision == "fp64" else torch.float32
            self._table = torch.zeros(self.nc * self._F * self._M, dtype=dt, device=self.device)
            self._table_prec = _lib.PREC_FP64 if self.precision == "fp64" else _lib.PREC_MIXED
            self._g.table = self._table.data_ptr()
            self._g.table_prec = self._table_prec
            self._solved = np.zeros(self.nc, dtype=bool)

    def _solve(self, cell0, ncells):
        self._ensure_table()
        if self.precision != "mixed":
            self._grid64                      # the float64 grid (materialised if needed)
        L = lib()
        rc = L.arb_coef_solve(self._g, self._table_prec, cell0, ncells,
                              self._table.data_ptr() + cell0 * self._F * self._M * self._table.element_size(),
                              self._status.data_ptr(), _stream())
        check(rc, "arb_coef_solve")
        if self.precision == "mixed":
            # the tensor-core solve reports a bounded device wait that ran out
            # in the status word; its rows are then not trustworthy
            st = self._fetch_status()
            if st & _lib.ARB_ERR_TIMEOUT:
                raise RuntimeError("arb_coef_solve: " + _lib.describe(st))
        self._solved[cell0:cell0 + ncells] = True

    def allCoeffs(self):
        """Solve every cell's coefficients (ARB:523-525, 1260-1262)."""
        self._solve(0, self.nc)

    def _table_meta(self):
        """Geometry, precision and a checksum of the grid values a table belongs to."""
        src = self._grid32 if self.precision == "mixed" else self._grid64
        v = src.to(torch.float64)
        w = torch.arange(1, v.numel() + 1, dtype=torch.float64, device=v.device) / v.numel()
        checks = torch.stack([v.sum(), (v * v).sum(), (v * w).sum()]).cpu().numpy()
        return {"dim": self._dim, "kind": self._kind, "nfield": self._F, "precision": self.precision,
                "n": np.array(self._n, dtype=np.int64),
                "lo": np.array(self._lo, dtype=np.float64), "hi": np.array(self._hi, dtype=np.float64),
                "h": np.array(self._h, dtype=np.float64), "checks": checks}

    def save_coefficients(self, path):
        """Write the whole coefficient table (solving it first if needed) to
        `path` (NumPy .npz): the cell-major table [nc][F][4^dim] in this
        interpolant's precision, plus the grid geometry and a checksum of the
        grid values (the reference's planned "save these coefficients to a
        file for later use", CHANGELOG.md v1.8.0)."""
        if not self._table_complete:
            self.allCoeffs()
        np.savez(path, table=self._table.cpu().numpy(), **self._table_meta())

    def load_coefficients(self, path):
        """Load a table written by `save_coefficients` for the same field
        (geometry, mode, precision and grid values must match; ValueError
        otherwise).  Later queries with strategy 'auto' or 'table' use it."""
        d = np.load(path)
        meta = self._table_meta()
        for k in ("dim", "kind", "nfield", "n", "lo", "hi", "h"):
            if not np.array_equal(np.asarray(d[k]), np.asarray(meta[k])):
                raise ValueError(f"coefficient file does not match this interpolant ({k} differs)")
        if str(d["precision"]) != self.precision:
            raise ValueError(f"coefficient file holds a {d['precision']} table; this interpolant is {self.precision}")
        if not np.allclose(d["checks"], meta["checks"], rtol=1e-12, atol=0):
            raise ValueError("coefficient file was solved from different grid values")
        t = d["table"]
        if t.size != self.nc * self._F * self._M:
            raise ValueError("coefficient file has the wrong table size")
        self._ensure_table()
        self._table.copy_(torch.from_numpy(t.reshape(-1)))
        self._solved[:] = True

    def calcCoefficients(self, alphaindex):
        """Solve one cell (ARB:570-603, 1322-1355)."""
        i = int(alphaindex)
        if 0 <= i < self.nc and (self._solved is None or not self._solved[i]):
            self._solve(i, 1)

    @property
    def _table_complete(self):
        return self._solved is not None and bool(self._solved.all())

    # ------------------------------------------------------------------ queries
    def _plan(self, qd, n, qs):
        """Strategy for this batch: forced by `strategy`, else the autotuner."""
        if self.strategy == "table":
            if not self._table_complete:
                self.allCoeffs()
            return {"table": True, "binned": n >= self.sort_threshold, "bin_shift": 0}
        if self.strategy == "otf":
            return {"table": False, "binned": n >= self.sort_threshold, "bin_shift": 0}
        return autotune.choose(self, qd, n, qs)

    def _use_table(self):
        return self.strategy == "table" or (self.strategy == "auto" and self._table_complete)

    def _drop_table(self):
        self._table = None
        self._table_prec = None
        self._solved = None
        self._g.table = None

    def _row_layout(self):
        """Interleaved output rows: (doubles per row, comps col, norm col, grads col);
        both mode (cx cy cz |B| gx gy gz [gt]), scalar/norm (v gx gy gz [gt ...]),
        vector (cx cy cz -).  One row is one or two 32-byte sectors."""
        dim, kind = self._dim, self._kind
        if kind == _lib.KIND_BOTH:
            return 8, 0, 3, 4
        if kind == _lib.KIND_VECTOR:
            return 4, 0, None, None
        return (4 if dim == 3 else 8), None, 0, 1

    def _packed_layout(self):
        """Rows holding only what the caller receives (no padding column):
        the layout downloaded to host arrays."""
        dim, kind = self._dim, self._kind
        if kind == _lib.KIND_BOTH:
            return 3 + 1 + dim, 0, 3, 4
        if kind == _lib.KIND_VECTOR:
            return 3, 0, None, None
        return 1 + dim, None, 0, 1

    def _outputs(self, n, want_oob, packed=False):
        dev = self.device
        dim = self._dim
        R, ci, ni, gi = self._packed_layout() if packed else self._row_layout()
        rows = torch.empty((n, R), dtype=torch.float64, device=dev)
        comps = rows[:, ci:ci + 3] if ci is not None else None
        norms = rows[:, ni:ni + 1] if ni is not None else None
        grads = rows[:, gi:gi + dim] if gi is not None else None
        inds = torch.empty(n, dtype=torch.int64, device=dev)
        oob = torch.empty(n, dtype=torch.int64, device=dev) if want_oob else None
        cnt = torch.zeros(1, dtype=torch.int64, device=dev) if want_oob else None
        return comps, norms, grads, inds, oob, cnt

    def _launch(self, qd, n, qs, writeback, want_oob, plan, res=None):
        """Launch one evaluation of device rows qd with a given plan (into
        the preallocated outputs res when given).  Does not wait for a
        single-pass grid fill still in flight (the launches queue behind it);
        the caller settles it at its next synchronisation."""
        L = lib()
        if res is None:
            res = self._outputs(n, want_oob)
        comps, norms, grads, inds, oob, cnt = res
        R = (comps if comps is not None else norms).stride(0)
        out = ArbQueryOut(_ptr(comps), _ptr(norms), _ptr(grads), _ptr(inds), _ptr(oob), _ptr(cnt), R, R, R)
        s = _stream()
        table = bool(plan["table"])
        prec = _lib.PREC_FP64 if self.precision == "fp64" else _lib.PREC_MIXED
        if plan["binned"]:
            # group queries by spatial bin first (cell-coherent gathers)
            self._gs.bin_shift = int(plan.get("bin_shift", 0))
            need = int(L.arb_query_sorted_work_bytes(self._gs, prec, n))
            if self._ws is None or self._ws.numel() < need:
                self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
            rc = L.arb_query_eval_sorted(self._gs, prec, int(table), qd.data_ptr(), n, qs, int(writeback),
                                         out, self._ws.data_ptr(), need, self._status.data_ptr(), s)
        elif table:
            rc = L.arb_query_eval(self._gs, qd.data_ptr(), n, qs, int(writeback), out,
                                  self._status.data_ptr(), s)
        else:
            rc = L.arb_query_eval_otf(self._gs, prec, qd.data_ptr(), n, qs, int(writeback), out,
                                      self._status.data_ptr(), s)
        check(rc, "query evaluation")
        return res

    def _run(self, qd, n, qs, writeback, want_oob):
        """Evaluate device rows qd with the planned strategy; returns device outputs."""
        plan = self._plan(qd, n, qs)
        self.last_plan = plan
        return self._launch(qd, n, qs, writeback, want_oob, plan)

    def _fetch_status(self):
        return lib().arb_status_fetch(self._status.data_ptr(), _stream())

    def _pack(self, comps, norms, grads):
        k = self._kind
        if k == _lib.KIND_VECTOR:
            return comps
        if k == _lib.KIND_BOTH:
            return comps, norms, grads
        return norms, grads

    def rQuery(self, query):
        """Range query (rQuery1/2/3, ARB:344-521 / 1064-1258).  Rows outside
        the interpolation volume come back NaN and are overwritten with NaN
        in the caller's array, as the reference does."""
        dim = self._dim
        if isinstance(query, torch.Tensor) and query.is_cuda:
            n, qs = int(query.shape[0]), int(query.shape[1])
            if qs < dim:
                raise IndexError("query rows need at least %d columns" % dim)
            direct = query.dtype == torch.float64 and query.is_contiguous()
            qd = query if direct else query.to(torch.float64).contiguous()
            res = self._run(qd, n, qs, True, False)
            if self.check or self._fill_pending:
                st = self._fetch_status()
                if self._fill_pending and self._settle_status(st):
                    # the grid was rewritten by the general ingest: evaluate
                    # again (rows already written back; indices of the first run)
                    st &= ~_lib.ARB_ERR_IRREGULAR_GRID
                    self._launch(qd, n, qs, False, False, self.last_plan,
                                 res=(res[0], res[1], res[2], None, None, None))
                    st |= self._fetch_status()
                if self.check and st & _lib.ARB_ERR_CELL_INDEX:
                    if not direct:
                        query.copy_(qd.to(query.dtype))
                    self._last_inds = res[3]
                    raise IndexError("cell index beyond the coefficient table (query on an upper face)")
            if not direct:
                query.copy_(qd.to(query.dtype))
            self._last_inds = res[3]
            return self._pack(*res[:3])
        qa = query if isinstance(query, np.ndarray) else np.asarray(query)
        n, qs = int(qa.shape[0]), int(qa.shape[1])
        if qs < dim:
            raise IndexError("query rows need at least %d columns" % dim)
        qc = np.ascontiguousarray(qa, dtype=np.float64)
        if n >= PIPELINE_MIN_ROWS:
            return self._rquery_host_pipelined(qa, qc, n, qs)
        self._settle()
        qd = torch.from_numpy(qc).to(self.device, non_blocking=True)
        comps, norms, grads, inds, oob, cnt = self._run(qd, n, qs, False, True)
        # one copy of the interleaved rows; the outputs are column views of it
        rows = (comps if comps is not None else norms)._base
        hrows = torch.empty(rows.shape, dtype=rows.dtype, pin_memory=True)
        hrows.copy_(rows, non_blocking=True)
        R, ci, ni, gi = self._row_layout()
        host = [None if c is None else hrows[:, c:c + w] for c, w in ((ci, 3), (ni, 1), (gi, dim))]
        st = self._fetch_status()          # synchronises the stream
        nbad = int(cnt.item())
        if nbad:
            _nan_rows(qa, oob[:nbad].cpu())  # in-place on the caller's array
        self._last_inds = inds
        if st & _lib.ARB_ERR_CELL_INDEX:
            raise IndexError("cell index beyond the coefficient table (query on an upper face)")
        out = [None if h is None else h.numpy() for h in host]
        return self._pack(*out)

    def _rquery_host_pipelined(self, qa, qc, n, qs):
        """rQuery of a large host array in chunks: every chunk's upload is
        queued on a copy-in stream, each chunk is binned and evaluated on the
        current stream as soon as it has arrived, and its output rows go back
        on a copy-out stream (the other direction of the link) while later
        chunks upload and evaluate.  Results, in-place NaN rows and
        queryInds are those of the single-shot path.  A single-pass grid fill
        still in flight is not waited for: the uploads start at once, the
        evaluations queue behind the fill, and its row check is read with the
        status at the end."""
        dev = self.device
        K = max(2, min(PIPELINE_MAX_CHUNKS, n // PIPELINE_MIN_CHUNK_ROWS))
        bounds = [n * k // K for k in range(K + 1)]
        src = torch.from_numpy(qc)
        cur = torch.cuda.current_stream(dev)
        s_in, s_out = _copy_streams(dev)
        qd = torch.empty((n, qs), dtype=torch.float64, device=dev)
        comps, norms, grads, inds, _, _ = self._outputs(n, False, packed=True)
        rows = (comps if comps is not None else norms)._base
        oob = torch.empty(n, dtype=torch.int64, device=dev)
        cnts = torch.zeros(K, dtype=torch.int64, device=dev)
        hrows = torch.empty(rows.shape, dtype=rows.dtype, pin_memory=True)
        ev_in = [torch.cuda.Event() for _ in range(K)]
        ev_done = [torch.cuda.Event() for _ in range(K)]
        s_in.wait_stream(cur)                       # the buffers were allocated on the current stream
        with torch.cuda.stream(s_in):
            qd[:bounds[1]].copy_(src[:bounds[1]], non_blocking=True)
            ev_in[0].record(s_in)
        # the plan for this chunk size, chosen before the other chunks' uploads
        # are queued: the autotuner times its candidates with the link idle
        cur.wait_event(ev_in[0])
        plan = self._plan(qd[:bounds[1]], bounds[1], qs)
        self.last_plan = plan
        with torch.cuda.stream(s_in):
            for k in range(1, K):
                a, b = bounds[k], bounds[k + 1]
                qd[a:b].copy_(src[a:b], non_blocking=True)
                ev_in[k].record(s_in)
        sl = lambda t, a, b: None if t is None else t[a:b]  # noqa: E731
        for k in range(K):
            a, b = bounds[k], bounds[k + 1]
            cur.wait_event(ev_in[k])
            res = (sl(comps, a, b), sl(norms, a, b), sl(grads, a, b), inds[a:b], oob[a:b], cnts[k:k + 1])
            self._launch(qd[a:b], b - a, qs, False, True, plan, res=res)
            ev_done[k].record(cur)
            s_out.wait_event(ev_done[k])
            with torch.cuda.stream(s_out):
                hrows[a:b].copy_(rows[a:b], non_blocking=True)
        st = self._fetch_status()                   # synchronises the current stream
        if self._fill_pending and self._settle_status(st):
            # the single-pass fill found a row out of meshgrid order and the
            # general ingest rewrote the grid: evaluate again on it (nothing
            # was written to the caller's array yet)
            s_out.synchronize()
            return self._rquery_host_pipelined(qa, qc, n, qs)
        c = cnts.cpu().numpy()
        if c.any():
            bad = torch.cat([oob[bounds[k]:bounds[k] + int(c[k])] + bounds[k] for k in range(K) if c[k]])
            _nan_rows(qa, bad.cpu())                # in-place on the caller's array
        s_out.synchronize()                         # every stream is idle before the buffers are released
        self._last_inds = inds
        if st & _lib.ARB_ERR_CELL_INDEX:
            raise IndexError("cell index beyond the coefficient table (query on an upper face)")
        R, ci, ni, gi = self._packed_layout()
        dim = self._dim
        out = [None if c_ is None else hrows[:, c_:c_ + w].numpy() for c_, w in ((ci, 3), (ni, 1), (gi, dim))]
        return self._pack(*out)

    def sQuery(self, query):
        """Single point (sQuery1/2/3, ARB:213-342 / 916-1062): np.nan outside
        the volume, otherwise components / (value, gradient) / both."""
        dim = self._dim
        is_t = isinstance(query, torch.Tensor)
        qv = [float(query[a]) for a in range(dim)]
        for a in range(dim):
            if qv[a] < self._lo[a] or qv[a] > self._hi[a]:
                return np.nan
        self._settle()
        row = torch.tensor([qv], dtype=torch.float64).to(self.device)
        comps, norms, grads, inds, _, _ = self._run(row, 1, dim, False, False)
        st = self._fetch_status()
        self._last_ind = inds
        if st & _lib.ARB_ERR_CELL_INDEX:
            raise IndexError("cell index beyond the coefficient table (query on an upper face)")
        k = self._kind
        if is_t:
            c = None if comps is None else comps[0]
            nv = None if norms is None else norms[0, 0]
            gv = None if grads is None else grads[0]
        else:
            c = None if comps is None else comps[0].cpu().numpy()
            nv = None if norms is None else np.float64(norms[0, 0].item())
            gv = None if grads is None else grads[0].cpu().numpy()
        if k == _lib.KIND_VECTOR:
            return c
        if k == _lib.KIND_BOTH:
            return c, nv, gv
        return nv, gv

    def _morton_order(self, x):
        """Permutation sorting positions x (N, 3) along a Z-order curve over
        the interpolation box (10 bits per axis): particles in a warp then
        gather neighbouring grid points.  Non-finite rows sort last."""
        lo = torch.tensor([float(v) for v in self._lo], dtype=torch.float64, device=x.device)
        hi = torch.tensor([float(v) for v in self._hi], dtype=torch.float64, device=x.device)
        u = ((x - lo) / (hi - lo)).clamp(0.0, 1.0)
        u = torch.nan_to_num(u, nan=1.0)
        k = (u * 1023.0).to(torch.int64)
        key = torch.zeros(x.shape[0], dtype=torch.int64, device=x.device)
        for b in range(10):
            for a in range(3):
                key |= ((k[:, a] >> b) & 1) << (3 * b + a)
        key = torch.where(torch.isfinite(x).all(1), key, torch.full_like(key, 1 << 31))
        return torch.argsort(key)

    def trajectories(self, x0, v0, dt, nsteps, coef=-1.0, gravity=(0.0, 0.0, 0.0), record_every=0,
                     spatial_sort=True):
        """Integrate particles through the field on the device (3D, scalar,
        norm or both mode): fourth-order Runge-Kutta on x' = v,
        v' = coef * grad f(x) + gravity, with f the interpolated scalar or |B|
        (coef = -mu/m for a weak-field seeker in a magnetic trap).

        x0, v0: (N, 3) NumPy arrays or CUDA tensors.  Returns (x, v) after
        nsteps steps of dt, and with record_every > 0 also the path
        (nsteps // record_every, N, 6) of (x, v) states; arrays of the input
        kind.  Particles that leave the interpolation volume come back NaN;
        `self.lost` counts them.  spatial_sort: integrate in Z-order (the
        results are returned in the caller's order either way)."""
        if self._dim != 3:
            raise NotImplementedError("trajectories are built for 3D fields")
        if self._kind == _lib.KIND_VECTOR:
            raise ValueError("trajectories need a gradient: scalar, norm or both mode")
        on_dev = isinstance(x0, torch.Tensor) and x0.is_cuda
        dev = self.device
        x = torch.as_tensor(x0, dtype=torch.float64).to(dev).reshape(-1, 3)
        v = torch.as_tensor(v0, dtype=torch.float64).to(dev).reshape(-1, 3)
        if x.shape != v.shape:
            raise ValueError("x0 and v0 must have the same shape")
        n = x.shape[0]
        perm = self._morton_order(x) if spatial_sort and n > 1 else None
        state = torch.cat([x, v], 1)
        state = (state[perm] if perm is not None else state).contiguous()
        nrec = nsteps // record_every if record_every > 0 else 0
        path = torch.empty((nrec, n, 6), dtype=torch.float64, device=dev) if nrec else None
        lost = torch.zeros(1, dtype=torch.int64, device=dev)
        grav = (ctypes.c_double * 3)(*[float(v_) for v_ in gravity])
        prec = _lib.PREC_FP64 if self.precision == "fp64" else _lib.PREC_MIXED
        check(lib().arb_rk4_trajectories(self._g, prec, state.data_ptr(), n, float(dt), int(nsteps), float(coef),
                                         grav, _ptr(path), int(record_every) if nrec else 0, lost.data_ptr(),
                                         _stream()), "arb_rk4_trajectories")
        self.lost = int(lost.item())
        if perm is not None:  # back to the caller's order
            st = torch.empty_like(state)
            st[perm] = state
            state = st
            if nrec:
                pt = torch.empty_like(path)
                pt[:, perm] = path
                path = pt
        out = [state[:, :3], state[:, 3:]] + ([path] if nrec else [])
        if not on_dev:
            out = [t.cpu().numpy() for t in out]
        return tuple(out)

    def Query(self, query):
        """Shape dispatch (Query1/2/3, ARB:177-211): rows -> rQuery, a single
        point -> sQuery."""
        shape = tuple(query.shape)
        if len(shape) >= 2 and shape[1] > 1:
            try:
                return self.rQuery(query)
            except IndexError:
                # The reference catches rQuery's IndexError and retries sQuery
                # on the 2-D array, whose scalar comparison raises ValueError.
                raise ValueError("The truth value of an array with more than one element is ambiguous. "
                                 "Use a.any() or a.all() (a query row fell on an upper face and its "
                                 "cell index exceeded the coefficient table)") from None
        return self.sQuery(query)

    # ---------------------------------------------------------- attributes
    @property
    def queryInds(self):
        return None if self._last_inds is None else self._last_inds.cpu().numpy()

    @property
    def queryInd(self):
        return None if self._last_ind is None else int(self._last_ind[0].item())

    @property
    def A(self):
        return matrices.A3() if self._dim == 3 else matrices.A4()

    @property
    def alphamask(self):
        m = np.zeros((self.nc + 1, 1))
        if self._solved is not None:
            m[:-1, 0] = self._solved
        m[-1] = 1
        return m

    def _alpha(self, f):
        cols = self.nc + 1 + (1 if self._extra_col else 0)
        out = np.zeros((self._M, cols))
        if self._table is not None:
            t = self._table.view(self.nc, self._F, self._M)[:, f, :]
            out[:, :self.nc] = t.to(torch.float64).T.cpu().numpy()
        if self._extra_col:
            out[:, -1] = np.nan
        elif self._sentinel_nan:
            out[:, self.nc] = np.nan
        return out

    def _field_index(self, name):
        k = self._kind
        if k == _lib.KIND_VECTOR:
            return {"alphax": 0, "alphay": 1, "alphaz": 2}.get(name)
        if k == _lib.KIND_BOTH:
            return {"alphax": 0, "alphay": 1, "alphaz": 2, "alphan": 3}.get(name)
        return {"alphan": 0}.get(name)

    def __getattr__(self, name):
        # lazily materialised reference attributes (device -> host on demand)
        if name in ("alphax", "alphay", "alphaz", "alphan"):
            f = self._field_index(name)
            if f is None:
                raise AttributeError(name)
            return self._alpha(f)
        if name in ("Bx", "By", "Bz", "Bn"):
            return self._values(name)
        if name == "inputfield":
            return self._inputfield()
        if name == "basePointInds":
            return self._base_point_inds()
        raise AttributeError(name)

    def _grid_vals(self):
        return self._grid64.view(self._npts, self._F)

    def _values(self, name):
        k = self._kind
        g = self._grid_vals()
        comp = {"Bx": 0, "By": 1, "Bz": 2}
        if name == "Bn":
            if k in (_lib.KIND_SCALAR, _lib.KIND_NORM):
                return g[:, 0].cpu().numpy()
            if k == _lib.KIND_BOTH:
                return g[:, 3].cpu().numpy()
            raise AttributeError(name)
        if k in (_lib.KIND_VECTOR, _lib.KIND_BOTH):
            return g[:, comp[name]].cpu().numpy()
        raise AttributeError(name)

    def _inputfield(self):
        dim = self._dim
        grids = torch.meshgrid(*reversed(self._axes_dev), indexing="ij")
        coords = [grids[dim - 1 - a].reshape(-1) for a in range(dim)]
        k = self._kind
        g = self._grid_vals()
        if k == _lib.KIND_SCALAR:
            vals = [g[:, 0]]
        elif k == _lib.KIND_NORM:
            r = self._raw.view(self._npts, 3)
            vals = [r[:, 0], r[:, 1], r[:, 2]]
        else:
            vals = [g[:, 0], g[:, 1], g[:, 2]]
        out = torch.stack(coords + vals, dim=1).cpu().numpy()
        return out.astype(self._field_dtype)

    def _base_point_inds(self):
        n = self._n
        idx = [np.arange(1, v - 2) for v in n]
        strides = np.cumprod([1] + n[:-1])
        tot = np.zeros(1, dtype=np.int64)
        for a in reversed(range(self._dim)):
            tot = (tot[:, None] + idx[a][None, :] * strides[a]).reshape(-1)
        return np.sort(tot)


class tricubic(_Interpolant):
    """Tricubic interpolant of a 3D scalar (N x 4) or vector (N x 6) field."""
    __version__ = "1.8"
    _dim = 3

    def _set_counts(self, n):
        self.nPos = np.array([n[0] - 3, n[1] - 3, n[2] - 3])

    def neighbourInd(self, ind0):
        """64 flat grid indices of the 4x4x4 block around base index ind0 (ARB:605-621)."""
        nx, ny = self._n[0], self._n[1]
        o = np.arange(4) - 1
        return (int(ind0) + (o[None, None, :] + nx * o[None, :, None] + nx * ny * o[:, None, None])).ravel()


class quadcubic(_Interpolant):
    """Quadcubic interpolant of a 4D scalar (N x 5) or vector (N x 7) field."""
    __version__ = "1.8"
    _dim = 4

    def _set_counts(self, n):
        self.nPosx, self.nPosy, self.nPosz, self.nPost = n

    def neighbourInd(self, ind0):
        """256 flat grid indices of the 4^4 block around base index ind0 (ARB:1357-1381)."""
        nx, ny, nz = self._n[0], self._n[1], self._n[2]
        o = np.arange(4) - 1
        off = (o[None, None, None, :] + nx * o[None, None, :, None] + nx * ny * o[None, :, None, None]
               + nx * ny * nz * o[:, None, None, None])
        return (int(ind0) + off).ravel()
