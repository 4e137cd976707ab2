"""Per-workload choice of query strategy and tile shape, measured on first use.

For a large query batch the interpolant can evaluate
  * on the fly from the grid, in query order ("plain") or grouped by spatial
    bins of 2^s cells per edge ("binned", s = the tile shape), or
  * from the coefficient table (built by `allCoeffs`), binned.
Which is fastest depends on the field size, the query count and density,
and whether a table already exists: the table costs one solve (HBM-bound
write of 1 KB per cell in 'both' mode) and then a cheaper evaluation; the
binned paths trade a counting sort for cache-friendly gathers.

The tuner times each candidate with CUDA events on the caller's own query
rows (evaluating a scratch copy, so the caller's array is untouched),
caches the winner in memory and in a JSON file keyed by GPU, dimension,
field count, precision and the log2 buckets of cell and query counts, and
reuses it for every later batch of that shape.  Set ARBINTERP_TUNE_DIR to
move the cache file, or ARBINTERP_TUNE=off to use the built-in defaults.
"""
from __future__ import annotations

import json
import math
import os
import threading

import torch

from . import _lib

_MEM: dict = {}
_LOCK = threading.Lock()
TABLE_TUNE_BYTES = 4 << 30      # only try the table strategy when it is this small or already built


def _cache_path():
    d = os.environ.get("ARBINTERP_TUNE_DIR") or os.path.join(os.path.expanduser("~"), ".cache",
                                                             "arbinterp_gb300")
    return os.path.join(d, "autotune.json")


def _load():
    p = _cache_path()
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key, plan):
    p = _cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        data = _load()
        data[key] = plan
        tmp = p + f".{os.getpid()}.tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def default_plan(interp, nq):
    return {"table": interp._table_complete, "binned": nq >= interp.sort_threshold, "bin_shift": 0}


_NAMES: dict = {}


def plan_key(interp, nq):
    dev = _NAMES.get(interp.device)
    if dev is None:
        dev = _NAMES[interp.device] = torch.cuda.get_device_name(interp.device)
    b = lambda v: int(math.log2(max(v, 1)))  # noqa: E731
    return (f"{dev}|d{interp._dim}|F{interp._F}|{interp.precision}|cells2^{b(interp.nc)}|"
            f"q2^{b(nq)}|table{int(interp._table_complete)}")


def choose(interp, qd, nq, qs):
    """Plan for evaluating nq rows qd (device, float64, stride qs)."""
    if os.environ.get("ARBINTERP_TUNE", "").lower() in ("off", "0", "no") or nq < (1 << 16):
        return default_plan(interp, nq)
    key = plan_key(interp, nq)
    with _LOCK:
        if key in _MEM:
            return _MEM[key]
        disk = _load()
        if key in disk:
            _MEM[key] = disk[key]
            return disk[key]
    plan = _measure(interp, qd, nq, qs)
    with _LOCK:
        _MEM[key] = plan
    _store(key, plan)
    return plan


def _candidates(interp):
    shifts = (2, 3, 4) if interp._dim == 3 else (1, 2, 3)
    cands = [{"table": False, "binned": True, "bin_shift": s} for s in shifts]
    cands.append({"table": False, "binned": False, "bin_shift": 0})
    table_bytes = interp.nc * interp._F * interp._M * (8 if interp.precision == "fp64" else 4)
    if interp._table_complete or table_bytes <= TABLE_TUNE_BYTES:
        cands.append({"table": True, "binned": True, "bin_shift": 0})
    return cands


def _measure(interp, qd, nq, qs):
    """Time each candidate (one warm-up, two timed runs) and return the fastest.
    A table candidate is charged its build when the table does not exist."""
    interp._settle()       # the grid is written and checked before candidates are timed on it
    best, best_t = None, float("inf")
    had_table = interp._table_complete
    build_t = 0.0
    for plan in _candidates(interp):
        if plan["table"] and not interp._table_complete:
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            interp.allCoeffs()
            e.record()
            torch.cuda.synchronize()
            build_t = s.elapsed_time(e)
        q = qd.clone()
        interp._launch(q, nq, qs, False, False, plan)           # warm-up
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(2):
            interp._launch(q, nq, qs, False, False, plan)
        e.record()
        torch.cuda.synchronize()
        t = s.elapsed_time(e) / 2 + (build_t if (plan["table"] and not had_table) else 0.0)
        plan = dict(plan, ms=round(t, 4))
        if t < best_t:
            best, best_t = plan, t
    if not best["table"] and not had_table and interp._table is not None:
        interp._drop_table()                                    # tuning built it; not chosen
    lib = _lib.lib()
    from .interp import _stream
    lib.arb_status_fetch(interp._status.data_ptr(), _stream())
    return best
