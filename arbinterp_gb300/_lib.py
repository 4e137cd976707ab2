"""ctypes binding of ``libarbinterp.so`` (the C ABI in include/arbinterp.h).

The library is the only compute path: if it cannot be loaded the package
raises instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libarbinterp.so")

ARB_OK = 0
ARB_ERR_INVALID = 1
ARB_ERR_CUDA = 2
ARB_ERR_IRREGULAR_GRID = 4
ARB_ERR_CELL_INDEX = 8
ARB_ERR_CAPACITY = 16
ARB_ERR_TIMEOUT = 32
ARB_ERR_UNSUPPORTED = 64

PREC_FP64 = 0
PREC_MIXED = 1

KIND_SCALAR, KIND_VECTOR, KIND_NORM, KIND_BOTH = 0, 1, 2, 3


class ArbGrid(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("kind", C.c_int32), ("nfield", C.c_int32), ("sentinel_nan", C.c_int32),
        ("n", C.c_int64 * 4), ("nc", C.c_int64),
        ("lo", C.c_double * 4), ("hi", C.c_double * 4), ("h", C.c_double * 4),
        ("grid64", C.c_void_p), ("grid32", C.c_void_p), ("table", C.c_void_p),
        ("table_prec", C.c_int32), ("bin_shift", C.c_int32),
    ]


class ArbQueryOut(C.Structure):
    _fields_ = [
        ("comps", C.c_void_p), ("norms", C.c_void_p), ("grads", C.c_void_p),
        ("inds", C.c_void_p), ("oob_rows", C.c_void_p), ("oob_count", C.c_void_p),
        ("comps_stride", C.c_int64), ("norms_stride", C.c_int64), ("grads_stride", C.c_int64),
    ]


_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64

# name -> (restype, argtypes)
SIGNATURES = {
    "arb_ingest_axes_work_bytes": (C.c_size_t, [_I32]),
    "arb_ingest_axes": (C.c_int, [_P, _I32, _I64, _I32, _I32, _I64, _P, _P, _P, C.c_size_t, _P, _P]),
    "arb_ingest_scatter": (C.c_int, [_P, _I32, _I64, _I32, _I32, _P, _I64, C.POINTER(C.c_int64), _I32,
                                     _P, _P, _P, _P, _P, _P]),
    "arb_ingest_ordered": (C.c_int, [_P, _I32, _I64, _I32, _I32, _I32, _I64, _P, _P, _P, _P, _P, _P, C.c_size_t,
                                     _P, _P]),
    "arb_ingest_ordered_probe": (C.c_int, [_P, _I32, _I64, _I32, _I32, _I32, _I64, _P, _P, _P, C.c_size_t,
                                           _P, _P]),
    "arb_ingest_ordered_fill": (C.c_int, [_P, _I32, _I64, _I32, _I32, _I32, _I64, _P, _P, C.c_size_t, _P, _P,
                                          _P, _P, _P]),
    "arb_ingest_summary": (C.c_int, [_P, _I64, _P, _I32, _P, _P, _P]),
    "arb_fd_planes": (C.c_int, [C.POINTER(ArbGrid), _P, _P]),
    "arb_coef_solve": (C.c_int, [C.POINTER(ArbGrid), _I32, _I64, _I64, _P, _P, _P]),
    "arb_query_eval": (C.c_int, [C.POINTER(ArbGrid), _P, _I64, _I64, _I32, C.POINTER(ArbQueryOut), _P, _P]),
    "arb_query_eval_otf": (C.c_int, [C.POINTER(ArbGrid), _I32, _P, _I64, _I64, _I32,
                                     C.POINTER(ArbQueryOut), _P, _P]),
    "arb_query_sorted_work_bytes": (C.c_size_t, [C.POINTER(ArbGrid), _I32, _I64]),
    "arb_query_eval_sorted": (C.c_int, [C.POINTER(ArbGrid), _I32, _I32, _P, _I64, _I64, _I32,
                                        C.POINTER(ArbQueryOut), _P, C.c_size_t, _P, _P]),
    "arb_adjoint": (C.c_int, [C.POINTER(ArbGrid), _I32, _P, _I64, _I64, _P, _P, _P, _P, _P, _P]),
    "arb_adjoint_work_bytes": (C.c_size_t, [C.POINTER(ArbGrid), _I64]),
    "arb_adjoint_binned": (C.c_int, [C.POINTER(ArbGrid), _I32, _P, _I64, _I64, _P, _P, _P, _P, _P, C.c_size_t,
                                     _P, _P]),
    "arb_grid_set_values": (C.c_int, [C.POINTER(ArbGrid), _P, _I32, _P, _P, _P]),
    "arb_batched_launch": (C.c_int, [_P, _I32, _I32, _P, _P, _I64, _I32, _I32, _P, _I64, _I32,
                                     C.POINTER(ArbQueryOut), _P, _P, _P]),
    "arb_query_bin": (C.c_int, [C.POINTER(ArbGrid), _I32, _P, _I64, _I64, _I32, C.POINTER(ArbQueryOut),
                                _P, C.c_size_t, _P, _P]),
    "arb_query_eval_binned": (C.c_int, [C.POINTER(ArbGrid), _I32, _I32, _I64, C.POINTER(ArbQueryOut), _P,
                                        C.c_size_t, _P]),
    "arb_query_eval_sorted_noalloc": (C.c_int, [C.POINTER(ArbGrid), _I32, _I32, _P, _I64, _I64, _I32,
                                                C.POINTER(ArbQueryOut), _P, _P]),
    "arb_rk4_trajectories": (C.c_int, [C.POINTER(ArbGrid), _I32, _P, _I64, C.c_double, _I64, C.c_double,
                                       C.POINTER(C.c_double), _P, _I64, _P, _P]),
    "arb_csv_count_work_bytes": (C.c_size_t, [_I64]),
    "arb_csv_count": (C.c_int, [_P, _I64, _P, C.c_size_t, _P, _P]),
    "arb_csv_lines_work_bytes": (C.c_size_t, [_I64]),
    "arb_csv_split": (C.c_int, [_P, _I64, _I64, _I32, _I32, _I64, _P, _P, C.c_size_t, _P, _P, _P]),
    "arb_csv_parse": (C.c_int, [_P, _I64, _I64, _I32, _I32, _P, C.c_size_t, _P, _P, _I64, _I64, _P, _P]),
    "arb_status_fetch": (C.c_int, [_P, _P]),
    "arb_status_clear": (C.c_int, [_P, _P]),
    "arb_test_set_mma_wait_limit": (C.c_int, [_I64]),
    "arb_version": (C.c_char_p, []),
}

_lib = None


def lib():
    """Load (once) and return the library; raise if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is not built. Build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'` or `python arbinterp_gb300/build.py`.")
    import torch  # noqa: F401  (loads libcudart.so.13 first so the library shares it)
    L = C.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(rc: int, what: str):
    if rc != ARB_OK:
        raise RuntimeError(f"{what} failed with arb_status {rc} ({describe(rc)})")


def describe(rc: int) -> str:
    names = {ARB_ERR_INVALID: "invalid argument", ARB_ERR_CUDA: "CUDA error",
             ARB_ERR_IRREGULAR_GRID: "field rows are not a full regular grid",
             ARB_ERR_CELL_INDEX: "cell index beyond the coefficient table",
             ARB_ERR_CAPACITY: "axis longer than the ingest capacity",
             ARB_ERR_TIMEOUT: "device wait timed out",
             ARB_ERR_UNSUPPORTED: "unsupported combination"}
    return ", ".join(v for k, v in names.items() if rc & k) or "unknown"
