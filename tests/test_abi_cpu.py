"""CPU-only checks: the C-ABI library builds and exports every entry point
declared in include/arbinterp.h; the closed-form matrices and host-side mode
dispatch match the reference.  No CUDA call is made."""
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"\b(arb_[a-z0-9_]+)\s*\(", src))
    return sorted(names)


def test_library_builds_and_exports_declared_symbols():
    from arbinterp_gb300 import build
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (arb_[a-z0-9_]+)", out))
    declared = _declared()
    assert declared, "no entry points found in include/"
    missing = [d for d in declared if d not in exported]
    assert not missing, missing
    # and nothing undeclared leaks out of the ABI
    extra = sorted(exported - set(declared))
    assert not extra, extra


def test_ctypes_signatures_cover_declarations():
    from arbinterp_gb300 import _lib
    assert set(_lib.SIGNATURES) == set(_declared())


def test_closed_form_matrices_equal_reference(golden):
    from arbinterp_gb300 import matrices
    assert np.array_equal(matrices.A3(), golden["A3"])
    assert np.array_equal(matrices.A4(), golden["A4"])


def test_bad_shape_exits_like_reference():
    from arbinterp_gb300 import tricubic, quadcubic
    with pytest.raises(SystemExit, match="N x 4 or N x 6"):
        tricubic(np.zeros((10, 5)), "quiet")
    with pytest.raises(SystemExit, match="N x 5 or N x 7"):
        quadcubic(np.zeros((10, 4)), "quiet")


def test_import_paths():
    import ARBInterp.ARBInterp as A
    from ARBTools.ARBInterp import tricubic as T
    assert A.__version__ == "1.8" and A.tricubic is T
    assert A.tricubic.__version__ == "1.8" and A.quadcubic.__version__ == "1.8"


def test_noalloc_capacity_stated_in_header():
    """The per-call row limits that include/arbinterp.h states for the
    allocation-free entry point on a 256^3 grid are the real ones: the last
    stated row count fits ARB_NOALLOC_SCRATCH_BYTES and one more does not
    (a host-side size computation; no CUDA call)."""
    from arbinterp_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "arbinterp.h")).read()
    cap = eval(re.search(r"#define ARB_NOALLOC_SCRATCH_BYTES \((\d+)u << (\d+)\)", src).expand(r"\1 << \2"))
    m = re.search(r"at most ([\d,]+)[\s*]+query[\s*]+rows per call in float64 and[\s*]+([\d,]+) in mixed", src)
    assert m, "row limits not found in the header"
    stated = [int(m.group(1).replace(",", "")), int(m.group(2).replace(",", ""))]
    L = _lib.lib()
    g = _lib.ArbGrid()
    g.dim, g.kind, g.nfield = 3, _lib.KIND_BOTH, 4
    for a in range(3):
        g.n[a] = 256
    g.n[3] = 1
    g.nc = 253 ** 3
    for prec, rows in zip((_lib.PREC_FP64, _lib.PREC_MIXED), stated):
        assert L.arb_query_sorted_work_bytes(g, prec, rows) <= cap < L.arb_query_sorted_work_bytes(g, prec, rows + 1)


def test_nan_rows_write_back():
    """The in-place NaN rows of a host query array (rQuery's write-back):
    the threaded path for C-contiguous float arrays and the NumPy path for
    other layouts give the same array; a read-only array raises as NumPy's
    assignment does."""
    import numpy as np
    import torch
    from arbinterp_gb300.interp import _nan_rows
    rng = np.random.default_rng(0)
    rows = torch.from_numpy(rng.choice(5000, 300, replace=False).astype(np.int64))
    for dt in (np.float64, np.float32):
        base = rng.standard_normal((5000, 4)).astype(dt)
        want = base.copy()
        want[rows.numpy()] = np.nan
        a = base.copy()
        _nan_rows(a, rows)                          # threaded path
        b = np.asfortranarray(base.copy())
        _nan_rows(b, rows)                          # NumPy path
        for x in (a, b):
            assert np.array_equal(np.isnan(x), np.isnan(want))
            assert np.array_equal(np.nan_to_num(x), np.nan_to_num(want))
    ro = np.zeros((10, 3))
    ro.setflags(write=False)
    with pytest.raises(ValueError):
        _nan_rows(ro, torch.tensor([1, 2]))
