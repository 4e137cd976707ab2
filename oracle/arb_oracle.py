"""CPU oracle for the ARBInterp interpolation path — TEST INFRASTRUCTURE ONLY.

This module is a float64 NumPy restatement of the reference algorithm in
``src/ARBInterp/ARBInterp.py`` (DurhamDecLab/ARBInterp v1.8).  It exists to
check the CUDA product path and to time a CPU baseline; nothing in the
``arbinterp_gb300`` package imports it.  Only ``tests/``, the graft entry's
``smoke()`` and ``bench.py`` (its CPU-baseline and reference arms) may use it.

Parity is pinned: ``tests/test_oracle_golden.py`` checks every function here
against golden vectors produced by the unmodified reference
(``tests/golden/make_golden.py``) and against the reference's own B-matrix
fixtures ``examples/B_Matrix_3D.csv`` / ``examples/B_Matrix_4D.csv``.

The algorithm is restated, not copied:
  * the B and D matrices are built from their definitions (derivative kind x
    corner rows, monomial / stencil-offset columns), and ``A = inv(B) @ D``;
  * the 4D D matrix keeps the reference's row-240 off-by-one (ARB:860);
  * the lazy per-cell solve ``alpha = A @ f[block]`` is vectorised over all
    cells a query batch touches (ARB:570-603, 1322-1355);
  * evaluation is the monomial sum with the reference's gradient scaling
    (divide by h inside the sum, ARB:452, 519, 1186).
"""
from __future__ import annotations

import numpy as np

__all__ = [
    "build_B3", "build_D3", "build_A3", "build_B4", "build_D4", "build_A4",
    "field_params3", "field_params4", "OracleTricubic", "OracleQuadcubic",
    "catmull_rom_A1",
]

# ----------------------------------------------------------------------------
# Matrices (ARB:107-175 for 3D, ARB:726-878 for 4D)
# ----------------------------------------------------------------------------
# Derivative kinds, in the row-block order the reference uses.
_KINDS3 = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1),
           (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)]          # ARB:121-128
_KINDS4 = [(0, 0, 0, 0),
           (1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0), (0, 0, 0, 1),
           (1, 1, 0, 0), (1, 0, 1, 0), (1, 0, 0, 1), (0, 1, 1, 0), (0, 1, 0, 1), (0, 0, 1, 1),
           (1, 1, 1, 0), (1, 1, 0, 1), (1, 0, 1, 1), (0, 1, 1, 1),
           (1, 1, 1, 1)]                                         # ARB:742-759


def _mono_deriv(e: int, c: float, a: int) -> float:
    """d^a/dt^a of t**e at t=c (a in {0,1}); 0**0 == 1 as in NumPy."""
    if a == 0:
        return c ** e
    return e * c ** abs(e - 1)


def _build_B(dim: int) -> np.ndarray:
    kinds = _KINDS3 if dim == 3 else _KINDS4
    nc = 1 << dim                      # corners, x fastest (ARB:110, 729)
    n = 4 ** dim                       # monomials, ex fastest (ARB:111, 730)
    B = np.zeros((n, n))
    for r, kind in enumerate(kinds):
        for k in range(nc):
            corner = [(k >> a) & 1 for a in range(dim)]
            for i in range(n):
                ex = [(i >> (2 * a)) & 3 for a in range(dim)]
                v = 1.0
                for a in range(dim):
                    v *= _mono_deriv(ex[a], float(corner[a]), kind[a])
                B[r * nc + k, i] = v
    return B


def build_B3() -> np.ndarray:
    """64x64 tricubic B (ARB:108-127)."""
    return _build_B(3)


def build_B4() -> np.ndarray:
    """256x256 quadcubic B (ARB:727-759)."""
    return _build_B(4)


def _build_D(dim: int, bug_row240: bool) -> np.ndarray:
    """Finite-difference matrix: row (kind r, corner k) holds the central
    difference stencil of derivative kind r centred on corner k of the 4^dim
    block, in unit-cell units (ARB:131-173, ARB:762-876)."""
    kinds = _KINDS3 if dim == 3 else _KINDS4
    ncrn = 1 << dim
    n = 4 ** dim
    strides = [4 ** a for a in range(dim)]
    D = np.zeros((n, n))

    def stencil(kind, k):
        row = np.zeros(n)
        centre = sum((1 + ((k >> a) & 1)) * strides[a] for a in range(dim))
        terms = [(centre, 1.0)]
        for a in range(dim):
            if kind[a]:
                terms = [(o + s * strides[a], w * 0.5 * s) for (o, w) in terms for s in (1, -1)]
        for o, w in terms:
            row[o] += w
        return row

    for r, kind in enumerate(kinds):
        for k in range(ncrn):
            D[r * ncrn + k] = stencil(kind, k)
    if dim == 4 and bug_row240:
        # ARB:860 enumerates range(241,256): row 240 stays zero and row 240+k
        # carries the d4f stencil of corner k-1.
        last = 15 * ncrn
        shifted = np.zeros((ncrn, n))
        for k in range(1, ncrn):
            shifted[k] = stencil(kinds[15], k - 1)
        D[last:last + ncrn] = shifted
    return D


def build_D3() -> np.ndarray:
    return _build_D(3, False)


def build_D4(bug_row240: bool = True) -> np.ndarray:
    return _build_D(4, bug_row240)


def build_A3() -> np.ndarray:
    """A = inv(B) @ D (ARB:175)."""
    return np.linalg.inv(build_B3()) @ build_D3()


def build_A4() -> np.ndarray:
    """A = inv(B) @ D with the reference's D (ARB:878)."""
    return np.linalg.inv(build_B4()) @ build_D4(True)


def catmull_rom_A1() -> np.ndarray:
    """The 1D factor: A3 == kron(A1, A1, A1) exactly (checked in tests)."""
    return np.array([[0.0, 1.0, 0.0, 0.0],
                     [-0.5, 0.0, 0.5, 0.0],
                     [1.0, -2.5, 2.0, -0.5],
                     [-0.5, 1.5, -1.5, 0.5]])


# ----------------------------------------------------------------------------
# Field ingest (ARB:528-568 for 3D, ARB:1264-1320 for 4D)
# ----------------------------------------------------------------------------
def _sort_rows(field: np.ndarray, ncoord: int) -> np.ndarray:
    # Lexicographic order with the last coordinate slowest (ARB:530-532,
    # 1266-1269).  lexsort's last key is the primary key.
    keys = tuple(field[:, a] for a in range(ncoord))
    return field[np.lexsort(keys)]


def field_params3(field: np.ndarray) -> dict:
    f = _sort_rows(np.asarray(field), 3)
    # axes found with exact float equality against the first sorted row (ARB:535-539)
    on_y0 = f[f[:, 1] == f[0, 1]]
    xaxis = on_y0[on_y0[:, 2] == on_y0[0, 2]]
    on_x0 = f[f[:, 0] == f[0, 0]]
    yaxis = on_x0[on_x0[:, 2] == on_x0[0, 2]]
    zaxis = on_x0[on_x0[:, 1] == on_x0[0, 1]]
    nx, ny, nz = len(xaxis), len(yaxis), len(zaxis)
    p = dict(inputfield=f, nx=nx, ny=ny, nz=nz,
             nPos=np.array([nx - 3, ny - 3, nz - 3]),
             hx=np.abs(xaxis[0, 0] - xaxis[1, 0]),                 # ARB:547-549
             hy=np.abs(yaxis[0, 1] - yaxis[1, 1]),
             hz=np.abs(zaxis[0, 2] - zaxis[1, 2]),
             xIntMin=f[1, 0], yIntMin=f[nx, 1], zIntMin=f[nx * ny, 2],   # ARB:551-556
             xIntMax=f[-2, 0], yIntMax=f[-2 * nx, 1], zIntMax=f[-2 * nx * ny, 2])
    # corner (1,1,1) of every cell, z-major x-fastest (ARB:559-565)
    cx, cy, cz = np.arange(nx - 3), np.arange(ny - 3), np.arange(nz - 3)
    base = (1 + cx)[None, None, :] + nx * (1 + cy)[None, :, None] + nx * ny * (1 + cz)[:, None, None]
    p["basePointInds"] = np.sort(base.ravel())
    p["nc"] = p["basePointInds"].size
    return p


def field_params4(field: np.ndarray) -> dict:
    f = _sort_rows(np.asarray(field), 4)
    x0, y0, z0, t0 = f[0, 0], f[0, 1], f[0, 2], f[0, 3]

    def axis(free):
        m = np.ones(len(f), bool)
        for a, v in enumerate((x0, y0, z0, t0)):
            if a != free:
                m &= f[:, a] == v
        return f[m]
    xa, ya, za, ta = axis(0), axis(1), axis(2), axis(3)             # ARB:1272-1290
    nx, ny, nz, nt = len(xa), len(ya), len(za), len(ta)
    p = dict(inputfield=f, nPosx=nx, nPosy=ny, nPosz=nz, nPost=nt,
             hx=np.abs(xa[0, 0] - xa[1, 0]), hy=np.abs(ya[0, 1] - ya[1, 1]),
             hz=np.abs(za[0, 2] - za[1, 2]), ht=np.abs(ta[0, 3] - ta[1, 3]),   # ARB:1292-1295
             xIntMin=f[1, 0], yIntMin=f[nx, 1], zIntMin=f[nx * ny, 2], tIntMin=f[nx * ny * nz, 3],
             xIntMax=f[-2, 0], yIntMax=f[-2 * nx, 1], zIntMax=f[-2 * nx * ny, 2],
             tIntMax=f[-2 * nx * ny * nz, 3])                          # ARB:1297-1305
    cx, cy, cz, ct = (np.arange(n - 3) for n in (nx, ny, nz, nt))
    base = ((1 + cx)[None, None, None, :] + nx * (1 + cy)[None, None, :, None]
            + nx * ny * (1 + cz)[None, :, None, None] + nx * ny * nz * (1 + ct)[:, None, None, None])
    p["basePointInds"] = np.sort(base.ravel())                        # ARB:1308-1317
    p["nc"] = p["basePointInds"].size
    return p


# ----------------------------------------------------------------------------
# Interpolators
# ----------------------------------------------------------------------------
def _powers(t: np.ndarray) -> np.ndarray:
    return np.stack([np.ones_like(t), t, t * t, t * t * t], axis=-1)


def _dpowers(t: np.ndarray) -> np.ndarray:
    return np.stack([np.zeros_like(t), np.ones_like(t), 2 * t, 3 * t * t], axis=-1)


class _OracleBase:
    dim = 3

    def _setup_mode(self, field, mode, ncoord):
        ncol = field.shape[1]
        vals = self.inputfield[:, ncoord:]
        self.sentinel = np.nan
        self.extra_col = False
        if ncol == ncoord + 1:                       # scalar (ARB:24-32, 641-649)
            self.kind = "scalar"
            self.fields = {"n": vals[:, 0]}
            self.sentinel = 0.0
        elif ncol == ncoord + 3:
            comps = {"x": vals[:, 0], "y": vals[:, 1], "z": vals[:, 2]}
            # ||(Bx,By,Bz)|| at every grid point (ARB:58, 74)
            bn = np.sqrt(vals[:, 0] * vals[:, 0] + vals[:, 1] * vals[:, 1] + vals[:, 2] * vals[:, 2])
            if mode == "norm":
                self.kind = "norm"
                self.fields = {"n": bn}
            elif mode == "both":
                self.kind = "both"
                self.fields = dict(comps, n=bn)
            else:
                self.kind = "vector"
                self.fields = comps
                if mode == "vector":                 # nc+2 columns, NaN in the last (ARB:42-45)
                    self.sentinel = 0.0
                    self.extra_col = True
        else:
            raise SystemExit("--- Input not shaped as expected ---")
        self.alpha = {k: np.zeros((self.nc, self.M)) for k in self.fields}
        self.solved = np.zeros(self.nc, bool)

    def alpha_matrix(self, key: str) -> np.ndarray:
        """The reference's coefficient-major (M, nc+1[+1]) array."""
        cols = self.nc + 1 + (1 if self.extra_col else 0)
        out = np.zeros((self.M, cols))
        out[:, :self.nc] = self.alpha[key].T
        if self.extra_col:
            out[:, -1] = np.nan
        else:
            out[:, self.nc] = self.sentinel
        return out

    def _solve(self, cells: np.ndarray):
        cells = np.unique(cells[(cells >= 0) & (cells < self.nc)])
        cells = cells[~self.solved[cells]]
        if cells.size == 0:
            return
        blocks = self.basePointInds[cells][:, None] + self.block_offsets[None, :]
        for k, vals in self.fields.items():
            self.alpha[k][cells] = vals[blocks] @ self.A.T         # alpha = A @ f[inds]
        self.solved[cells] = True

    def all_coeffs(self):
        self._solve(np.arange(self.nc))

    def _row(self, key, idx):
        """alpha rows for flat indices, honouring the sentinel columns."""
        nc = self.nc
        out = np.empty((idx.size, self.M))
        ok = idx < nc
        out[ok] = self.alpha[key][idx[ok]]
        out[idx == nc] = self.sentinel
        return out

    def query(self, q: np.ndarray):
        """Range query with the reference's semantics (rQuery*, ARB:344-521 /
        1064-1258).  Mutates ``q`` in place (OOB rows -> NaN) and returns a
        dict with 'comps', 'norms', 'grads', 'inds' as the mode provides."""
        d = self.dim
        lo, hi, h = self.lo, self.hi, self.h
        bad = np.zeros(len(q), bool)
        for a in range(d):
            bad |= (q[:, a] < lo[a]) | (q[:, a] > hi[a])
        q[bad] = np.nan
        iu = [(q[:, a] - lo[a]) / h[a] for a in range(d)]
        fl = [np.floor(u) for u in iu]
        ind = fl[0].copy()
        mul = 1
        for a in range(1, d):
            mul = mul * self.ncell[a - 1]
            ind = ind + fl[a] * mul
        ind[np.isnan(ind)] = self.nc
        ind = ind.astype(np.int64)
        if np.any(ind > self.nc):
            # alphamask has nc+1 entries; the reference's mask lookup raises
            raise IndexError("cell index beyond the coefficient table")
        frac = [u - f for u, f in zip(iu, fl)]
        self._solve(ind)
        P = [_powers(t) for t in frac]
        dP = [_dpowers(t) for t in frac]
        mono = self._outer(P)
        out = {"inds": ind}
        vals = {k: (self._row(k, ind) * mono).sum(axis=1) for k in self.fields}
        if "x" in self.fields:
            out["comps"] = np.stack([vals["x"], vals["y"], vals["z"]], axis=1)
        if "n" in self.fields:
            out["norms"] = vals["n"][:, None]
            rows = self._row("n", ind)
            g = []
            for a in range(d):
                Pa = list(P)
                Pa[a] = dP[a]
                g.append(((rows * self._outer(Pa)) / h[a]).sum(axis=1))
            out["grads"] = np.stack(g, axis=1)
        return out

    def adjoint(self, q, dval, dgrad=None):
        """Float64 reference gradient of a loss w.r.t. the grid samples of the
        interpolated scalar field (grid order), given dL/dvalue (n,) and
        optionally dL/dgrad (n, dim).  The reference has no backward pass;
        this is the transpose of its forward map: value = p(x) . (A f_block)
        and grad_a = (dp_a(x) . (A f_block)) / h_a (ARB:399-454), so
        dL/df_block = (dval p + sum_a dgrad_a dp_a / h_a) A."""
        d = self.dim
        q = np.asarray(q, dtype=np.float64)
        bad = np.zeros(len(q), bool)
        for a in range(d):
            bad |= (q[:, a] < self.lo[a]) | (q[:, a] > self.hi[a]) | np.isnan(q[:, a])
        iu = [(q[:, a] - self.lo[a]) / self.h[a] for a in range(d)]
        fl = [np.floor(u) for u in iu]
        ind = fl[0].copy()
        mul = 1
        for a in range(1, d):
            mul = mul * self.ncell[a - 1]
            ind = ind + fl[a] * mul
        ok = ~bad
        ind = np.where(ok, ind, 0).astype(np.int64)
        ok &= ind < self.nc
        frac = [u - f for u, f in zip(iu, fl)]
        P = [_powers(np.where(ok, t, 0.0)) for t in frac]
        dP = [_dpowers(np.where(ok, t, 0.0)) for t in frac]
        coef = dval[:, None] * self._outer(P)
        if dgrad is not None:
            for a in range(d):
                Pa = list(P)
                Pa[a] = dP[a]
                coef = coef + (dgrad[:, a] / self.h[a])[:, None] * self._outer(Pa)
        w = coef @ self.A                          # (n, M) weights on the block samples
        w[~ok] = 0.0
        gg = np.zeros(len(self.inputfield))
        blocks = self.basePointInds[ind][:, None] + self.block_offsets[None, :]
        np.add.at(gg, blocks[ok], w[ok])
        return gg

    def _outer(self, P):
        # monomial index ex + 4 ey + 16 ez (+ 64 et), x fastest
        m = P[0]
        for a in range(1, self.dim):
            m = (P[a][:, :, None] * m[:, None, :]).reshape(len(m), -1)
        return m


class OracleTricubic(_OracleBase):
    """Restatement of ``tricubic`` (ARB:8-621)."""
    dim = 3
    M = 64

    def __init__(self, field, mode=None):
        field = np.asarray(field)
        p = field_params3(field)
        self.__dict__.update(p)
        self.A = build_A3()
        self.lo = (self.xIntMin, self.yIntMin, self.zIntMin)
        self.hi = (self.xIntMax, self.yIntMax, self.zIntMax)
        self.h = (self.hx, self.hy, self.hz)
        self.ncell = (self.nx - 3, self.ny - 3, self.nz - 3)
        nx, ny = self.nx, self.ny
        # 4x4x4 block offsets relative to corner (1,1,1) (ARB:605-621)
        o = np.arange(4) - 1
        self.block_offsets = (o[None, None, :] + nx * o[None, :, None] + nx * ny * o[:, None, None]).ravel()
        self._setup_mode(field, mode, 3)


class OracleQuadcubic(_OracleBase):
    """Restatement of ``quadcubic`` (ARB:627-1381)."""
    dim = 4
    M = 256

    def __init__(self, field, mode=None):
        field = np.asarray(field)
        p = field_params4(field)
        self.__dict__.update(p)
        self.A = build_A4()
        self.lo = (self.xIntMin, self.yIntMin, self.zIntMin, self.tIntMin)
        self.hi = (self.xIntMax, self.yIntMax, self.zIntMax, self.tIntMax)
        self.h = (self.hx, self.hy, self.hz, self.ht)
        nx, ny, nz = self.nPosx, self.nPosy, self.nPosz
        self.ncell = (nx - 3, ny - 3, nz - 3, self.nPost - 3)
        o = np.arange(4) - 1
        self.block_offsets = (o[None, None, None, :] + nx * o[None, None, :, None]
                              + nx * ny * o[None, :, None, None]
                              + nx * ny * nz * o[:, None, None, None]).ravel()   # ARB:1357-1381
        self._setup_mode(field, mode, 4)
