"""Seeded synthetic fields and query sets for the benchmark workloads.

The reference ships no data (its example fields are not distributed), so these
generators stand in for it.  Fields are returned as N x (ncoord + nval) row
arrays, the input format of ``tricubic`` / ``quadcubic``.  Rows come out in
``meshgrid(indexing='ij')`` order (x slowest), which is NOT the interpolator's
internal z-major order, so every construction exercises the ingest sort.

Everything is computed with torch in float64 on the device given (CPU for
small test grids, CUDA for the 256^3 workloads).
"""
from __future__ import annotations

import math

import numpy as np
import torch

__all__ = ["gaussian_field3", "dipole_field3", "moving_gaussian_field4",
           "uniform_queries", "batched_fields"]


def _axes(n, h, origin, device, dtype=torch.float64):
    return [origin[a] + h[a] * torch.arange(n[a], dtype=dtype, device=device) for a in range(len(n))]


def _rows(axes, values):
    grids = torch.meshgrid(*axes, indexing="ij")
    coords = [g.reshape(-1) for g in grids]
    vals = [v.reshape(-1) for v in values]
    return torch.stack(coords + vals, dim=1)


def gaussian_field3(n=(41, 41, 41), h=(0.1, 0.12, 0.08), seed=0, device="cpu",
                    n_gauss=8, origin=None, dtype=torch.float64):
    """Scalar 3D field: sum of isotropic Gaussians (the 41^3 scalar workload).

    Origin uniform in [-5, 5]^3, centres uniform in the box, widths in
    [0.3, 1.5], amplitudes N(0, 1).  Returns an N x 4 tensor (x, y, z, U)."""
    rng = np.random.default_rng(seed)
    if origin is None:
        origin = rng.uniform(-5, 5, 3)
    ext = [h[a] * (n[a] - 1) for a in range(3)]
    cen = origin + rng.uniform(0, 1, (n_gauss, 3)) * np.array(ext)
    wid = rng.uniform(0.3, 1.5, n_gauss)
    amp = rng.standard_normal(n_gauss)
    ax = _axes(n, h, origin, device)
    X, Y, Z = torch.meshgrid(*ax, indexing="ij")
    U = torch.zeros_like(X)
    for c, w, a in zip(cen, wid, amp):
        r2 = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2
        U += a * torch.exp(-r2 / (2 * w * w))
    out = _rows(ax, [U])
    return out.to(dtype)


def dipole_field3(n=(256, 256, 256), seed=1, device="cpu", n_dip=16, half=1.0):
    """Vector 3D field: superposition of point dipoles outside the box.

    Box [-half, half]^3; dipole positions uniform in [-3h, 3h]^3 but outside
    [-1.25h, 1.25h]^3; moments with random direction and magnitude
    log-uniform in [1, 100].  B = (3 (m.r) r / |r|^5 - m / |r|^3).
    Returns an N x 6 tensor (x, y, z, Bx, By, Bz)."""
    rng = np.random.default_rng(seed)
    pos = []
    while len(pos) < n_dip:
        p = rng.uniform(-3 * half, 3 * half, 3)
        if np.max(np.abs(p)) > 1.25 * half:
            pos.append(p)
    pos = np.array(pos)
    dirs = rng.standard_normal((n_dip, 3))
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    mag = np.exp(rng.uniform(math.log(1.0), math.log(100.0), n_dip))
    mom = dirs * mag[:, None]
    h = [2 * half / (n[a] - 1) for a in range(3)]
    ax = _axes(n, h, [-half] * 3, device)
    X, Y, Z = torch.meshgrid(*ax, indexing="ij")
    Bx = torch.zeros_like(X)
    By = torch.zeros_like(X)
    Bz = torch.zeros_like(X)
    for p, m in zip(pos, mom):
        rx, ry, rz = X - p[0], Y - p[1], Z - p[2]
        r2 = rx * rx + ry * ry + rz * rz
        inv_r = torch.rsqrt(r2)
        inv_r3 = inv_r * inv_r * inv_r
        mdr = (m[0] * rx + m[1] * ry + m[2] * rz) * inv_r * inv_r
        Bx += (3 * mdr * rx - m[0]) * inv_r3
        By += (3 * mdr * ry - m[1]) * inv_r3
        Bz += (3 * mdr * rz - m[2]) * inv_r3
    return _rows(ax, [Bx, By, Bz])


def moving_gaussian_field4(n=(64, 64, 64, 32), h=(0.1, 0.1, 0.1, 0.1), seed=2, device="cpu",
                           n_gauss=6):
    """Scalar 4D field (x, y, z, t): Gaussians on linear trajectories with
    amplitude a cos(w t); widths in [0.2, 1.0], w in [0.5, 3].
    Returns an N x 5 tensor (x, y, z, t, U)."""
    rng = np.random.default_rng(seed)
    ext = np.array([h[a] * (n[a] - 1) for a in range(3)])
    c0 = rng.uniform(0, 1, (n_gauss, 3)) * ext
    vel = rng.uniform(-1, 1, (n_gauss, 3)) * ext / max(h[3] * (n[3] - 1), 1e-9) * 0.5
    wid = rng.uniform(0.2, 1.0, n_gauss)
    amp = rng.standard_normal(n_gauss)
    omg = rng.uniform(0.5, 3.0, n_gauss)
    ax = _axes(n, h, [0.0] * 4, device)
    X, Y, Z, T = torch.meshgrid(*ax, indexing="ij")
    U = torch.zeros_like(X)
    for a in range(n_gauss):
        cx = c0[a, 0] + vel[a, 0] * T
        cy = c0[a, 1] + vel[a, 1] * T
        cz = c0[a, 2] + vel[a, 2] * T
        r2 = (X - cx) ** 2 + (Y - cy) ** 2 + (Z - cz) ** 2
        U += amp[a] * torch.cos(omg[a] * T) * torch.exp(-r2 / (2 * wid[a] ** 2))
    return _rows(ax, [U])


def uniform_queries(lo, hi, n_in, n_out, h, seed=3, device="cpu", ncols=None):
    """n_in points uniform in [lo, hi] per axis plus n_out points in a shell
    just outside the interpolatable volume (up to two grid spacings beyond
    one of its faces), which must come back NaN.  Rows shuffled."""
    d = len(lo)
    g = torch.Generator(device="cpu").manual_seed(seed)
    lo_t = torch.tensor(lo, dtype=torch.float64)
    hi_t = torch.tensor(hi, dtype=torch.float64)
    h_t = torch.tensor(h, dtype=torch.float64)
    qin = lo_t + (hi_t - lo_t) * torch.rand(n_in, d, generator=g, dtype=torch.float64)
    qout = lo_t + (hi_t - lo_t) * torch.rand(n_out, d, generator=g, dtype=torch.float64)
    if n_out:
        axis = torch.randint(0, d, (n_out,), generator=g)
        side = torch.randint(0, 2, (n_out,), generator=g)
        depth = (1e-3 + 2.0 * torch.rand(n_out, generator=g, dtype=torch.float64)) * h_t[axis]
        val = torch.where(side == 1, hi_t[axis] + depth, lo_t[axis] - depth)
        qout[torch.arange(n_out), axis] = val
    q = torch.cat([qin, qout], 0)
    q = q[torch.randperm(len(q), generator=g)]
    if ncols is not None and ncols > d:
        q = torch.cat([q, torch.zeros(len(q), ncols - d, dtype=torch.float64)], 1)
    return q.to(device)


def batched_fields(n_fields=512, seed=4, edge_range=(16, 128), q_range=(1e3, 1e6), device="cpu"):
    """Many scalar fields for the batched workload: cube edges log-uniform in
    edge_range, anisotropic spacings in [0.05, 0.2], Gaussian-sum values; query
    counts log-uniform in q_range.  Yields (field_rows, n_queries, seed)."""
    rng = np.random.default_rng(seed)
    for i in range(n_fields):
        e = int(round(math.exp(rng.uniform(math.log(edge_range[0]), math.log(edge_range[1])))))
        h = tuple(rng.uniform(0.05, 0.2, 3))
        nq = int(round(math.exp(rng.uniform(math.log(q_range[0]), math.log(q_range[1])))))
        f = gaussian_field3(n=(e, e, e), h=h, seed=int(rng.integers(1 << 30)), device=device)
        yield f, nq, int(rng.integers(1 << 30))



def field_csv_text(n=(256, 256, 256), nfield=3, seed=5, origin=-1.0, inv_h=128, device="cpu"):
    """A field file in the reference's layout (np.savetxt fmt '%.18e',
    delimiter ','; README.md:64-72) as a 1-D uint8 tensor on ``device``: rows
    x, y, z, then nfield values, x fastest.  Coordinates are the grid
    origin + i / inv_h (exact decimals, formatted by Python); field values are
    random 19-significant-digit decimals with random signs and exponents in
    [-20, 20], so each value has the savetxt width of its sign (24 or 25
    characters)."""
    nx, ny, nz = n
    rows = nx * ny * nz
    ncol = 3 + nfield
    W = 26                                   # sign slot + 24 characters + delimiter
    gen = torch.Generator(device=device).manual_seed(seed)
    u8 = dict(dtype=torch.uint8, device=device)
    arr = torch.empty((rows, ncol * W), **u8)
    keep = torch.ones((rows, ncol * W), dtype=torch.bool, device=device)
    arr[:, W - 1::W] = ord(",")
    arr[:, -1] = ord("\n")
    r = torch.arange(rows, dtype=torch.int64, device=device)
    idx = (r % nx, torch.div(r, nx, rounding_mode="floor") % ny, torch.div(r, nx * ny, rounding_mode="floor"))
    for a, m in enumerate((nx, ny, nz)):
        strs = ["%.18e" % (origin + i / inv_h) for i in range(m)]
        tab = torch.tensor(list("".join(s.rjust(25) for s in strs).encode()), **u8).reshape(m, 25)
        arr[:, a * W:a * W + 25] = tab[idx[a]]
        keep[:, a * W] = tab[idx[a], 0] == ord("-")
    for k in range(3, ncol):
        o = k * W
        arr[:, o] = ord("-")
        keep[:, o] = torch.rand(rows, generator=gen, device=device) < 0.5
        arr[:, o + 1] = torch.randint(ord("1"), ord("9") + 1, (rows,), generator=gen, **u8)
        arr[:, o + 2] = ord(".")
        arr[:, o + 3:o + 21] = torch.randint(ord("0"), ord("9") + 1, (rows, 18), generator=gen, **u8)
        arr[:, o + 21] = ord("e")
        e = torch.randint(-20, 21, (rows,), generator=gen, device=device)
        arr[:, o + 22] = torch.where(e < 0, ord("-"), ord("+")).to(torch.uint8)
        arr[:, o + 23] = (e.abs() // 10 + ord("0")).to(torch.uint8)
        arr[:, o + 24] = (e.abs() % 10 + ord("0")).to(torch.uint8)
    return arr[keep]
