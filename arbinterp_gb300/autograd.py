"""Differentiable tricubic interpolation of a scalar field (torch.autograd).

The reference has no backward pass.  `TricubicField` wraps one scalar
interpolant (fixed grid geometry) so that

    value, grad = field(values, queries)

is differentiable with respect to the grid sample values (1-D tensor in grid
order: z-major, x fastest) and the query coordinates.  Forward runs the
query kernels of ``libarbinterp.so``; backward runs ``arb_adjoint`` (atomic
scatter of dL/dvalue and dL/dgrad through the Catmull-Rom weights, and
dL/dq from the interpolant's gradient and Hessian), or in mixed precision
with at least as many query rows as cells on ``arb_adjoint_binned`` (the
same with the queries grouped by bin and the scatter accumulated per bin in
shared memory).  A row whose upstream dL/dvalue is NaN scatters nothing and gets a
NaN query gradient.

Rows outside the interpolation volume give NaN values (as the reference
does) and no gradient; mask them out of the loss.
"""
from __future__ import annotations

import torch

from . import _lib
from .interp import _stream, tricubic

__all__ = ["TricubicField", "TricubicFunction"]


class TricubicFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, values, queries, field):
        interp = field.interp
        L = _lib.lib()
        v = values.detach().contiguous()
        is32 = int(v.dtype == torch.float32)
        if v.dtype not in (torch.float32, torch.float64):
            v = v.to(torch.float64)
            is32 = 0
        if v.numel() != interp._npts:
            raise ValueError(f"values must hold {interp._npts} grid samples, got {v.numel()}")
        _lib.check(L.arb_grid_set_values(interp._g, v.data_ptr(), is32, interp._grid64.data_ptr(),
                                         None if interp._grid32 is None else interp._grid32.data_ptr(),
                                         _stream()), "arb_grid_set_values")
        if interp._table is not None:
            interp._drop_table()
        q = queries.detach().to(torch.float64).contiguous()
        n = q.shape[0]
        plan = {"table": False, "binned": n >= interp.sort_threshold, "bin_shift": 0}
        _, norms, grads, _, _, _ = interp._launch(q, n, q.shape[1], False, False, plan)
        ctx.field = field
        ctx.values_dtype = values.dtype
        ctx.queries_dtype = queries.dtype
        ctx.save_for_backward(q)
        return norms[:, 0].to(values.dtype), grads.to(values.dtype)

    @staticmethod
    def backward(ctx, dvalue, dgrad):
        (q,) = ctx.saved_tensors
        interp = ctx.field.interp
        L = _lib.lib()
        n = q.shape[0]
        mixed = interp.precision == "mixed"
        gg = torch.zeros(interp._npts, dtype=torch.float32 if mixed else torch.float64, device=q.device)
        want_q = ctx.needs_input_grad[1]
        qg = torch.empty((n, 3), dtype=torch.float64, device=q.device) if want_q else None
        dv = None if dvalue is None else dvalue.detach().to(torch.float64).contiguous()
        dgr = None if dgrad is None else dgrad.detach().to(torch.float64).contiguous()
        prec = _lib.PREC_MIXED if mixed else _lib.PREC_FP64
        args = (None if dv is None else dv.data_ptr(), None if dgr is None else dgr.data_ptr(), gg.data_ptr(),
                None if qg is None else qg.data_ptr())
        binned = ctx.field.binned_adjoint
        if binned is None:
            # grouping pays once a bin holds several hundred queries (the
            # binning passes, each bin's tile and one flush of its 1331
            # points): at least as many queries as cells
            binned = n >= max(interp.sort_threshold, interp.nc)
        if mixed and binned:
            # grouped by bin: dL/df accumulated per bin in shared memory
            need = int(L.arb_adjoint_work_bytes(interp._g, n))
            if interp._ws is None or interp._ws.numel() < need:
                interp._ws = torch.empty(need, dtype=torch.uint8, device=q.device)
            _lib.check(L.arb_adjoint_binned(interp._g, prec, q.data_ptr(), n, q.shape[1], *args,
                                            interp._ws.data_ptr(), need, interp._status.data_ptr(), _stream()),
                       "arb_adjoint_binned")
        else:
            _lib.check(L.arb_adjoint(interp._g, prec, q.data_ptr(), n, q.shape[1], *args,
                                     interp._status.data_ptr(), _stream()), "arb_adjoint")
        gvals = gg.to(ctx.values_dtype) if ctx.needs_input_grad[0] else None
        gq = qg.to(ctx.queries_dtype) if want_q else None
        return gvals, gq, None


class TricubicField:
    """A scalar field on a fixed regular grid, differentiable in its sample
    values and the query points.

    field_rows: N x 4 (x, y, z, U) rows, any order, defining the geometry and
    the initial values (NumPy or torch).  precision: 'fp64' or 'mixed'.
    """

    def __init__(self, field_rows, precision="fp64", device=None, sort_threshold=1 << 15, binned_adjoint=None):
        self.interp = tricubic(field_rows, "quiet", precision=precision, strategy="otf", device=device,
                               sort_threshold=sort_threshold)
        self.binned_adjoint = binned_adjoint   # None: by query density; True / False: forced (mixed only)
        if self.interp._F != 1:
            raise ValueError("TricubicField needs a scalar field (N x 4 rows)")

    @property
    def shape(self):
        """(nz, ny, nx) of the grid-ordered values."""
        n = self.interp._n
        return (n[2], n[1], n[0])

    def initial_values(self):
        """The sample values in grid order (a float64 copy)."""
        return self.interp._grid64.view(-1).clone()

    def __call__(self, values, queries):
        """values: (npts,) grid-ordered samples; queries: (N, >=3) points.
        Returns (value (N,), gradient (N, 3))."""
        return TricubicFunction.apply(values, queries, self)
