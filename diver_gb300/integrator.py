"""Feature integrator with the reference's interface.

Drop-in for `integrate(voxels, coord_i, coord_o)` of utils/integrator.py:62
and for the implicit stage's `integrate_mlp(voxel_mlp, N, C, coord_i,
coord_o)` (utils/integrator.py:3-59),
as a torch.autograd.Function whose backward is the CUDA scatter kernel
(dv_integrate_bwd).  Gradients flow to `voxels` only: the coordinates come
from the traversal, which the reference does not differentiate either
(utils/ray_voxel_intersection/__init__.py:46-48,82-84).
"""
from __future__ import annotations

import torch
from torch.autograd import Function

from . import _native as N


def _coords(coord_i: torch.Tensor, coord_o: torch.Tensor):
    """Accepts [S,3] tensors, including the two column halves of one [S,6]
    tensor; returns (coord_i, coord_o, row_stride) without copying when the
    rows share a stride."""
    for name, t in (("coord_i", coord_i), ("coord_o", coord_o)):
        if not isinstance(t, torch.Tensor) or not t.is_cuda or t.dtype != torch.float32:
            raise ValueError(f"{name} must be a float32 CUDA tensor")
        if t.dim() != 2 or t.shape[1] != 3:
            raise ValueError(f"{name} must be [S, 3], got {tuple(t.shape)}")
    if coord_i.shape != coord_o.shape:
        raise ValueError("coord_i and coord_o must have the same shape")
    if (coord_i.stride(1) == 1 and coord_o.stride(1) == 1 and coord_i.stride(0) == coord_o.stride(0)
            and coord_i.stride(0) >= 3):
        return coord_i, coord_o, coord_i.stride(0)
    return coord_i.contiguous(), coord_o.contiguous(), 3


def _grid(voxels: torch.Tensor):
    N.need_cuda("voxels", voxels, torch.float32)
    if voxels.dim() != 4 or voxels.shape[-1] % 4 != 0:
        raise ValueError(f"voxels must be [Nz, Ny, Nx, C] with C a multiple of 4, got {tuple(voxels.shape)}")
    nz, ny, nx, c = voxels.shape
    return nx, ny, nz, c


def integrate_forward(voxels, coord_i, coord_o):
    nx, ny, nz, c = _grid(voxels)
    ci, co, stride = _coords(coord_i, coord_o)
    S = ci.shape[0]
    out = torch.empty(S, c, dtype=torch.float32, device=voxels.device)
    N.call("dv_integrate_fwd", N.ptr(voxels), nx, ny, nz, c, N.ptr(ci), N.ptr(co), stride, S, N.ptr(out),
           N.stream(voxels.device))
    return out


def integrate_backward(grad_feature, grid_shape, coord_i, coord_o, out=None):
    nz, ny, nx, c = grid_shape
    ci, co, stride = _coords(coord_i, coord_o)
    g = grad_feature.contiguous()
    if out is None:
        out = torch.zeros(grid_shape, dtype=torch.float32, device=g.device)
    N.call("dv_integrate_bwd", N.ptr(g), nx, ny, nz, c, N.ptr(ci), N.ptr(co), stride, ci.shape[0], N.ptr(out),
           N.stream(g.device))
    return out


class Integrate(Function):
    @staticmethod
    def forward(ctx, voxels, coord_i, coord_o):
        ctx.grid_shape = tuple(voxels.shape)
        ctx.save_for_backward(coord_i, coord_o)
        return integrate_forward(voxels, coord_i, coord_o)

    @staticmethod
    def backward(ctx, grad):
        coord_i, coord_o = ctx.saved_tensors
        gv = integrate_backward(grad, ctx.grid_shape, coord_i, coord_o) if ctx.needs_input_grad[0] else None
        return gv, None, None


def integrate(voxels, coord_i, coord_o):
    """Integrated features [S, C] (reference utils/integrator.py:62-112)."""
    return Integrate.apply(voxels, coord_i, coord_o)


# --- implicit stage ----------------------------------------------------------

def corner_rows(coord_i: torch.Tensor, coord_o: torch.Tensor, n_vert: int) -> torch.Tensor:
    """[S, 8] int64 linear corner indices (z * n + y) * n + x (dv_corner_rows)."""
    ci, co, stride = _coords(coord_i, coord_o)
    rows = torch.empty(ci.shape[0], 8, dtype=torch.int64, device=ci.device)
    N.call("dv_corner_rows", N.ptr(ci), N.ptr(co), stride, ci.shape[0], int(n_vert), N.ptr(rows), N.stream(ci.device))
    return rows


class IntegrateTable(Function):
    """Integral over segments of features held in a table of corner rows."""

    @staticmethod
    def forward(ctx, table, rows, coord_i, coord_o):
        N.need_cuda("table", table, torch.float32)
        ci, co, stride = _coords(coord_i, coord_o)
        S, C = ci.shape[0], table.shape[1]
        out = torch.empty(S, C, dtype=torch.float32, device=table.device)
        N.call("dv_integrate_table_fwd", N.ptr(table), table.shape[0], C, N.ptr(rows), N.ptr(ci), N.ptr(co), stride, S,
               N.ptr(out), N.stream(table.device))
        ctx.save_for_backward(rows, coord_i, coord_o)
        ctx.table_shape = tuple(table.shape)
        return out

    @staticmethod
    def backward(ctx, grad):
        rows, coord_i, coord_o = ctx.saved_tensors
        if not ctx.needs_input_grad[0]:
            return None, None, None, None
        ci, co, stride = _coords(coord_i, coord_o)
        g = grad.contiguous()
        gt = torch.zeros(ctx.table_shape, dtype=torch.float32, device=g.device)
        N.call("dv_integrate_table_bwd", N.ptr(g), ctx.table_shape[0], ctx.table_shape[1], N.ptr(rows), N.ptr(ci),
               N.ptr(co), stride, ci.shape[0], N.ptr(gt), N.stream(g.device))
        return gt, None, None, None


def integrate_mlp(voxel_mlp, N_vert: int, C: int, coord_i: torch.Tensor, coord_o: torch.Tensor) -> torch.Tensor:
    """Integrated features [S, C] of an implicit grid (utils/integrator.py:3-59):
    the segments' corners, deduplicated, go through `voxel_mlp` (any torch
    module mapping [U, 3] positions (z, y, x) / (N / 2) - 1 to [U, C]
    features, e.g. the reference's ImplicitMLP: its GEMMs are library calls),
    and the integral reads the resulting table.  Gradients flow to the MLP."""
    rows = corner_rows(coord_i, coord_o, N_vert)
    rows_u, inv = torch.unique(rows.reshape(-1), return_inverse=True)
    n = int(N_vert)
    z, rem = rows_u // (n * n), rows_u % (n * n)
    y, x = rem // n, rem % n
    pts = torch.stack([z, y, x], -1).float() / (n * 0.5) - 1.0  # the reference's (z, y, x) corner order
    table = voxel_mlp(pts).float().contiguous()
    if table.shape[1] != C:
        raise ValueError(f"voxel_mlp returned {table.shape[1]} channels, expected {C}")
    return IntegrateTable.apply(table, inv.reshape(-1, 8).contiguous(), coord_i, coord_o)
