"""Feature integrator with the reference's interface.

Drop-in for `integrate(voxels, coord_i, coord_o)` of utils/integrator.py:62,
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
