"""Real-time traversal operators with the reference's interface.

Drop-in for utils/ray_march/__init__.py (reference :16-17):
`aabb_intersect(o, v, center, finish, rgba, octrees, voxel_num)` and
`ray_march(o, v, mask, finish, voxel_num)`, both mutating caller-owned
buffers in place exactly as the reference's extension does
(utils/ray_march/src/ray_march.cpp:20-51).  `o` is the [8, H, W, 6] hit buffer,
`v` the [H, W, 3] directions; the batch is v.numel() // 3 as in the reference
(v.size(0) * v.size(1)).  Unlike the reference, nothing synchronises the
device and any N that is a multiple of 64 is accepted (the reference
instantiates 128 and 256 only).
"""
from __future__ import annotations

import torch
import torch.nn.functional as NF

from . import _native as N


def _u8(name: str, t: torch.Tensor) -> torch.Tensor:
    N.need_cuda(name, t)
    if t.dtype == torch.bool:
        return t.view(torch.uint8)
    if t.dtype != torch.uint8:
        raise TypeError(f"{name} must be bool or uint8, got {t.dtype}")
    return t


def _batch(o: torch.Tensor, v: torch.Tensor) -> int:
    N.need_cuda("o", o, torch.float32)
    N.need_cuda("v", v, torch.float32)
    if v.shape[-1] != 3:
        raise ValueError("v must end in a dimension of 3")
    B = v.numel() // 3
    if o.numel() != 8 * B * 6:
        raise ValueError(f"o must hold [8, B, 6] floats for B={B}, got {tuple(o.shape)}")
    return B


def aabb_intersect(o, v, center, finish, rgba, octrees, voxel_num):
    """First occupied 4^3 block per ray (reference utils/ray_march/src/ray_march.cu:237-266)."""
    B = _batch(o, v)
    N.need_cuda("center", center, torch.float32)
    N.need_cuda("rgba", rgba, torch.float32)
    fin = _u8("finish", finish)
    oct8 = _u8("octrees", octrees)
    n = int(voxel_num)
    if n % 64 != 0:
        raise ValueError(f"voxel_num must be a multiple of 64, got {n}")
    cells = (n // 64) ** 3 + (n // 16) ** 3 + (n // 4) ** 3
    if oct8.numel() != cells:
        raise ValueError(f"octrees must hold {cells} cells for voxel_num={n}, got {oct8.numel()}")
    if fin.numel() != B or rgba.numel() != 4 * B:
        raise ValueError("finish must hold B entries and rgba B x 4")
    N.call("dv_aabb_intersect", B, N.ptr(o), N.ptr(v), N.ptr(center), N.ptr(fin), N.ptr(rgba),
           N.ptr(oct8), n, N.stream(o.device))


def ray_march(o, v, mask, finish, voxel_num):
    """Next <= 8 occupied voxels per unfinished ray (reference utils/ray_march/src/ray_march.cu:268-296)."""
    B = _batch(o, v)
    m8 = _u8("mask", mask)
    fin = _u8("finish", finish)
    n = int(voxel_num)
    if m8.numel() != n ** 3:
        raise ValueError(f"mask must hold {n}^3 cells, got {m8.numel()}")
    if fin.numel() != B:
        raise ValueError("finish must hold B entries")
    N.call("dv_ray_march", B, N.ptr(o), N.ptr(v), N.ptr(m8), N.ptr(fin), n, N.stream(o.device))


def build_octree_levels(voxel_mask: torch.Tensor) -> torch.Tensor:
    """The reference's three max-pooled occupancy levels (scales 64, 16, 4),
    flattened and concatenated coarsest first (eval_rt.py:76-79)."""
    m = voxel_mask[None, None].float()
    levels = [NF.max_pool3d(m, s, stride=s)[0, 0].bool().reshape(-1) for s in (64, 16, 4)]
    return torch.cat(levels, 0).contiguous()
