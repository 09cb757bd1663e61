"""Occupancy extraction: the reference's prune.py (:86-145 alpha map and mask,
:150-216 bias sampling) on the CUDA path.

  extract_alpha_map(field, rays)   alpha_map [N,N,N]: per voxel, the largest
                                   rendering weight alpha_i T_i of any training
                                   ray segment in it (the reference scatters
                                   with torch_scatter's max); voxels of the
                                   boundary band `pad` are left out
  prune_mask(alpha_map, thresh)    voxel_mask = alpha_map > thresh
  rays_hitting(field, o, d, mask)  which rays cross at least one voxel of the
                                   pruned mask (the bias-sampling selection:
                                   masked_intersect(...).mask.any(1))
"""
from __future__ import annotations

import torch

from . import _native as N
from .ray_voxel_intersection import _check_mask, _check_rays
from .renderer import DIVeRField


@torch.no_grad()
def extract_alpha_map(field: DIVeRField, rays, batch: int = 4000, pad: int = 0, form: str = "fp32") -> torch.Tensor:
    """rays: a [R, >=6] tensor (origin xyz, direction xyz, ...) or an iterable
    of them, on the field's device; processed `batch` rays at a time like the
    reference's loop.  Returns alpha_map [N, N, N] ([z][y][x])."""
    n = field.voxel_num
    alpha = torch.zeros(n, n, n, device=field.voxels.device)
    chunks = [rays] if isinstance(rays, torch.Tensor) else rays
    for r in chunks:
        for b in range(0, r.shape[0], batch):
            part = r[b:b + batch]
            field.accumulate_alpha(part[:, :3], part[:, 3:6], alpha, pad, form)
    return alpha


def prune_mask(alpha_map: torch.Tensor, thresh: float = 1e-2) -> torch.Tensor:
    return alpha_map > thresh


@torch.no_grad()
def rays_hitting(field: DIVeRField, o: torch.Tensor, d: torch.Tensor, voxel_mask: torch.Tensor,
                 mask_scale: float = 1.0) -> torch.Tensor:
    """bool [B]: the ray crosses at least one voxel set in voxel_mask."""
    o, d = o.contiguous(), d.contiguous()
    B = _check_rays(o, d)
    m8 = _check_mask(voxel_mask.contiguous(), field.voxel_num, mask_scale)
    num = torch.empty(B, dtype=torch.int32, device=o.device)
    if B:
        N.call("dv_masked_count", B, float(field.xyzmin), float(field.voxel_num), float(field.voxel_size),
               float(mask_scale), N.ptr(o), N.ptr(d), N.ptr(m8), N.ptr(num), None, None, N.stream(o.device))
    return num > 0
