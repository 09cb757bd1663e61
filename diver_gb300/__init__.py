"""diver_gb300: GB300-native (sm_103a) DIVeR rendering hot path.

Operators keep the reference's names and tensor layouts so callers can swap
the import (reference modules in brackets):
  ray_voxel_intersect, masked_intersect   [utils.ray_voxel_intersection]
  aabb_intersect, ray_march               [utils.ray_march]
All compute runs in libdiver_gb300.so (C ABI: include/diver_gb300.h); there is
no CPU path.
"""
from .ray_march import aabb_intersect, build_octree_levels, ray_march
from .ray_voxel_intersection import (
    Segments,
    dense_segments,
    masked_intersect,
    masked_segments,
    ray_voxel_intersect,
)

__all__ = [
    "ray_voxel_intersect", "masked_intersect", "masked_segments", "dense_segments", "Segments",
    "aabb_intersect", "ray_march", "build_octree_levels",
]
