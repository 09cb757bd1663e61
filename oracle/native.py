"""ORACLE — test infrastructure only.  ctypes + numpy wrappers of the C
restatements in dda.c and mlp_eval.c (see oracle/__init__.py)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import build as _build

_lib = None
P = C.c_void_p
I = C.c_int
F = C.c_float


def lib():
    global _lib
    if _lib is None:
        h = C.CDLL(str(_build.build()))
        h.oracle_dense_walk.argtypes = [I, I, F, F, F, P, P, P, P, P, I]
        h.oracle_masked_walk.argtypes = [I, I, F, F, F, F, P, P, P, P, P, P, I]
        h.oracle_masked_walk_grid.argtypes = [I, I, P, P, F, P, P, P, P, P, P]
        h.oracle_masked_walk_grid.restype = None
        h.oracle_aabb.argtypes = [I, P, P, P, P, P, P, I, I]
        h.oracle_ray_march.argtypes = [I, P, P, P, P, I, I]
        for n in ("oracle_mlp_eval_f32", "oracle_mlp_eval_f64"):
            getattr(h, n).argtypes = [I, I, P, P, P, I, P, P, P, P]
        h.oracle_walk_cap_hits.argtypes = [I]
        h.oracle_walk_cap_hits.restype = C.c_longlong
        for n in ("oracle_dense_walk", "oracle_masked_walk", "oracle_aabb", "oracle_ray_march",
                  "oracle_mlp_eval_f32", "oracle_mlp_eval_f64"):
            getattr(h, n).restype = None
        _lib = h
    return _lib


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32))


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def dense_walk(o, v, xyzmin, voxel_num, voxel_size, max_n=None, fused=True):
    """Reference ray_voxel_intersect_kernel on the CPU: (intersection [B,max_n,3], num [B], tns [B,max_n])."""
    o, v = _f32(o), _f32(v)
    B = o.shape[0]
    max_n = int(voxel_num * 3) + 1 if max_n is None else max_n
    inter = np.zeros((B, max_n, 3), np.float32)
    tns = np.full((B, max_n), -1.0, np.float32)
    num = np.zeros(B, np.int32)
    lib().oracle_dense_walk(B, max_n, xyzmin, float(voxel_num), voxel_size, _p(o), _p(v), _p(inter), _p(num),
                            _p(tns), int(fused))
    return inter, num, tns


def masked_walk(o, v, xyzmin, voxel_num, voxel_size, mask, mask_scale, max_n=None, fused=True):
    o, v = _f32(o), _f32(v)
    m = np.ascontiguousarray(np.asarray(mask).astype(np.uint8))
    B = o.shape[0]
    max_n = int(voxel_num * 3) if max_n is None else max_n
    inter = np.zeros((B, max_n, 6), np.float32)
    tns = np.full((B, max_n), -1.0, np.float32)
    num = np.zeros(B, np.int32)
    lib().oracle_masked_walk(B, max_n, xyzmin, float(voxel_num), voxel_size, mask_scale, _p(o), _p(v), _p(m),
                             _p(inter), _p(num), _p(tns), int(fused))
    return inter, num, tns


def masked_walk_grid(o, v, xyzmin, dims, voxel_size, mask, max_n=None):
    """Masked walk over a per-axis grid: xyzmin (3,), dims (nx, ny, nz), mask [nz][ny][nx]."""
    o, v = _f32(o), _f32(v)
    m = np.ascontiguousarray(np.asarray(mask).astype(np.uint8))
    x0 = _f32(xyzmin)
    dd = np.ascontiguousarray(np.asarray(dims, np.int32))
    B = o.shape[0]
    max_n = int(sum(dims)) if max_n is None else max_n
    inter = np.zeros((B, max_n, 6), np.float32)
    tns = np.full((B, max_n), -1.0, np.float32)
    num = np.zeros(B, np.int32)
    lib().oracle_masked_walk_grid(B, max_n, _p(x0), _p(dd), voxel_size, _p(o), _p(v), _p(m), _p(inter), _p(num),
                                  _p(tns))
    return inter, num, tns


def trim(inter, num, tns):
    """The reference's slice to max(count) (utils/ray_voxel_intersection/__init__.py:41-43)."""
    k = int(num.max()) if num.size else 0
    return inter[:, :k], tns[:, :k] >= 0, tns[:, :k]


def aabb(coords, v, center, finish, rgba, octrees, N, fused=True):
    """In place, like the reference extension."""
    lib().oracle_aabb(finish.size, _p(coords), _p(_f32(v)), _p(_f32(center)), _p(finish), _p(rgba),
                      _p(np.ascontiguousarray(octrees.astype(np.uint8))), int(N), int(fused))


def ray_march(coords, v, mask, finish, N, fused=True):
    lib().oracle_ray_march(finish.size, _p(coords), _p(_f32(v)), _p(np.ascontiguousarray(mask.astype(np.uint8))),
                           _p(finish), int(N), int(fused))


def mlp_eval(width, coords, feats, vmap, params, v, rgba, finish, double=False):
    """In place on rgba/finish (float32 / uint8 numpy arrays)."""
    fn = lib().oracle_mlp_eval_f64 if double else lib().oracle_mlp_eval_f32
    vmap = np.ascontiguousarray(vmap.astype(np.int32))
    ms = round(vmap.size ** (1 / 3))
    fn(int(width), finish.size, _p(_f32(coords)), _p(_f32(feats)), _p(vmap), ms, _p(_f32(params)), _p(_f32(v)),
       _p(rgba), _p(finish))


def csr_from_padded(inter, num):
    """Rows [b, :num[b]] of a padded buffer, concatenated ray by ray (boolean-mask order)."""
    return np.concatenate([inter[b, :num[b]] for b in range(inter.shape[0])], 0) if inter.shape[0] else inter[:0, 0]


def walk_cap_hits(reset: bool = True) -> int:
    """Walks of the C restatement that stopped at their step bound since the last reset."""
    return int(lib().oracle_walk_cap_hits(int(reset)))
