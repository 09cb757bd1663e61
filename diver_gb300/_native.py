"""ctypes binding of libdiver_gb300.so (the C ABI declared in include/diver_gb300.h).

There is no fallback: if the library cannot be loaded (or built, when nvcc is
present and the library is missing or stale) every operator raises.
"""
from __future__ import annotations

import ctypes as C
import threading

import torch

from . import build as _build

_lock = threading.Lock()
_lib = None

P = C.c_void_p
I32 = C.c_int
I64 = C.c_longlong
F32 = C.c_float

# name -> (restype, argtypes)
SIGNATURES = {
    "dv_version": (I32, []),
    "dv_status_string": (C.c_char_p, [I32]),
    "dv_ray_voxel_intersect": (I32, [I32, I32, F32, F32, F32, F32, P, P, P, P, P, P, P]),
    "dv_ray_voxel_count": (I32, [I32, F32, F32, F32, P, P, P, P, P]),
    "dv_masked_intersect": (I32, [I32, I32, F32, F32, F32, F32, F32, P, P, P, P, P, P, P, P]),
    "dv_masked_count": (I32, [I32, F32, F32, F32, F32, P, P, P, P, P, P, P]),
    "dv_masked_segments": (I32, [I32, F32, F32, F32, F32, P, P, P, P, P, P, P, P, P]),
    "dv_masked_segments_slots": (I32, [I32, F32, F32, F32, F32, P, P, P, I64, P, P, P, P, P]),
    "dv_compact_slots": (I32, [I32, I64, P, P, P, P, P, P, P]),
    "dv_masked_count_grid": (I32, [I32, P, P, F32, P, P, P, P, P, P, P]),
    "dv_masked_segments_grid": (I32, [I32, P, P, F32, P, P, P, P, P, P, P, P, P]),
    "dv_dense_segments": (I32, [I32, F32, F32, F32, P, P, P, P, P, P, P]),
    "dv_dense_pair_counts": (I32, [I32, P, P, P]),
    "dv_camera_rays": (I32, [I32, I32, F32, P, I64, I64, P, P, P]),
    "dv_scan_scratch_bytes": (I64, [I64]),
    "dv_walk_cap_hits": (I64, [I32]),
    "dv_exclusive_scan": (I32, [P, I64, P, P, P]),
    "dv_exclusive_scan_static_max": (I64, []),
    "dv_exclusive_scan_static": (I32, [P, I64, P, P]),
    "dv_integrate_fwd": (I32, [P, I32, I32, I32, I32, P, P, I64, I64, P, P]),
    "dv_integrate_bwd": (I32, [P, I32, I32, I32, I32, P, P, I64, I64, P, P]),
    "dv_corner_rows": (I32, [P, P, I64, I64, I32, P, P]),
    "dv_mark_corner_rows": (I32, [P, I64, P, I32, I32, I32, P, P]),
    "dv_clear_marked_rows": (I32, [P, I32, I32, I32, I32, P, P]),
    "dv_integrate_table_fwd": (I32, [P, I64, I32, P, P, P, I64, I64, P, P]),
    "dv_integrate_table_bwd": (I32, [P, I64, I32, P, P, P, I64, I64, P, P]),
    "dv_decoder_param_count": (I32, [I32, I32]),
    "dv_ray_pe": (I32, [I32, I32, P, I32, P, P, P, P]),
    "dv_decode_fwd": (I32, [I32, I32, P, P, I32, I32, I32, P, P, I64, P, P, P, P]),
    "dv_composite_fwd": (I32, [I32, P, P, I32, P, P, P, P]),
    "dv_composite_bwd": (I32, [I32, P, P, P, P, F32, P, P, P]),
    "dv_reg_mean": (I32, [I32, P, P, F32, P, P, P]),
    "dv_l2_loss_fwd": (I32, [I64, P, P, P, F32, P, P]),
    "dv_l2_loss_bwd": (I32, [I64, P, P, P, F32, P, P, P]),
    "dv_occupancy_max": (I32, [I32, P, P, P, I32, I32, P, P]),
    "dv_decode_bwd": (I32, [I32, I32, P, P, I32, I32, I32, P, P, I64, P, P, P, P, P, P, P]),
    "dv_decode_fwd_tc": (I32, [I32, I32, I32, P, I32, P, I32, P, I32, P, P, I32, I32, I32, P, P, I64, P, P, P, P, I64, P,
                               P]),
    "dv_decode_tc_save_bytes": (I64, [I32, I32, I64]),
    "dv_decode_fwd_tc_split": (I32, [I32, I32, P, I32, P, I32, P, I32, P, I32, I32, I32, P, P, I64, P, P, P, P, I64,
                                     P, P]),
    "dv_decode_tc_split_save_bytes": (I64, [I32, I32, I64]),
    "dv_tc_image": (I32, [P, I64, P, I64, I32, P, P]),
    "dv_decode_bwd_tc_split": (I32, [I32, I32, P, I32, P, I32, I32, I32, I32, P, P, I64, P, P, P, P, I64, P, P, P,
                                     P, P, P]),
    "dv_wait_selftest": (I32, [I32, P, P]),
    "dv_decode_bwd_tc": (I32, [I32, I32, I32, P, I32, P, I32, P, P, I32, P, I32, P, I32, I32, I32, P, P, I64, P, P,
                               P, P, P, I64, P, P, P, P, P]),
    "dv_realtime_packed_size": (I32, [I32]),
    "dv_realtime_pack": (I32, [I32, P, P, P]),
    "dv_mlp_eval": (I32, [I32, I32, P, P, P, I32, P, P, P, P, P]),
    "dv_realtime_tc_bytes": (I32, [I32]),
    "dv_realtime_tc_pack": (I32, [I32, P, P, P]),
    "dv_mlp_eval_tc": (I32, [I32, I32, P, P, P, I32, P, P, P, P, P, P, P]),
    "dv_realtime_frame": (I32, [I32, I32, P, P, P, I32, P, P, P, I32, P, P, P]),
    "dv_aabb_intersect": (I32, [I32, P, P, P, P, P, P, I32, P]),
    "dv_ray_march": (I32, [I32, P, P, P, P, I32, P]),
}


def lib():
    """Returns the loaded library, building it first if it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = _build.LIB
            if not _build.up_to_date():
                path = _build.build()
            handle = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def call(name: str, *args) -> None:
    """Calls an entry point and raises RuntimeError on a non-zero status."""
    st = getattr(lib(), name)(*args)
    if st != 0:
        msg = lib().dv_status_string(st).decode()
        raise RuntimeError(f"{name} failed: {msg} (status {st})")


def ptr(t: torch.Tensor | None) -> int | None:
    return None if t is None else t.data_ptr()


def stream(device: torch.device | None = None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def need_cuda(name: str, t: torch.Tensor, dtype: torch.dtype | None = None) -> None:
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise ValueError(f"{name} must be a CUDA tensor (diver_gb300 has no CPU path)")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must have dtype {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
