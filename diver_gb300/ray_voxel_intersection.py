"""Ray–voxel traversal operators with the reference's interface.

Drop-in for utils/ray_voxel_intersection/__init__.py (reference :18-87):
`ray_voxel_intersect(o, v, xyzmin, xyzmax, voxel_num, voxel_size)` and
`masked_intersect(o, v, xyzmin, xyzmax, voxel_num, voxel_size, mask, mask_scale)`
return `(intersection[:, :K], tns >= 0, tns[:, :K])` with K = max count, the
same values the reference returns.  The reference fills [B, 3N] padded buffers
and slices them; here a counting walk finds K first (the same single host
read of max(count) the reference does) and the filling walk writes [B, K]
rows only.

`masked_segments` / `dense_segments` return the compacted segment lists that
DIVeR.extract_features builds from those buffers by boolean indexing
(model/diver.py:86-103), without the padded intermediate.
"""
from __future__ import annotations

import torch
from torch.autograd import Function

from . import _native as N


def _check_rays(o: torch.Tensor, v: torch.Tensor) -> int:
    N.need_cuda("o", o, torch.float32)
    N.need_cuda("v", v, torch.float32)
    if o.dim() != 2 or o.shape[1] != 3 or v.shape != o.shape:
        raise ValueError(f"o and v must be [B, 3] with equal shapes, got {tuple(o.shape)} and {tuple(v.shape)}")
    if o.device != v.device:
        raise ValueError("o and v must be on the same device")
    return o.shape[0]


def mask_side(voxel_num: float, mask_scale: float) -> int:
    """int(voxel_num * mask_scale) with the product rounded to float32, as the reference computes it."""
    return int(torch.tensor(float(voxel_num), dtype=torch.float32).mul(float(mask_scale)).item())


def _check_mask(mask: torch.Tensor, voxel_num: float, mask_scale: float) -> torch.Tensor:
    N.need_cuda("mask", mask)
    if mask.dtype not in (torch.bool, torch.uint8):
        raise TypeError(f"mask must be bool or uint8, got {mask.dtype}")
    m = mask_side(voxel_num, mask_scale)
    if mask.numel() != m * m * m:
        raise ValueError(f"mask must hold {m}^3 cells for voxel_num={voxel_num}, mask_scale={mask_scale}; got {tuple(mask.shape)}")
    return mask.view(torch.uint8) if mask.dtype == torch.bool else mask


def _max_count(counter: torch.Tensor) -> int:
    return int(counter.item())


class RayVoxelIntersect(Function):
    @staticmethod
    def forward(ctx, o, v, xyzmin, xyzmax, voxel_num, voxel_size):
        """Dense traversal (reference utils/ray_voxel_intersection/__init__.py:19-43).
        Returns B x K x 3 points, B x K hit indicator, B x K distances."""
        B = _check_rays(o, v)
        dev = o.device
        st = N.stream(dev)
        num = torch.empty(B, dtype=torch.int32, device=dev)
        mx = torch.zeros(1, dtype=torch.int32, device=dev)
        N.call("dv_ray_voxel_count", B, float(xyzmin), float(voxel_num), float(voxel_size),
               N.ptr(o), N.ptr(v), N.ptr(num), N.ptr(mx), st)
        K = _max_count(mx)
        inter = torch.zeros(B, K, 3, dtype=torch.float32, device=dev)
        tns = torch.full((B, K), -1.0, dtype=torch.float32, device=dev)
        if K > 0:
            N.call("dv_ray_voxel_intersect", B, K, float(xyzmin), float(xyzmax), float(voxel_num),
                   float(voxel_size), N.ptr(o), N.ptr(v), N.ptr(inter), N.ptr(num), N.ptr(tns), None, st)
        return inter, tns >= 0, tns

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None, None


class MaskedIntersect(Function):
    @staticmethod
    def forward(ctx, o, v, xyzmin, xyzmax, voxel_num, voxel_size, mask, mask_scale):
        """Masked traversal (reference utils/ray_voxel_intersection/__init__.py:51-79).
        Returns B x K x 6 (entry, exit), B x K hit indicator, B x K exit distances."""
        B = _check_rays(o, v)
        m8 = _check_mask(mask, voxel_num, mask_scale)
        dev = o.device
        st = N.stream(dev)
        num = torch.empty(B, dtype=torch.int32, device=dev)
        mx = torch.zeros(1, dtype=torch.int32, device=dev)
        N.call("dv_masked_count", B, float(xyzmin), float(voxel_num), float(voxel_size), float(mask_scale),
               N.ptr(o), N.ptr(v), N.ptr(m8), N.ptr(num), N.ptr(mx), None, st)
        K = _max_count(mx)
        inter = torch.zeros(B, K, 6, dtype=torch.float32, device=dev)
        tns = torch.full((B, K), -1.0, dtype=torch.float32, device=dev)
        if K > 0:
            N.call("dv_masked_intersect", B, K, float(xyzmin), float(xyzmax), float(voxel_num),
                   float(voxel_size), float(mask_scale), N.ptr(o), N.ptr(v), N.ptr(m8), N.ptr(inter),
                   N.ptr(num), N.ptr(tns), None, st)
        return inter, tns >= 0, tns

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None, None, None, None


ray_voxel_intersect = RayVoxelIntersect.apply
masked_intersect = MaskedIntersect.apply


def exclusive_scan(counts: torch.Tensor) -> torch.Tensor:
    """int32 counts [n] -> int64 offsets [n+1] on the device (no host sync)."""
    N.need_cuda("counts", counts, torch.int32)
    n = counts.numel()
    out = torch.empty(n + 1, dtype=torch.int64, device=counts.device)
    scratch = torch.empty(max(int(N.lib().dv_scan_scratch_bytes(n)), 8), dtype=torch.uint8, device=counts.device)
    N.call("dv_exclusive_scan", N.ptr(counts), n, N.ptr(out), N.ptr(scratch), N.stream(counts.device))
    return out


class Segments:
    """Compacted per-ray segment lists (CSR).

    offsets [B+1] int64, seg [S, 6] float32 (entry xyz, exit xyz, voxel units),
    t [S] float32 distances, ray [S] int32 ray index, counts [B] int32.

    Built with a fixed `capacity`, the buffers hold that many rows and only the
    first offsets[B] are segments; the count (offsets[B]) and max_dev (max
    segments per ray, int32 [1]) then stay on the device and max_count is None.
    """

    __slots__ = ("offsets", "seg", "t", "ray", "counts", "max_count", "max_dev")

    def __init__(self, offsets, seg, t, ray, counts, max_count=None, max_dev=None):
        self.offsets, self.seg, self.t, self.ray, self.counts = offsets, seg, t, ray, counts
        self.max_dev = max_dev
        if max_dev is not None:
            self.max_count = max_count
        else:
            self.max_count = int(counts.max()) if max_count is None and counts.numel() else (max_count or 0)

    @property
    def coord_in(self) -> torch.Tensor:
        return self.seg[:, :3]

    @property
    def coord_out(self) -> torch.Tensor:
        return self.seg[:, 3:]

    @property
    def total(self) -> int:
        """Rows of the buffers: the segment count, or the capacity."""
        return self.seg.shape[0]

    @property
    def count_ptr(self) -> int | None:
        """Device address of the segment count (offsets[B]) for the decode entry points."""
        if self.offsets.numel() == 0:
            return None
        return self.offsets.data_ptr() + (self.offsets.numel() - 1) * self.offsets.element_size()


def _totals(offsets: torch.Tensor, counts: torch.Tensor) -> tuple[int, int]:
    """(total segments, max per ray) with a single device-to-host read."""
    if counts.numel() == 0:
        return 0, 0
    S, M = torch.stack([offsets[-1], counts.max().to(torch.int64)]).tolist()
    return int(S), int(M)


def _capacity(capacity: int, B: int, planes: int) -> int:
    need = B * (planes + 3)
    if capacity < need:
        raise ValueError(f"capacity {capacity} is below the {need} segments that {B} rays can produce")
    return int(capacity)


def _buffers(S: int, dev):
    return (torch.empty(S, 6, dtype=torch.float32, device=dev), torch.empty(S, dtype=torch.float32, device=dev),
            torch.empty(S, dtype=torch.int32, device=dev))


class SlotWalk:
    """The first half of a fixed-capacity masked traversal: every ray's
    segments in its own range of `slot` rows, the per-ray counts, their
    exclusive scan and the longest ray, all on the device."""

    __slots__ = ("sseg", "st", "num", "offsets", "mx", "slot", "S")

    def __init__(self, sseg, st, num, offsets, mx, slot, S):
        self.sseg, self.st, self.num, self.offsets, self.mx, self.slot, self.S = sseg, st, num, offsets, mx, slot, S


def masked_slot_walk(o, v, xyzmin, voxel_num, voxel_size, mask, mask_scale, capacity: int) -> SlotWalk:
    """Walks the rays into per-ray slots (dv_masked_segments_slots) and scans
    the counts on the device; compact_slot_walk turns the result into CSR
    segments."""
    B = _check_rays(o, v)
    m8 = _check_mask(mask, voxel_num, mask_scale)
    dev = o.device
    S = _capacity(capacity, B, 3 * int(voxel_num))
    slot = 3 * int(voxel_num) + 3
    num = torch.empty(B, dtype=torch.int32, device=dev)
    mx = torch.zeros(1, dtype=torch.int32, device=dev)
    sseg = torch.empty(B * slot, 6, dtype=torch.float32, device=dev)
    st = torch.empty(B * slot, dtype=torch.float32, device=dev)
    if B > 0:
        N.call("dv_masked_segments_slots", B, float(xyzmin), float(voxel_num), float(voxel_size), float(mask_scale),
               N.ptr(o), N.ptr(v), N.ptr(m8), slot, N.ptr(sseg), N.ptr(st), N.ptr(num), N.ptr(mx), N.stream(dev))
    return SlotWalk(sseg, st, num, exclusive_scan(num), mx, slot, S)


def compact_slot_walk(w: SlotWalk) -> Segments:
    """CSR segments of a slot walk (dv_compact_slots), in buffers of the walk's capacity."""
    B = w.num.numel()
    dev = w.num.device
    seg, t, ray = _buffers(w.S, dev)
    if B > 0:
        N.call("dv_compact_slots", B, w.slot, N.ptr(w.offsets), N.ptr(w.sseg), N.ptr(w.st), N.ptr(seg), N.ptr(t),
               N.ptr(ray), N.stream(dev))
    return Segments(w.offsets, seg, t, ray, w.num, None, w.mx)


class PendingSegments:
    """An exact masked traversal whose count walk and scan are queued on the
    device: finish() reads the total back (one host read) and queues the
    emission walk.  Launching the count walks of several batches (on their
    own streams) before finishing any lets them run together."""

    __slots__ = ("args", "num", "offsets", "last")

    def __init__(self, args, num, offsets, last):
        self.args, self.num, self.offsets, self.last = args, num, offsets, last

    def finish(self) -> Segments:
        o, v, xyzmin, voxel_num, voxel_size, m8, mask_scale = self.args
        dev = o.device
        S, M = _totals(self.offsets, self.num)
        seg, t, ray = _buffers(S, dev)
        if S > 0:
            N.call("dv_masked_segments", self.num.numel(), float(xyzmin), float(voxel_num), float(voxel_size),
                   float(mask_scale), N.ptr(o), N.ptr(v), N.ptr(m8), N.ptr(self.offsets), N.ptr(seg), N.ptr(t),
                   N.ptr(ray), N.ptr(self.last), N.stream(dev))
        return Segments(self.offsets, seg, t, ray, self.num, M, None)


def masked_segments_begin(o, v, xyzmin, voxel_num, voxel_size, mask, mask_scale) -> PendingSegments:
    """The first half of masked_segments without capacity: count walk and scan."""
    B = _check_rays(o, v)
    m8 = _check_mask(mask, voxel_num, mask_scale)
    dev = o.device
    num = torch.empty(B, dtype=torch.int32, device=dev)
    last = torch.empty(B, dtype=torch.int32, device=dev)  # where each ray's emission walk may stop
    if B > 0:
        N.call("dv_masked_count", B, float(xyzmin), float(voxel_num), float(voxel_size), float(mask_scale),
               N.ptr(o), N.ptr(v), N.ptr(m8), N.ptr(num), None, N.ptr(last), N.stream(dev))
    return PendingSegments((o, v, xyzmin, voxel_num, voxel_size, m8, mask_scale), num, exclusive_scan(num), last)


def masked_segments(o, v, xyzmin, voxel_num, voxel_size, mask, mask_scale, capacity: int | None = None) -> Segments:
    """Segments of occupied voxels; equals coord[mask] of masked_intersect's output
    (model/diver.py:86-93), t = exit distance.  With `capacity`: fixed-size
    buffers, no host read (see Segments)."""
    if capacity is None:
        return masked_segments_begin(o, v, xyzmin, voxel_num, voxel_size, mask, mask_scale).finish()
    if o.shape[0] > 0:
        # fixed capacity: one walk writes every ray into its own range of rows
        # (slots), then the slots are compacted into the CSR lists
        return compact_slot_walk(masked_slot_walk(o, v, xyzmin, voxel_num, voxel_size, mask, mask_scale, capacity))
    B = _check_rays(o, v)
    _check_mask(mask, voxel_num, mask_scale)
    dev = o.device
    S = _capacity(capacity, B, 3 * int(voxel_num))
    seg, t, ray = _buffers(S, dev)
    return Segments(torch.zeros(1, dtype=torch.int64, device=dev), seg, t, ray,
                    torch.empty(0, dtype=torch.int32, device=dev), None, torch.zeros(1, dtype=torch.int32, device=dev))


def dense_segments(o, v, xyzmin, voxel_num, voxel_size, capacity: int | None = None) -> Segments:
    """Consecutive crossing points paired into segments; equals
    (coord[:, :-1][mask], coord[:, 1:][mask]) of model/diver.py:95-103, t = entry distance.
    With `capacity`: fixed-size buffers, no host read (see Segments)."""
    B = _check_rays(o, v)
    dev = o.device
    st = N.stream(dev)
    num = torch.empty(B, dtype=torch.int32, device=dev)
    N.call("dv_ray_voxel_count", B, float(xyzmin), float(voxel_num), float(voxel_size),
           N.ptr(o), N.ptr(v), N.ptr(num), None, st)
    pairs = torch.empty_like(num)
    N.call("dv_dense_pair_counts", B, N.ptr(num), N.ptr(pairs), st)
    offsets = exclusive_scan(pairs)
    mx = None
    if capacity is None:
        S, M = _totals(offsets, pairs)
    else:
        S, M = _capacity(capacity, B, 3 * int(voxel_num)), None
        mx = pairs.max().reshape(1) if B > 0 else torch.zeros(1, dtype=torch.int32, device=dev)
    seg, t, ray = _buffers(S, dev)
    if S > 0 and B > 0:
        N.call("dv_dense_segments", B, float(xyzmin), float(voxel_num), float(voxel_size),
               N.ptr(o), N.ptr(v), N.ptr(offsets), N.ptr(seg), N.ptr(t), N.ptr(ray), st)
    return Segments(offsets, seg, t, ray, pairs, M, mx)


def masked_segments_grid(o, v, xyzmin, dims, voxel_size, mask, capacity: int | None = None) -> Segments:
    """Occupied-voxel segments over a grid with per-axis extents: xyzmin = world
    position of corner (0,0,0) per axis, dims = (nx, ny, nz) voxels, mask
    [nz][ny][nx].  The reference supports cubic grids only; with equal values on
    the three axes this is exactly masked_segments with mask_scale 1."""
    B = _check_rays(o, v)
    nx, ny, nz = (int(x) for x in dims)
    N.need_cuda("mask", mask)
    if mask.numel() != nx * ny * nz:
        raise ValueError(f"mask must hold {nz}x{ny}x{nx} cells, got {tuple(mask.shape)}")
    m8 = mask.view(torch.uint8) if mask.dtype == torch.bool else mask
    import ctypes

    x0 = (ctypes.c_float * 3)(*[float(x) for x in xyzmin])
    dd = (ctypes.c_int * 3)(nx, ny, nz)
    dev = o.device
    st = N.stream(dev)
    num = torch.empty(B, dtype=torch.int32, device=dev)
    last = torch.empty(B, dtype=torch.int32, device=dev)
    mx = torch.zeros(1, dtype=torch.int32, device=dev) if capacity is not None else None
    N.call("dv_masked_count_grid", B, ctypes.addressof(x0), ctypes.addressof(dd), float(voxel_size), N.ptr(o), N.ptr(v),
           N.ptr(m8), N.ptr(num), N.ptr(mx), N.ptr(last), st)
    offsets = exclusive_scan(num)
    if capacity is None:
        S, M = _totals(offsets, num)
    else:
        S, M = _capacity(capacity, B, nx + ny + nz), None
    seg, t, ray = _buffers(S, dev)
    if S > 0 and B > 0:
        N.call("dv_masked_segments_grid", B, ctypes.addressof(x0), ctypes.addressof(dd), float(voxel_size), N.ptr(o),
               N.ptr(v), N.ptr(m8), N.ptr(offsets), N.ptr(seg), N.ptr(t), N.ptr(ray), N.ptr(last), st)
    return Segments(offsets, seg, t, ray, num, M, mx)
