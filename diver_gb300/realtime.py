"""Real-time path: serialized model, reference-compatible operators, frame loop.

  convert(state_dict, alpha_map)   the reference's convert.py (:17-161): sparse
                                   feature table of the 8 corners of every
                                   occupied voxel, folded/packed decoder params
  RealtimeModel.from_serialized    eval_rt.py:52-82: voxel index map, occupancy
                                   mask, three max-pooled octree levels; the
                                   packed weights re-laid out for the kernel
  RealtimeModel.render_frame       eval_rt.py:115-122: aabb_intersect, then
                                   rounds of ray_march + mlp_eval until every
                                   pixel is finished; rgb = rgba.rgb + T

The decoder kind is taken from the decoder's own layers (mlp1.4 present means
DIVeR32).  The reference chooses by feature width (convert.py:63), which sends
a DIVeR64 decoder over 32-channel features into the DIVeR32 branch and fails;
here DIVeR64 over 32 channels packs to the layout its kernel reads
(utils/mlp_evaluation64/src/mlp_eval.cu: 8288 floats).
"""
from __future__ import annotations

import torch

from . import _native as N
from .decoder import Decoder, pack_realtime, premultiply_features
from .ray_march import aabb_intersect, build_octree_levels, ray_march


def convert(state_dict: dict, alpha_map: torch.Tensor, thresh: float = 1e-2) -> dict:
    """Serialized real-time model {'f','i','m','p'} from a training state dict
    (keys as DIVeR's: voxels, mlp1.*, mlp2.*) and the alpha map of prune.py."""
    sd = {k.replace("model.", ""): v for k, v in state_dict.items() if "mlp_voxel" not in k}
    voxel_mask = alpha_map > thresh
    kind = "diver32" if "mlp1.4.weight" in sd else "diver64"
    dec = Decoder.from_state_dict(kind, sd)
    voxels = sd["voxels"].float()
    dev = voxels.device
    voxel_mask = voxel_mask.to(dev)
    nv = voxels.shape[0]
    occ = torch.nonzero(voxel_mask)  # [K,3] (z, y, x) of occupied voxels
    offs = torch.stack(torch.meshgrid(*[torch.arange(2, device=dev)] * 3, indexing="ij"), -1).reshape(-1, 3)
    idx = (occ[None] + offs[:, None]).reshape(-1, 3).unique(dim=0)  # sorted lexicographically
    feats = voxels[idx[:, 0], idx[:, 1], idx[:, 2]]
    feats = premultiply_features(dec, feats) if kind == "diver32" else feats.contiguous()
    n = nv - 1
    valid = (idx < n).all(1)
    m = torch.zeros(idx.shape[0], dtype=torch.bool, device=dev)
    iv = idx[valid]
    m[valid] = voxel_mask[iv[:, 0], iv[:, 1], iv[:, 2]]
    inds = idx[:, 0] * nv * nv + idx[:, 1] * nv + idx[:, 2]
    return {"f": feats.contiguous(), "i": inds.int(), "m": m, "p": pack_realtime(dec), "kind": kind}


class RealtimeModel:
    """A resident real-time model: feature table, index map, occupancy, octree
    levels and packed decoder weights, all on one device (several can coexist)."""

    def __init__(self, features, voxel_map, voxel_masks, octrees, packed, width, voxel_num, xyzmin, voxel_size):
        self.features, self.voxel_map, self.voxel_masks = features, voxel_map, voxel_masks
        self.octrees, self.packed, self.width = octrees, packed, width
        self.voxel_num, self.xyzmin, self.voxel_size = voxel_num, xyzmin, voxel_size

    @staticmethod
    def pack_params(ref_params: torch.Tensor, width: int, device) -> torch.Tensor:
        p = ref_params.to(device=device, dtype=torch.float32).contiguous()
        out = torch.empty(N.lib().dv_realtime_packed_size(width), device=device)
        N.call("dv_realtime_pack", width, N.ptr(p), N.ptr(out), N.stream(device))
        return out

    @staticmethod
    def from_serialized(ser: dict, voxel_num: int, xyzmin: float, voxel_size: float, device="cuda",
                        width: int | None = None) -> "RealtimeModel":
        nv = voxel_num + 1
        inds = ser["i"].to(device).long()
        ii, rem = inds // (nv * nv), inds % (nv * nv)
        jj, kk = rem // nv, rem % nv
        masks = torch.zeros(voxel_num, voxel_num, voxel_num, dtype=torch.bool, device=device)
        mm = ser["m"].to(device).bool()
        masks[ii[mm], jj[mm], kk[mm]] = True
        vmap = torch.zeros(nv, nv, nv, dtype=torch.int32, device=device)
        vmap[ii, jj, kk] = torch.arange(inds.numel(), dtype=torch.int32, device=device)
        p = ser["p"]
        if width is None:
            width = 32 if p.numel() == 3168 else 64
        masks = masks.contiguous()
        return RealtimeModel(ser["f"].to(device).float().contiguous(), vmap.contiguous(), masks,
                             build_octree_levels(masks), RealtimeModel.pack_params(p, width, device), width,
                             voxel_num, xyzmin, voxel_size)

    def tc_blob(self) -> torch.Tensor:
        """Tensor-core images of the folded layers (three BF16 terms), made once
        per model from the aligned params on the device."""
        blob = getattr(self, "_tc_blob", None)
        if blob is None:
            dev = self.packed.device
            blob = torch.empty(N.lib().dv_realtime_tc_bytes(self.width), dtype=torch.uint8, device=dev)
            N.call("dv_realtime_tc_pack", self.width, N.ptr(self.packed), N.ptr(blob), N.stream(dev))
            self._tc_blob = blob
            self.tc_err = torch.zeros(1, dtype=torch.int32, device=dev)
        return blob

    def mlp_eval(self, rgba, coords, v, finish, tensor_cores: bool = False):
        """One round of the fused decoder on the recorded hits (mlp_eval.cu:32-231),
        in place on rgba / finish; tensor_cores: the tcgen05 form (dv_mlp_eval_tc)."""
        fin = finish.view(torch.uint8) if finish.dtype == torch.bool else finish
        B = v.numel() // 3
        if tensor_cores:
            blob = self.tc_blob()
            N.call("dv_mlp_eval_tc", self.width, B, N.ptr(coords), N.ptr(self.features), N.ptr(self.voxel_map),
                   self.voxel_map.shape[0], N.ptr(self.packed), N.ptr(blob), N.ptr(v), N.ptr(rgba), N.ptr(fin),
                   N.ptr(self.tc_err), N.stream(v.device))
            return
        N.call("dv_mlp_eval", self.width, B, N.ptr(coords), N.ptr(self.features), N.ptr(self.voxel_map),
               self.voxel_map.shape[0], N.ptr(self.packed), N.ptr(v), N.ptr(rgba), N.ptr(fin), N.stream(v.device))

    def render_frame(self, eye: torch.Tensor, dirs: torch.Tensor, max_rounds: int | None = None,
                     fused: bool | None = None, mode: str = "tc"):
        """rgb [B,3] of B rays from camera centre `eye` (world) with unit
        directions `dirs` [B,3] (eval_rt.py:106-122); also returns the number of
        host rounds.  mode:
          "tc"     (default) the reference's loop of aabb_intersect, then rounds
                   of ray_march + the tensor-core decoder (dv_mlp_eval_tc,
                   FP32-grade) until every pixel is finished
          "fused"  the whole frame in one launch with the FP32 decoder
                   (dv_realtime_frame)
          "loop"   the reference's loop with the FP32 decoder (dv_mlp_eval);
                   same result as "fused"
        fused=True / False select "fused" / "loop" (the earlier form of this
        argument); max_rounds caps the rounds of the loops."""
        if fused is not None:
            mode = "fused" if fused else "loop"
        if mode not in ("tc", "fused", "loop"):
            raise ValueError(f"unknown real-time frame mode {mode!r}")
        dev = dirs.device
        B = dirs.shape[0]
        v = dirs.contiguous()
        center = ((eye.float().cpu() - self.xyzmin) / self.voxel_size).to(dev).contiguous()
        if mode == "fused":
            rgba = torch.empty(B, 4, device=dev)
            m8 = self.voxel_masks.view(torch.uint8) if self.voxel_masks.dtype == torch.bool else self.voxel_masks
            o8 = self.octrees.view(torch.uint8) if self.octrees.dtype == torch.bool else self.octrees
            N.call("dv_realtime_frame", self.width, B, N.ptr(v), N.ptr(center), N.ptr(o8), self.voxel_num, N.ptr(m8),
                   N.ptr(self.features), N.ptr(self.voxel_map), self.voxel_map.shape[0], N.ptr(self.packed),
                   N.ptr(rgba), N.stream(dev))
            return rgba[:, :3] + rgba[:, 3:], 1
        coords = torch.zeros(8, B, 6, device=dev)
        rgba = torch.zeros(B, 4, device=dev)
        finish = torch.zeros(B, dtype=torch.bool, device=dev)
        aabb_intersect(coords, v, center, finish, rgba, self.octrees, self.voxel_num)
        rounds = 0
        limit = max_rounds if max_rounds is not None else 3 * self.voxel_num
        if mode == "loop":
            while rounds < limit and not bool(finish.all()):
                ray_march(coords, v, self.voxel_masks, finish, self.voxel_num)
                self.mlp_eval(rgba, coords, v, finish, False)
                rounds += 1
            return rgba[:, :3] + rgba[:, 3:], rounds
        # "tc": the host learns one round late that every pixel has finished, so
        # round k + 1 is queued while it waits for round k's flag (a round after
        # the last pixel finished changes nothing; the frame is the same, the
        # round count at most one higher)
        if getattr(self, "_flags", None) is None:
            self._flags = (torch.zeros(2, dtype=torch.bool, pin_memory=True), [torch.cuda.Event(), torch.cuda.Event()])
        flags, events = self._flags
        while rounds < limit:
            ray_march(coords, v, self.voxel_masks, finish, self.voxel_num)
            self.mlp_eval(rgba, coords, v, finish, True)
            rounds += 1
            slot = rounds % 2
            flags[slot:slot + 1].copy_(finish.all().reshape(1), non_blocking=True)
            events[slot].record()
            if rounds >= 2:
                events[1 - slot].synchronize()
                if bool(flags[1 - slot]):
                    break
        return rgba[:, :3] + rgba[:, 3:], rounds


# --- module-level drop-in for utils.mlp_evaluation / utils.mlp_evaluation64 ------

_CURRENT: dict[int, tuple] = {}


def upload_weight(device_id: int, params: torch.Tensor, voxel_map: torch.Tensor, width: int = 32):
    """Reference upload_weight (utils/mlp_evaluation/__init__.py:30-41): makes
    (params, voxel_map) the model that `mlp_eval` uses.  The buffers stay
    per-width device tensors instead of a global texture and constant bank."""
    dev = torch.device("cuda", device_id)
    packed = RealtimeModel.pack_params(params, width, dev)
    _CURRENT[width] = (packed, voxel_map.to(dev, torch.int32).contiguous())
    return torch.Tensor([0])


def mlp_eval(rgba, coord, voxels, v, mask, width: int = 32):
    """Reference mlp_eval (utils/mlp_evaluation/__init__.py:18-28), in place on rgba / mask."""
    if width not in _CURRENT:
        raise RuntimeError("upload_weight must be called before mlp_eval")
    packed, vmap = _CURRENT[width]
    N.need_cuda("voxels", voxels, torch.float32)
    fin = mask.view(torch.uint8) if mask.dtype == torch.bool else mask
    B = v.numel() // 3
    N.call("dv_mlp_eval", width, B, N.ptr(coord), N.ptr(voxels), N.ptr(vmap), vmap.shape[0], N.ptr(packed), N.ptr(v),
           N.ptr(rgba), N.ptr(fin), N.stream(v.device))
    return torch.Tensor([0])
