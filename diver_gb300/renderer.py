"""Training / offline render path: traversal -> integral -> decoder -> compositing.

`render_segments` is a torch.autograd.Function over the CUDA pipeline:
  forward   dv_ray_pe, dv_decode_fwd, dv_composite_fwd
  backward  dv_composite_bwd, dv_decode_bwd (recomputes each segment's decode
            instead of storing activations; grid gradient by vector atomics)
It returns per-ray rgb and the reference's sparsity term
mean(log(1 + sigma^2 / 0.5)) over the padded [B, M] sigma (train.py:84-85),
so `mse(rgb, target) + l_s * reg` is the reference's training loss
(train.py:109-113) and autograd delivers gradients for the feature grid and
the packed decoder parameters.

`DIVeRField` bundles a scene's grid, occupancy mask and decoder the way the
reference's DIVeR module does (model/diver.py:16-207) for callers that want a
module.
"""
from __future__ import annotations

import torch
from torch.autograd import Function

from . import _native as N
from .decoder import Decoder, pack_plain, tc_index_maps
from .ray_voxel_intersection import (Segments, dense_segments, masked_segments, masked_segments_begin,
                                     masked_segments_grid)

KIND_ID = {"diver32": 32, "diver64": 64}
WIDTH = {32: 32, 64: 64}

# Optional per-kernel timing: when set to a dict, the pipeline records a CUDA
# event pair (on the launching stream) around each decoder / compositing launch,
# keyed by entry-point name.
KERNEL_EVENTS: dict | None = None


def _timed(name: str, *args) -> None:
    if KERNEL_EVENTS is None:
        N.call(name, *args)
        return
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    N.call(name, *args)
    e.record()
    KERNEL_EVENTS.setdefault(name, []).append((s, e))


def _grid(voxels: torch.Tensor):
    N.need_cuda("voxels", voxels, torch.float32)
    if voxels.dim() != 4 or voxels.shape[-1] not in (32, 64):
        raise ValueError(f"voxels must be [Nz, Ny, Nx, 32|64], got {tuple(voxels.shape)}")
    nz, ny, nx, c = voxels.shape
    return nx, ny, nz, c


def _check_params(kind: int, channels: int, params: torch.Tensor):
    n = N.lib().dv_decoder_param_count(kind, channels)
    if n <= 0:
        raise ValueError(f"unsupported decoder kind {kind} with {channels} channels")
    N.need_cuda("params", params, torch.float32)
    if params.numel() != n:
        raise ValueError(f"packed decoder must hold {n} floats, got {params.numel()}")


# Decoder forms: 'fp32' (plain FP32 kernels), 'bf16' / 'fp16' (tensor-core
# decoder with 16-bit operands: the render form; a 16-bit copy of the grid
# without autograd), 'bf16s' (tensor-core decoder with split BF16 operands:
# FP32-grade products from BF16 tensor cores, the accurate training form).
FORMS = ("fp32", "bf16", "fp16", "bf16s")


class TcWeights:
    """Decoder weights in the tensor-core operand layout on the device.  The
    images are gathered from the packed plain parameters on the device
    (`refresh`), into buffers that keep their addresses, so a refresh after an
    optimizer step needs no host round trip and can sit inside a captured CUDA
    graph.  mode: 'bf16', 'fp16', or 'bf16s' (every image as three BF16 terms,
    one after the other, for the split-operand kernels)."""

    def __init__(self, kind: str, channels: int, device, bf16: bool = True, mode: str | None = None):
        mode = mode or ("bf16" if bf16 else "fp16")
        if mode not in ("bf16", "fp16", "bf16s"):
            raise ValueError(f"unknown tensor-core form {mode!r}")
        maps = tc_index_maps(kind, channels)
        self.kind, self.channels, self.mode = kind, channels, mode
        self.bf16 = mode != "fp16"
        self.terms = 3 if mode == "bf16s" else 1
        self.dtype = torch.float16 if mode == "fp16" else torch.bfloat16
        self._i_fwd = maps["fwd"].to(device)
        self._i_bias = maps["bias"].to(device)
        self.table = maps["table"].contiguous()
        self.term_bytes = self._i_fwd.numel() * 2
        self.blob = torch.zeros(self.terms * self.term_bytes, dtype=torch.uint8, device=device)
        self.bias = torch.zeros(self._i_bias.numel(), dtype=torch.float32, device=device)
        self.err = torch.zeros(1, dtype=torch.int32, device=device)
        self.bwd = None
        self._i_bwd = None
        if "bwd" in maps and self.bf16:
            self._i_bwd = maps["bwd"].to(device)
            self.bwd = (torch.zeros(self.terms * self._i_bwd.numel() * 2, dtype=torch.uint8, device=device),
                        maps["bwd_table"].contiguous())
        self.version = None

    @staticmethod
    def from_decoder(decoder: Decoder, device, bf16: bool = True, mode: str | None = None) -> "TcWeights":
        tw = TcWeights(decoder.kind, decoder.channels, device, bf16, mode)
        tw.refresh(pack_plain(decoder).to(device))
        return tw

    def _fill(self, blob: torch.Tensor, index: torch.Tensor, params: torch.Tensor, form: int) -> None:
        _timed("dv_tc_image", N.ptr(params), params.numel(), N.ptr(index), index.numel(), form, N.ptr(blob),
               N.stream(params.device))

    def refresh(self, params: torch.Tensor) -> None:
        """Rebuilds the images from the packed plain parameters: one gather
        launch per image (dv_tc_image), no host round trip."""
        p = params.detach().reshape(-1).contiguous()
        N.need_cuda("params", p, torch.float32)
        form = 3 if self.terms > 1 else (2 if self.mode == "fp16" else 1)
        self._fill(self.blob, self._i_fwd, p, form)
        self._fill(self.bias, self._i_bias, p, 0)
        if self.bwd is not None:
            self._fill(self.bwd[0], self._i_bwd, p, form)

    def save_buffer(self, kind: int, channels: int, n_seg: int, device) -> torch.Tensor | None:
        """Buffer for the forward's layer inputs, read back by the tensor-core
        backward (None when this decoder / form has no tensor-core backward)."""
        if self.bwd is None:
            return None
        fn = "dv_decode_tc_split_save_bytes" if self.terms > 1 else "dv_decode_tc_save_bytes"
        n = int(getattr(N.lib(), fn)(kind, channels, n_seg))
        return torch.empty(max(n, 16), dtype=torch.uint8, device=device)

    def marks_rows(self, saved) -> bool:
        """Whether backward() with this save buffer also sets the row marks
        of dv_mark_corner_rows (the split form does, in its scatter)."""
        return self.bwd is not None and self.terms > 1 and saved is not None

    def backward(self, kind, voxels, seg, pe_feat, pe_out, d4, gv, gp, st, saved=None, out4=None,
                 touched=None) -> bool:
        """Tensor-core backward (DIVeR32, BF16 / split BF16); False when this
        decoder / form has none (the caller then runs the FP32 CUDA backward).
        With `saved` (the forward's save buffer) and its `out4` the forward is
        read back instead of recomputed; the split form requires it, and sets
        the row marks in `touched` when given (marks_rows)."""
        if self.bwd is None or (self.terms > 1 and saved is None):
            return False
        nx, ny, nz, c = _grid(voxels)
        wb, tb = self.bwd
        if self.terms > 1:
            _timed("dv_decode_bwd_tc_split", kind, c, N.ptr(wb), wb.numel() // self.terms, tb.data_ptr(),
                   tb.shape[0], nx, ny, nz, N.ptr(seg.seg), N.ptr(seg.ray), seg.total, seg.count_ptr,
                   N.ptr(pe_feat), N.ptr(d4), N.ptr(saved), saved.numel(), N.ptr(out4), N.ptr(gv), N.ptr(gp),
                   N.ptr(touched), N.ptr(self.err), st)
            return True
        _timed("dv_decode_bwd_tc", kind, c, int(self.bf16), N.ptr(self.blob), self.blob.numel(), N.ptr(self.bias),
               self.bias.numel(), self.table.data_ptr(), N.ptr(wb), wb.numel(), tb.data_ptr(), tb.shape[0],
               N.ptr(voxels), nx, ny, nz, N.ptr(seg.seg), N.ptr(seg.ray), seg.total, seg.count_ptr, N.ptr(pe_feat),
               N.ptr(pe_out), N.ptr(d4), N.ptr(saved), 0 if saved is None else saved.numel(),
               N.ptr(out4 if saved is not None else None), N.ptr(gv), N.ptr(gp), N.ptr(self.err), st)
        return True

    def decode(self, kind, channels, voxels, seg, pe_out, out4, st, voxels16=None, save=None):
        nx, ny, nz, c = _grid(voxels)
        if self.terms > 1:
            _timed("dv_decode_fwd_tc_split", kind, c, N.ptr(self.blob), self.term_bytes, N.ptr(self.bias),
                   self.bias.numel(), self.table.data_ptr(), self.table.shape[0], N.ptr(voxels), nx, ny, nz,
                   N.ptr(seg.seg), N.ptr(seg.ray), seg.total, seg.count_ptr, N.ptr(pe_out), N.ptr(out4),
                   N.ptr(save), 0 if save is None else save.numel(), N.ptr(self.err), st)
            return
        _timed("dv_decode_fwd_tc", kind, c, int(self.bf16), N.ptr(self.blob), self.blob.numel(), N.ptr(self.bias),
               self.bias.numel(), self.table.data_ptr(), self.table.shape[0], N.ptr(voxels), N.ptr(voxels16),
               nx, ny, nz, N.ptr(seg.seg), N.ptr(seg.ray), seg.total, seg.count_ptr, N.ptr(pe_out), N.ptr(out4),
               N.ptr(save), 0 if save is None else save.numel(), N.ptr(self.err), st)


class SegmentRender(Function):
    @staticmethod
    def forward(ctx, voxels, params, seg: Segments, dirs, kind: int, white_back: bool, tc: TcWeights | None = None,
                voxels16: torch.Tensor | None = None, training: bool = False, grad_voxels=None, pe=None):
        nx, ny, nz, c = _grid(voxels)
        _check_params(kind, c, params)
        N.need_cuda("dirs", dirs, torch.float32)
        B = dirs.shape[0]
        dev = voxels.device
        st = N.stream(dev)
        W = WIDTH[kind]
        if pe is None:
            pe_feat = torch.empty(B, 28, device=dev)
            pe_out = torch.empty(B, W, device=dev)
            _timed("dv_ray_pe", kind, c, N.ptr(params), B, N.ptr(dirs), N.ptr(pe_feat), N.ptr(pe_out), st)
        else:
            pe_feat, pe_out = pe
        S = seg.total
        out4 = torch.empty(S, 4, device=dev)
        if tc is None:
            _timed("dv_decode_fwd", kind, c, N.ptr(params), N.ptr(voxels), nx, ny, nz, N.ptr(seg.seg), N.ptr(seg.ray),
                   S, seg.count_ptr, N.ptr(pe_out), N.ptr(out4), st)
        else:
            # training: keep the layer inputs for the tensor-core backward
            save = tc.save_buffer(kind, c, S, dev) if training else None
            tc.decode(kind, c, voxels, seg, pe_out, out4, st, voxels16, save)
            ctx.saved_layers = save
        rgb = torch.empty(B, 3, device=dev)
        reg = torch.empty(B, device=dev)
        _timed("dv_composite_fwd", B, N.ptr(seg.offsets), N.ptr(out4), int(bool(white_back)), N.ptr(rgb), None,
               N.ptr(reg), st)
        # mean over the padded [B, M]; M (max segments per ray) stays on the
        # device when the segments were built without a host read
        reg_mean = torch.empty((), device=dev)
        inv_m = torch.empty(1, device=dev)
        on_dev = seg.max_count is None
        _timed("dv_reg_mean", B, N.ptr(reg), N.ptr(seg.max_dev) if on_dev else None,
               0.0 if on_dev else float(seg.max_count), N.ptr(reg_mean), N.ptr(inv_m), st)
        ctx.save_for_backward(voxels, params, dirs, pe_feat, pe_out, out4, rgb)
        ctx.seg, ctx.kind, ctx.inv_m, ctx.tc, ctx.grad_voxels = seg, kind, inv_m, tc, grad_voxels
        return rgb, reg_mean

    @staticmethod
    def backward(ctx, g_rgb, g_reg):
        voxels, params, dirs, pe_feat, pe_out, out4, rgb = ctx.saved_tensors
        seg = ctx.seg
        nx, ny, nz, c = _grid(voxels)
        dev = voxels.device
        st = N.stream(dev)
        B = dirs.shape[0]
        g_rgb = (g_rgb if g_rgb is not None else torch.zeros(B, 3, device=dev)).contiguous()
        # d reg / d sigma carries dL/dreg / (B M): 1/B on the host, dL/dreg / M
        # as a device scalar (no host read of either)
        scale = None
        if g_reg is not None:
            scale = (g_reg.detach().float().reshape(1) * ctx.inv_m).contiguous()
        d4 = torch.empty_like(out4)
        _timed("dv_composite_bwd", B, N.ptr(seg.offsets), N.ptr(out4), N.ptr(rgb), N.ptr(g_rgb),
               1.0 / B if scale is not None else 0.0, N.ptr(scale), N.ptr(d4), st)
        if ctx.grad_voxels is not None:
            # caller-owned buffer, zeroed on another stream while the forward
            # ran; wait for that, then mark the rows this step writes when the
            # caller clears only those (dv_clear_marked_rows)
            gv, filled, *touched = ctx.grad_voxels
            touched = touched[0] if touched else None
            torch.cuda.current_stream(dev).wait_event(filled)
        else:
            gv, touched = torch.zeros_like(voxels), None
        saved = getattr(ctx, "saved_layers", None)
        # the split tensor-core backward sets the row marks in its scatter
        if touched is not None and not (ctx.tc is not None and ctx.tc.marks_rows(saved)):
            N.call("dv_mark_corner_rows", N.ptr(seg.seg), seg.total, seg.count_ptr, nx, ny, nz, N.ptr(touched), st)
            touched = None
        gp = torch.zeros_like(params)
        if ctx.tc is not None and ctx.tc.backward(ctx.kind, voxels, seg, pe_feat, pe_out, d4, gv, gp, st, saved, out4,
                                                  touched):
            return gv, gp, None, None, None, None, None, None, None, None, None
        _timed("dv_decode_bwd", ctx.kind, c, N.ptr(params), N.ptr(voxels), nx, ny, nz, N.ptr(seg.seg), N.ptr(seg.ray),
               seg.total, seg.count_ptr, N.ptr(pe_feat), N.ptr(pe_out), N.ptr(d4), N.ptr(gv), N.ptr(gp), st)
        return gv, gp, None, None, None, None, None, None, None, None, None


class L2Loss(Function):
    """mse(rgb, target) + l_s * reg (train.py:84-85,109-113) as one launch
    forward (dv_l2_loss_fwd) and one backward (dv_l2_loss_bwd)."""

    @staticmethod
    def forward(ctx, rgb, reg, target, l_s: float):
        dev = rgb.device
        loss = torch.empty((), device=dev)
        _timed("dv_l2_loss_fwd", rgb.numel(), N.ptr(rgb), N.ptr(target), N.ptr(reg), l_s, N.ptr(loss),
               N.stream(dev))
        ctx.save_for_backward(rgb, target)
        ctx.l_s = l_s
        return loss

    @staticmethod
    def backward(ctx, g):
        rgb, target = ctx.saved_tensors
        d_rgb = torch.empty_like(rgb)
        d_reg = torch.empty((), device=rgb.device)
        g = g.detach().float().contiguous()
        _timed("dv_l2_loss_bwd", rgb.numel(), N.ptr(rgb), N.ptr(target), N.ptr(g), ctx.l_s, N.ptr(d_rgb),
               N.ptr(d_reg), N.stream(rgb.device))
        return d_rgb, d_reg, None, None


def l2_loss(rgb: torch.Tensor, reg: torch.Tensor, target: torch.Tensor, l_s: float) -> torch.Tensor:
    """The training loss mean((rgb - target)^2) + l_s * reg of a render (reg:
    the sparsity term, a 0-d tensor), differentiable in rgb and reg."""
    N.need_cuda("rgb", rgb, torch.float32)
    N.need_cuda("target", target, torch.float32)
    N.need_cuda("reg", reg, torch.float32)
    if target.shape != rgb.shape or reg.numel() != 1:
        raise ValueError("target must match rgb and reg must be a single value")
    return L2Loss.apply(rgb, reg, target, float(l_s))


def render_segments(voxels, params, seg: Segments, dirs, kind="diver32", white_back=True, tc: TcWeights | None = None,
                    voxels16: torch.Tensor | None = None, grad_voxels=None, pe=None):
    """(rgb [B,3], sparsity term) for the CSR segments of B rays.  `tc` selects
    the tensor-core decoder; `voxels16` (inference) is a BF16/FP16 copy of the
    grid the tensor-core forward reads its corner rows from.  grad_voxels
    (training, optional): (buffer, event) — a grid-shaped buffer that is all
    zeros once `event` has completed; the grid gradient is accumulated into it
    and returned as it, so its zero fill can overlap the forward.  A third
    element, a uint8 byte per grid row, has the backward mark the rows it
    writes (dv_mark_corner_rows) for the caller's next dv_clear_marked_rows.
    pe (optional): (pe_feat [B,28], pe_out [B,W]) of dv_ray_pe for these
    directions and parameters, when the caller computed them already."""
    # whether a backward will follow is known here, not inside the Function's
    # forward (which always runs with grad mode off): only then does the
    # tensor-core forward keep its layer tiles for the backward
    training = torch.is_grad_enabled() and (voxels.requires_grad or params.requires_grad)
    return SegmentRender.apply(voxels, params, seg, dirs, KIND_ID.get(kind, kind), white_back, tc, voxels16, training,
                               grad_voxels, pe)


class DIVeRField(torch.nn.Module):
    """Explicit-grid DIVeR on the CUDA path: voxels [N+1]^3 x C and a packed
    decoder as parameters, an occupancy mask as a buffer."""

    def __init__(self, voxels: torch.Tensor, decoder: Decoder, mask: torch.Tensor | None, xyzmin,
                 voxel_size: float, mask_scale: float = 1.0, white_back: bool = True):
        super().__init__()
        self.voxels = torch.nn.Parameter(voxels.contiguous())
        self.params = torch.nn.Parameter(pack_plain(decoder).to(voxels.device))
        self.register_buffer("voxel_mask", None if mask is None else mask.contiguous())
        self.kind = decoder.kind
        self.voxel_num = voxels.shape[0] - 1
        self.dims = (voxels.shape[2] - 1, voxels.shape[1] - 1, voxels.shape[0] - 1)  # (nx, ny, nz)
        self.aniso = isinstance(xyzmin, (tuple, list)) or len(set(self.dims)) > 1
        self.xyzmin = tuple(float(x) for x in xyzmin) if isinstance(xyzmin, (tuple, list)) else float(xyzmin)
        self.voxel_size = float(voxel_size)
        self.mask_scale = float(mask_scale)
        self.white_back = white_back
        self.decoder = decoder
        self._tc = {}
        self.refresh_always = False

    def tc_weights(self, form: str) -> TcWeights | None:
        """Tensor-core weights for form 'bf16' / 'fp16' / 'bf16s' (None for
        'fp32'), refreshed on the device whenever the decoder parameters
        changed (or on every call while `refresh_always` is set, as inside a
        captured graph, so that each replay packs the parameters of that
        moment)."""
        if form not in FORMS:
            raise ValueError(f"unknown decoder form {form!r} (one of {FORMS})")
        if form == "fp32":
            return None
        tw = self._tc.get(form)
        if tw is None:
            tw = self._tc[form] = TcWeights(self.kind, self.voxels.shape[-1], self.voxels.device, mode=form)
        if self.refresh_always or tw.version != self.params._version:
            tw.refresh(self.params)
            tw.version = self.params._version
        return tw

    @staticmethod
    def from_scene(scene, device="cuda") -> "DIVeRField":
        return DIVeRField(scene.features.to(device), scene.decoder, scene.mask.to(device), scene.xyzmin,
                          scene.voxel_size, scene.mask_scale, scene.white_back)

    def segment_capacity(self, batch: int) -> int:
        """Segments that `batch` rays can produce at most: a ray crosses at most
        nx + ny + nz + 3 grid planes, one per walk step."""
        return batch * (sum(self.dims) + 3)

    def segments(self, os: torch.Tensor, ds: torch.Tensor, capacity: int | None = None) -> Segments:
        """CSR segments of the rays.  With `capacity` (at least
        segment_capacity(B)) the buffers have that fixed size and the count
        stays on the device: no host read, so the call can be captured."""
        if self.aniso:
            x0 = self.xyzmin if isinstance(self.xyzmin, tuple) else (self.xyzmin,) * 3
            return masked_segments_grid(os, ds, x0, self.dims, self.voxel_size, self.voxel_mask, capacity)
        if self.voxel_mask is not None:
            return masked_segments(os, ds, self.xyzmin, self.voxel_num, self.voxel_size, self.voxel_mask,
                                   self.mask_scale, capacity)
        return dense_segments(os, ds, self.xyzmin, self.voxel_num, self.voxel_size, capacity)

    def begin_segments(self, os: torch.Tensor, ds: torch.Tensor):
        """Exact segments in two halves: the count walk and scan are queued now and
        the returned object's finish() reads the total and queues the emission
        (an occupancy-masked cubic grid; other grids are traversed at once and
        returned finished)."""
        if self.aniso or self.voxel_mask is None:
            return self.segments(os, ds)
        return masked_segments_begin(os.contiguous(), ds.contiguous(), self.xyzmin, self.voxel_num, self.voxel_size,
                                     self.voxel_mask, self.mask_scale)

    def grid16(self, form: str) -> torch.Tensor | None:
        """BF16/FP16 copy of the feature grid for tensor-core rendering (made
        once per grid version; None for the FP32 and split forms, which read
        the FP32 grid)."""
        if form in ("fp32", "bf16s"):
            return None
        key = ("grid16", form, self.voxels._version)
        if getattr(self, "_g16key", None) != key:
            dt = torch.bfloat16 if form == "bf16" else torch.float16
            self._g16 = self.voxels.detach().to(dt).contiguous()
            self._g16key = key
        return self._g16

    @torch.no_grad()
    def accumulate_alpha(self, os: torch.Tensor, ds: torch.Tensor, alpha_map: torch.Tensor, pad: int = 0,
                         form: str = "fp32") -> None:
        """alpha_map [N,N,N] (x fastest) = max(alpha_map, rendering weight) over
        the voxels the rays' segments cross (prune.py:86-131)."""
        N.need_cuda("alpha_map", alpha_map, torch.float32)
        if alpha_map.numel() != self.voxel_num ** 3 or self.aniso:
            raise ValueError("alpha_map must hold voxel_num^3 cells of a cubic grid")
        os, ds = os.contiguous(), ds.contiguous()
        seg = self.segments(os, ds)
        if seg.total == 0:
            return
        nx, ny, nz, c = _grid(self.voxels)
        kind = KIND_ID[self.kind]
        dev, st, B = self.voxels.device, N.stream(self.voxels.device), ds.shape[0]
        pe_feat = torch.empty(B, 28, device=dev)
        pe_out = torch.empty(B, WIDTH[kind], device=dev)
        _timed("dv_ray_pe", kind, c, N.ptr(self.params), B, N.ptr(ds), N.ptr(pe_feat), N.ptr(pe_out), st)
        out4 = torch.empty(seg.total, 4, device=dev)
        tc = self.tc_weights(form)
        if tc is None:
            _timed("dv_decode_fwd", kind, c, N.ptr(self.params), N.ptr(self.voxels), nx, ny, nz, N.ptr(seg.seg),
                   N.ptr(seg.ray), seg.total, seg.count_ptr, N.ptr(pe_out), N.ptr(out4), st)
        else:
            tc.decode(kind, c, self.voxels, seg, pe_out, out4, st, self.grid16(form))
        _timed("dv_occupancy_max", B, N.ptr(seg.offsets), N.ptr(out4), N.ptr(seg.seg), self.voxel_num, int(pad),
               N.ptr(alpha_map), st)

    def forward(self, os: torch.Tensor, ds: torch.Tensor, form: str = "fp32", capacity: int | None = None,
                grad_voxels=None, segments: Segments | None = None):
        """(rgb [B,3], sparsity term); reference DIVeR.forward + render (model/diver.py:141-207).
        form: 'fp32' (plain), 'bf16' or 'fp16' (tensor-core decoder; without
        autograd they read a 16-bit copy of the grid) or 'bf16s' (tensor-core
        decoder with split BF16 operands: FP32-grade, the accurate training form).
        capacity: fixed segment buffers, no host synchronisation (see segments).
        grad_voxels: see render_segments.
        segments: the rays' segments when the caller traversed them already
        (the traversal is then skipped)."""
        os, ds = os.contiguous(), ds.contiguous()
        N.need_cuda("dirs", ds, torch.float32)
        dev = self.voxels.device
        kind = KIND_ID[self.kind]
        # the tensor-core weight images and the directions' encoding do not
        # depend on the segments: they run on a side stream beside the
        # traversal, which occupies one warp per SM (the outputs are
        # allocated on the calling stream, which waits for the side stream)
        main = torch.cuda.current_stream(dev)
        side = self._side_stream(dev)
        pe = (torch.empty(ds.shape[0], 28, device=dev), torch.empty(ds.shape[0], WIDTH[kind], device=dev))
        side.wait_stream(main)
        with torch.cuda.stream(side):
            tc = self.tc_weights(form)
            if ds.shape[0]:
                _check_params(kind, self.voxels.shape[-1], self.params)
                _timed("dv_ray_pe", kind, self.voxels.shape[-1], N.ptr(self.params), ds.shape[0], N.ptr(ds),
                       N.ptr(pe[0]), N.ptr(pe[1]), N.stream(dev))
        seg = segments if segments is not None else self.segments(os, ds, capacity)
        main.wait_stream(side)
        g16 = self.grid16(form) if not torch.is_grad_enabled() else None
        return render_segments(self.voxels, self.params, seg, ds, self.kind, self.white_back, tc, g16, grad_voxels,
                               pe)

    def _side_stream(self, dev) -> torch.cuda.Stream:
        s = getattr(self, "_side", None)
        if s is None or s.device != dev:
            s = self._side = torch.cuda.Stream(dev)
        return s
