"""CUDA-graph forms of the training step and of frame rendering.

The eager pipeline reads two numbers back to the host per step (the segment
count, to size the segment buffers, and the longest ray, for the sparsity
term's mean over the padded [B, M]) and pays Python and launch overhead for
about twenty launches.  With fixed-capacity segment buffers
(`DIVeRField.segments(..., capacity)`) both numbers stay on the device, every
launch reads its sizes there, and the whole step, traversal through weight
gradients, is recorded once in a CUDA graph and replayed.

  TrainStepGraph   loss = mse(rgb, target) + l_s * reg and its gradients for
                   the feature grid and the packed decoder parameters
                   (train.py:84-85,109-113), for a fixed batch size
  RenderGraph      rgb of a fixed number of rays (no autograd)

Inputs are copied into the graph's own buffers before each replay; outputs
are the graph's buffers (overwritten by the next replay; clone to keep them).
The grid gradient is zeroed on a second stream at the start of the step, and
the backward waits for that.  By default only the rows the previous replay
wrote are zeroed (dv_clear_marked_rows; the backward marks its segments'
corner cells with dv_mark_corner_rows): about a fifth of a 256^3 x 32 grid's
2.2 GB for a 4096-ray batch.  The returned grid gradient must then be treated
as read-only between replays (clone it to change it); sparse_clear=False
zero-fills the whole buffer every step instead.
The tensor-core weight images are repacked from the parameters inside the
graph, so optimizer steps between replays are seen by the next replay.
"""
from __future__ import annotations

import torch

from . import _native as N
from .renderer import DIVeRField, _grid, l2_loss


def _warm_and_capture(fn, warmup: int):
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(warmup):
            fn()
    torch.cuda.current_stream().wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        out = fn()
    return graph, out


class TrainStepGraph:
    """One captured training step of `field` on batches shaped like the
    example (o [B,3], d [B,3], target [B,3])."""

    def __init__(self, field: DIVeRField, o: torch.Tensor, d: torch.Tensor, target: torch.Tensor,
                 form: str = "bf16", l_s: float = 1e-5, warmup: int = 2, sparse_clear: bool = True):
        self.field, self.form, self.l_s = field, form, float(l_s)
        self.o, self.d, self.target = o.clone().contiguous(), d.clone().contiguous(), target.clone().contiguous()
        self.capacity = field.segment_capacity(o.shape[0])
        self._grid_grad = torch.zeros_like(field.voxels)
        self._shape = _grid(field.voxels)
        nx, ny, nz, _ = self._shape
        # a byte per grid row: the cells whose corners the last replay wrote
        self._touched = torch.zeros(nz * ny * nx, dtype=torch.uint8, device=o.device) if sparse_clear else None
        self._fill = torch.cuda.Stream(o.device)
        field.refresh_always = True
        try:
            self.graph, (self.loss, self.grad_voxels, self.grad_params) = _warm_and_capture(self._step, warmup)
        finally:
            field.refresh_always = False

    def _step(self):
        f = self.field
        main = torch.cuda.current_stream()
        self._fill.wait_stream(main)  # the previous step's use of the buffer is done
        with torch.cuda.stream(self._fill):
            if self._touched is None:
                self._grid_grad.zero_()
            else:
                nx, ny, nz, c = self._shape
                N.call("dv_clear_marked_rows", N.ptr(self._grid_grad), c, nx, ny, nz, N.ptr(self._touched),
                       N.stream(self._grid_grad.device))
            filled = torch.cuda.Event()
            filled.record()
        rgb, reg = f(self.o, self.d, form=self.form, capacity=self.capacity,
                     grad_voxels=(self._grid_grad, filled, self._touched))
        loss = l2_loss(rgb, reg, self.target, self.l_s)
        gv, gp = torch.autograd.grad(loss, [f.voxels, f.params])
        return loss.detach(), gv, gp

    def __call__(self, o: torch.Tensor, d: torch.Tensor, target: torch.Tensor):
        """(loss, grad_voxels, grad_params) of this batch: the graph's own
        buffers, overwritten by the next replay.  With sparse clearing (the
        default) only the grid-gradient rows a replay writes are zeroed before
        the next one, so grad_voxels is read-only for the caller: clone it
        before changing it (an optimizer or hook that adds into it in place
        would carry its change into every later step)."""
        self.o.copy_(o, non_blocking=True)
        self.d.copy_(d, non_blocking=True)
        self.target.copy_(target, non_blocking=True)
        self.graph.replay()
        return self.loss, self.grad_voxels, self.grad_params


class RenderGraph:
    """Captured forward render of B rays (o, d like the example)."""

    def __init__(self, field: DIVeRField, o: torch.Tensor, d: torch.Tensor, form: str = "bf16", warmup: int = 2):
        self.field, self.form = field, form
        self.o, self.d = o.clone().contiguous(), d.clone().contiguous()
        self.capacity = field.segment_capacity(o.shape[0])
        field.refresh_always = True
        try:
            with torch.no_grad():
                self.graph, self.rgb = _warm_and_capture(self._render, warmup)
        finally:
            field.refresh_always = False

    def _render(self):
        rgb, _ = self.field(self.o, self.d, form=self.form, capacity=self.capacity)
        return rgb

    def __call__(self, o: torch.Tensor, d: torch.Tensor) -> torch.Tensor:
        self.o.copy_(o, non_blocking=True)
        self.d.copy_(d, non_blocking=True)
        self.graph.replay()
        return self.rgb
