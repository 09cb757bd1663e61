"""GPU: clearing a grid gradient only where a step wrote it
(dv_mark_corner_rows + dv_clear_marked_rows) and the captured training step
that uses it.

Exact checks: after marking a step's segments and clearing, the zeroed rows
are exactly the union of the segments' 8 corner rows (lower corner
min(int(p0 + 1e-4), int(p1 + 1e-4)) per axis, upper corner clamped to the grid,
as the integration computes them), every other row keeps its value, and the
byte map is all zero again.  Graph replays with sparse clearing give the same
loss and gradients as the dense fill (1e-5 relative to the largest magnitude:
atomics accumulate in a different order) and leave no row of an earlier
batch non-zero."""
import pytest
import torch

from diver_gb300 import _native as N

pytestmark = pytest.mark.gpu


def corner_rows(seg: torch.Tensor, nx: int, ny: int, nz: int) -> torch.Tensor:
    """Linear row indices [S, 8] of each segment's corners (float32 arithmetic)."""
    p0 = seg[:, :3].float().cpu()
    p1 = seg[:, 3:].float().cpu()
    eps = torch.tensor(1e-4, dtype=torch.float32)
    lo = torch.minimum((p0 + eps).long(), (p1 + eps).long())
    hi_lim = torch.tensor([nx - 1, ny - 1, nz - 1])
    lo = torch.maximum(torch.minimum(lo, hi_lim), torch.zeros(3, dtype=torch.long))
    hi = torch.minimum(lo + 1, hi_lim)
    rows = []
    for j in range(8):
        x = hi[:, 0] if j & 1 else lo[:, 0]
        y = hi[:, 1] if j & 2 else lo[:, 1]
        z = hi[:, 2] if j & 4 else lo[:, 2]
        rows.append((z * ny + y) * nx + x)
    return torch.stack(rows, 1)


def walk_segments(n_vox: int, rays: int, seed: int):
    """Segments of `rays` random rays through an n_vox^3 grid with a random mask."""
    from diver_gb300.ray_voxel_intersection import masked_segments

    g = torch.Generator().manual_seed(seed)
    o = (torch.rand(rays, 3, generator=g) * 2 - 1) * 2.0
    d = torch.nn.functional.normalize(-o + (torch.rand(rays, 3, generator=g) - 0.5), dim=1)
    mask = (torch.rand(n_vox, n_vox, n_vox, generator=g) < 0.5).cuda()
    segs = masked_segments(o.cuda(), d.cuda(), -1.0, n_vox, 2.0 / n_vox, mask, 1.0)
    return segs


@pytest.mark.parametrize("channels,shape", [(32, (33, 33, 33)), (64, (17, 17, 17)), (12, (33, 33, 33))])
def test_clear_zeroes_exactly_the_written_rows(channels, shape):
    nz, ny, nx = shape
    segs = walk_segments(nx - 1, 300, channels)
    S = segs.total
    assert S > 100
    grid = torch.randn(nz, ny, nx, channels, device="cuda") + 5.0  # no zero entries
    before = grid.clone()
    touched = torch.zeros(nz * ny * nx, dtype=torch.uint8, device="cuda")
    st = N.stream(grid.device)
    N.call("dv_mark_corner_rows", N.ptr(segs.seg), S, None, nx, ny, nz, N.ptr(touched), st)
    N.call("dv_clear_marked_rows", N.ptr(grid), channels, nx, ny, nz, N.ptr(touched), st)
    torch.cuda.synchronize()
    expect = torch.zeros(nz * ny * nx, dtype=torch.bool)
    expect[corner_rows(segs.seg[:S], nx, ny, nz).reshape(-1)] = True
    flat, ref = grid.reshape(-1, channels).cpu(), before.reshape(-1, channels).cpu()
    zero = (flat == 0).all(1)
    assert torch.equal(zero, expect)
    assert torch.equal(flat[~expect], ref[~expect])
    assert int(touched.sum().item()) == 0


def test_clear_of_long_lines():
    """Lines of 800 rows (25 chunks of 32 rows; the x - 1 neighbour's mark
    carried from chunk to chunk); random segments."""
    nz, ny, nx, channels = 4, 5, 800, 32
    g = torch.Generator().manual_seed(3)
    p0 = torch.rand(500, 3, generator=g) * torch.tensor([nx - 1.0, ny - 1.0, nz - 1.0])
    p1 = (p0 + torch.rand(500, 3, generator=g) * 0.9).clamp_max(torch.tensor([nx - 1.0, ny - 1.0, nz - 1.0]))
    seg = torch.cat([p0, p1], 1).float().cuda().contiguous()
    grid = torch.randn(nz, ny, nx, channels, device="cuda") + 5.0
    before = grid.clone()
    touched = torch.zeros(nz * ny * nx, dtype=torch.uint8, device="cuda")
    st = N.stream(grid.device)
    N.call("dv_mark_corner_rows", N.ptr(seg), seg.shape[0], None, nx, ny, nz, N.ptr(touched), st)
    N.call("dv_clear_marked_rows", N.ptr(grid), channels, nx, ny, nz, N.ptr(touched), st)
    torch.cuda.synchronize()
    expect = torch.zeros(nz * ny * nx, dtype=torch.bool)
    expect[corner_rows(seg, nx, ny, nz).reshape(-1)] = True
    flat, ref = grid.reshape(-1, channels).cpu(), before.reshape(-1, channels).cpu()
    assert torch.equal((flat == 0).all(1), expect)
    assert torch.equal(flat[~expect], ref[~expect])
    assert int(touched.sum().item()) == 0


def test_mark_stops_at_the_device_count():
    nz = ny = nx = 33
    segs = walk_segments(32, 200, 7)
    S = segs.total
    half = S // 2
    count = torch.tensor([half], dtype=torch.int64, device="cuda")
    grid = torch.ones(nz, ny, nx, 32, device="cuda")
    touched = torch.zeros(nz * ny * nx, dtype=torch.uint8, device="cuda")
    st = N.stream(grid.device)
    N.call("dv_mark_corner_rows", N.ptr(segs.seg), S, N.ptr(count), nx, ny, nz, N.ptr(touched), st)
    N.call("dv_clear_marked_rows", N.ptr(grid), 32, nx, ny, nz, N.ptr(touched), st)
    torch.cuda.synchronize()
    expect = torch.zeros(nz * ny * nx, dtype=torch.bool)
    expect[corner_rows(segs.seg[:half], nx, ny, nz).reshape(-1)] = True
    assert torch.equal((grid.reshape(-1, 32).cpu() == 0).all(1), expect)


def test_sparse_and_dense_clearing_steps_agree():
    from diver_gb300 import scenes
    from diver_gb300.graphs import TrainStepGraph
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    sc.decoder.layers[sc.decoder.n_mlp1 - 1][1][0] += 0.6  # density above zero
    field = DIVeRField.from_scene(sc, "cuda")
    batches = []
    for k in range(4):
        o, d = scenes.small_view("cuda", seed_offset=k)
        pick = torch.randperm(o.shape[0], generator=torch.Generator().manual_seed(k))[:2048].cuda()
        tgt = torch.rand(2048, 3, generator=torch.Generator().manual_seed(10 + k)).cuda()
        batches.append((o[pick].contiguous(), d[pick].contiguous(), tgt))
    sparse = TrainStepGraph(field, *batches[0], form="bf16")
    dense = TrainStepGraph(field, *batches[0], form="bf16", sparse_clear=False)
    for o, d, tgt in batches[1:] + batches[:1]:
        ls, gvs, gps = (t.clone() for t in sparse(o, d, tgt))
        ld, gvd, gpd = (t.clone() for t in dense(o, d, tgt))
        torch.cuda.synchronize()
        assert abs(ls.item() - ld.item()) <= 1e-6 * abs(ld.item())
        scale = gvd.abs().max().item()
        assert (gvs - gvd).abs().max().item() <= 1e-5 * scale
        assert (gps - gpd).abs().max().item() <= 1e-5 * gpd.abs().max().item()
        # rows this batch does not write are exactly zero in both
        untouched = (gvd == 0).all(-1)
        assert int((gvs[untouched] != 0).sum().item()) == 0


def test_caller_writes_to_the_returned_gradient_outside_the_written_rows_persist():
    """The contract of the sparse-clearing captured step: its grid gradient
    is the graph's own buffer and only the rows a replay writes are cleared
    before the next one, so a caller that changes other rows of it (instead
    of cloning first) sees the change in every later step."""
    from diver_gb300 import scenes
    from diver_gb300.graphs import TrainStepGraph
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    field = DIVeRField.from_scene(sc, "cuda")
    o, d = scenes.small_view("cuda")
    pick = torch.arange(0, o.shape[0], 37, device="cuda")[:1024]
    tgt = torch.rand(pick.numel(), 3, generator=torch.Generator().manual_seed(2)).cuda()
    step = TrainStepGraph(field, o[pick].contiguous(), d[pick].contiguous(), tgt, form="bf16s")
    _, gv, _ = step(o[pick], d[pick], tgt)
    torch.cuda.synchronize()
    untouched = torch.nonzero((gv == 0).all(-1).reshape(-1))[:, 0]
    assert untouched.numel() > 0
    row = int(untouched[0])
    gv.view(-1, gv.shape[-1])[row] = 1.0  # a caller write to a row the step does not write
    _, gv2, _ = step(o[pick], d[pick], tgt)
    torch.cuda.synchronize()
    assert gv2.data_ptr() == gv.data_ptr()
    assert bool((gv2.view(-1, gv2.shape[-1])[row] == 1.0).all())
