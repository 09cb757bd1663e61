"""Grids with per-axis extents (the reference is cubic only): the per-axis walk
equals the cubic walk on cubic grids, matches the oracle's restatement on a
wide grid bit-exactly, and the wide-scene render matches the FP64 oracle."""
import numpy as np
import pytest
import torch

from oracle import native as orc
from oracle import torch_ref
from tests.test_traverse_oracle import same_bits

pytestmark = pytest.mark.gpu


def test_per_axis_walk_equals_cubic_walk_on_cubic_grid():
    from diver_gb300 import masked_segments, scenes
    from diver_gb300.ray_voxel_intersection import masked_segments_grid

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cuda")
    mk = sc.mask.cuda()
    a = masked_segments(o, v, sc.xyzmin, 64, sc.voxel_size, mk, 1.0)
    b = masked_segments_grid(o, v, (sc.xyzmin,) * 3, (64, 64, 64), sc.voxel_size, mk)
    assert torch.equal(a.seg, b.seg) and torch.equal(a.t, b.t) and torch.equal(a.offsets, b.offsets)


def wide_small():
    from diver_gb300 import scenes

    sc = scenes.wide_scene("cpu", dims=(80, 80, 40))
    sc.voxel_size = 1.0 / 40  # same world box, coarser grid
    cams = scenes.ellipse_cameras(6)
    o, v = scenes.camera_rays(cams[1], 96, 128, 150.0, "cpu")
    return sc, o, v


def test_per_axis_walk_matches_oracle_on_wide_grid():
    from diver_gb300.ray_voxel_intersection import masked_segments_grid

    sc, o, v = wide_small()
    seg = masked_segments_grid(o.cuda(), v.cuda(), sc.xyzmin, sc.dims, sc.voxel_size, sc.mask.cuda())
    inter, num, tns = orc.masked_walk_grid(o.numpy(), v.numpy(), sc.xyzmin, sc.dims, sc.voxel_size, sc.mask.numpy())
    assert np.array_equal(seg.counts.cpu().numpy(), num) and num.sum() > 1000
    assert same_bits(seg.seg.cpu().numpy(), orc.csr_from_padded(inter, num))
    assert same_bits(seg.t.cpu().numpy(), orc.csr_from_padded(tns[..., None], num)[:, 0])


@pytest.mark.parametrize("form,tol", [("fp32", 1e-5), ("fp16", 1e-3), ("bf16", 1e-2)])
def test_wide_scene_render_matches_fp64_oracle(form, tol):
    from diver_gb300.renderer import DIVeRField

    sc, o, v = wide_small()
    field = DIVeRField(sc.features.cuda(), sc.decoder, sc.mask.cuda(), sc.xyzmin, sc.voxel_size)
    with torch.no_grad():
        rgb, _ = field(o.cuda(), v.cuda(), form=form)
    inter, num, _ = orc.masked_walk_grid(o.numpy(), v.numpy(), sc.xyzmin, sc.dims, sc.voxel_size, sc.mask.numpy())
    segs = torch.from_numpy(orc.csr_from_padded(inter, num)).double()
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    L = [(w.double(), b.double()) for w, b in sc.decoder.layers]
    ref, _, _ = torch_ref.forward(sc.features.double(), L, 3, segs, ray, torch.from_numpy(num), v.double(),
                                  per_axis=True)
    assert np.abs(rgb.cpu().numpy() - ref.numpy()).max() <= tol
