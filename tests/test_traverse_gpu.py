"""GPU: the sm_103a traversal kernels against the reference kernels' fixtures
and the C oracle (bit-exact), plus size-independent properties at full size."""
import numpy as np
import pytest
import torch

from oracle import native as orc
from tests.test_traverse_oracle import maxpool, octree_march_oracle, same_bits, unpack

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g(golden):
    return golden("traverse_ref.npz")


def cuda(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return t if dtype is None else t.to(dtype)


def csr(t, num):
    t = t.cpu().numpy()
    num = num.cpu().numpy()
    return np.concatenate([t[b, :num[b]] for b in range(len(num))], 0)


def test_dense_matches_reference_fixture(g):
    from diver_gb300 import ray_voxel_intersect

    n, x0, vs = int(g["walk_n"]), float(g["walk_xyzmin"]), float(g["walk_vs"])
    inter, hit, tns = ray_voxel_intersect(cuda(g["walk_o"]), cuda(g["walk_v"]), x0, -x0, n, vs)
    num = hit.sum(1).int()
    assert np.array_equal(num.cpu().numpy(), g["dense_num"])
    assert inter.shape[1] == int(g["dense_num"].max())
    assert same_bits(csr(inter, num), g["dense_pts"])
    assert same_bits(csr(tns[..., None], num)[:, 0], g["dense_tns"])
    assert same_bits(inter[:, 0].cpu().numpy(), g["dense_row0"])
    # padding is the reference's: zeros and -1
    pad = ~hit
    pad[:, 0] = False
    assert (inter[pad] == 0).all() and (tns[~hit] == -1).all()


@pytest.mark.parametrize("tag,scale", [("m1", 1.0), ("m05", 0.5), ("m025", 0.25)])
def test_masked_matches_reference_fixture(g, tag, scale):
    from diver_gb300 import masked_intersect, masked_segments

    n, x0, vs = int(g["walk_n"]), float(g["walk_xyzmin"]), float(g["walk_vs"])
    m = unpack(g["mask64"], n)
    if scale != 1.0:
        m = maxpool(m, int(round(1 / scale)))
    o, v, mt = cuda(g["walk_o"]), cuda(g["walk_v"]), cuda(m)
    inter, hit, tns = masked_intersect(o, v, x0, -x0, n, vs, mt, scale)
    num = hit.sum(1).int()
    assert np.array_equal(num.cpu().numpy(), g[f"masked_{tag}_num"])
    assert same_bits(csr(inter, num), g[f"masked_{tag}_seg"])
    assert same_bits(csr(tns[..., None], num)[:, 0], g[f"masked_{tag}_tns"])
    sg = masked_segments(o, v, x0, n, vs, mt, scale)
    assert same_bits(sg.seg.cpu().numpy(), g[f"masked_{tag}_seg"])
    assert same_bits(sg.t.cpu().numpy(), g[f"masked_{tag}_tns"])
    assert np.array_equal(sg.counts.cpu().numpy(), g[f"masked_{tag}_num"])


@pytest.mark.parametrize("N", [128, 256])
def test_octree_and_march_match_reference_fixture(g, N):
    from diver_gb300 import aabb_intersect, ray_march

    m = unpack(g[f"oct{N}_mask"], N)
    octs = np.concatenate([maxpool(m, s).reshape(-1) for s in (64, 16, 4)])
    v = cuda(g[f"oct{N}_v"])
    B = v.shape[0]
    coords = torch.zeros(8, B, 6, device="cuda")
    rgba = torch.zeros(B, 4, device="cuda")
    finish = torch.zeros(B, dtype=torch.bool, device="cuda")
    aabb_intersect(coords, v, cuda(g[f"oct{N}_center"]), finish, rgba, cuda(octs), N)
    ref_fin = g[f"oct{N}_finish"].astype(bool)
    assert np.array_equal(finish.cpu().numpy(), ref_fin)
    assert same_bits(coords[7, :, 3:].cpu().numpy()[~ref_fin], g[f"oct{N}_resume"][~ref_fin])
    assert same_bits(rgba.cpu().numpy(), g[f"oct{N}_rgba"])
    mt = cuda(m)
    hits = [[] for _ in range(B)]
    rounds = 0
    while not bool(finish.all()) and rounds < 4 * N:
        active = (~finish).cpu().numpy()
        ray_march(coords, v, mt, finish, N)
        c = coords.cpu().numpy()
        for b in np.nonzero(active)[0]:
            for h in range(8):
                if c[h, b, 0] < 0:
                    break
                hits[b].append(c[h, b])
        finish |= (coords[:, :, 0] < 0).any(0)
        rounds += 1
    num = np.array([len(h) for h in hits], np.int32)
    assert np.array_equal(num, g[f"oct{N}_hit_num"])
    assert same_bits(np.concatenate([np.asarray(h, np.float32).reshape(-1, 6) for h in hits]), g[f"oct{N}_hits"])
    assert rounds == int(g[f"oct{N}_rounds"])


def small_inputs():
    from diver_gb300 import scenes

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cpu")
    return sc, o, v


def test_masked_and_dense_match_oracle_on_small_view():
    """Every ray of the 200x200 view of the 64^3 scene, bit-exact against the oracle."""
    from diver_gb300 import masked_intersect, ray_voxel_intersect

    sc, o, v = small_inputs()
    n = sc.voxel_num
    inter, hit, tns = masked_intersect(o.cuda(), v.cuda(), sc.xyzmin, sc.xyzmax, n, sc.voxel_size, sc.mask.cuda(), 1.0)
    oi, on, ot = orc.trim(*orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, n, sc.voxel_size, sc.mask.numpy(), 1.0))
    assert same_bits(inter.cpu().numpy(), oi) and np.array_equal(hit.cpu().numpy(), on)
    assert same_bits(tns.cpu().numpy(), ot)
    inter, hit, tns = ray_voxel_intersect(o.cuda(), v.cuda(), sc.xyzmin, sc.xyzmax, n, sc.voxel_size)
    oi, on, ot = orc.trim(*orc.dense_walk(o.numpy(), v.numpy(), sc.xyzmin, n, sc.voxel_size))
    assert same_bits(inter.cpu().numpy(), oi) and np.array_equal(hit.cpu().numpy(), on)
    assert same_bits(tns.cpu().numpy(), ot)


def test_segments_equal_boolean_compaction_of_padded_outputs():
    """dense_segments / masked_segments == what DIVeR.extract_features builds
    from the padded outputs (model/diver.py:86-103)."""
    from diver_gb300 import dense_segments, masked_intersect, masked_segments, ray_voxel_intersect

    sc, o, v = small_inputs()
    o, v, mk = o.cuda(), v.cuda(), sc.mask.cuda()
    n = sc.voxel_num
    coord, mask, ts = masked_intersect(o, v, sc.xyzmin, sc.xyzmax, n, sc.voxel_size, mk, 1.0)
    sg = masked_segments(o, v, sc.xyzmin, n, sc.voxel_size, mk, 1.0)
    assert torch.equal(sg.seg, coord[mask]) and torch.equal(sg.t, ts[mask])
    assert torch.equal(sg.ray.long(), torch.nonzero(mask)[:, 0])
    coord, mask, ts = ray_voxel_intersect(o, v, sc.xyzmin, sc.xyzmax, n, sc.voxel_size)
    ts = ts[:, :-1]
    coord = coord.clamp_min(0)
    pm = mask[:, :-1] & mask[:, 1:]
    sd = dense_segments(o, v, sc.xyzmin, n, sc.voxel_size)
    assert torch.equal(sd.coord_in, coord[:, :-1][pm]) and torch.equal(sd.coord_out, coord[:, 1:][pm])
    assert torch.equal(sd.t, ts[pm])


def test_full_size_masked_is_occupancy_filter_of_dense():
    """256^3 blob scene, 200x200 view: the masked walk's segments are exactly the
    dense walk's consecutive pairs whose voxel is occupied (a size-independent
    identity), and a 2048-ray sample is bit-exact against the oracle."""
    from diver_gb300 import dense_segments, masked_segments, scenes

    sc = scenes.grid_scene(256, 32, device="cuda")
    c2w = scenes.sphere_cameras(1, 4.0, 3)[0]
    o, v = scenes.camera_rays(c2w, 200, 200, 240.0, "cuda")
    n = sc.voxel_num
    sd = dense_segments(o, v, sc.xyzmin, n, sc.voxel_size)
    sm = masked_segments(o, v, sc.xyzmin, n, sc.voxel_size, sc.mask, 1.0)
    cell = torch.minimum(sd.coord_in + 1e-4, sd.coord_out + 1e-4).long()
    lin = (cell[:, 2] * n + cell[:, 1]) * n + cell[:, 0]  # the kernels' linear cell index
    inb = lin < n ** 3
    occ = torch.zeros_like(inb)
    occ[inb] = sc.mask.reshape(-1)[lin[inb]]
    assert torch.equal(sd.seg[occ], sm.seg)
    assert torch.equal(sd.ray[occ], sm.ray)
    # offsets are a proper CSR
    assert int(sm.offsets[0]) == 0 and bool((sm.offsets[1:] >= sm.offsets[:-1]).all())
    idx = torch.randperm(o.shape[0], generator=torch.Generator().manual_seed(7))[:2048]
    oi, on, ot = orc.trim(*orc.masked_walk(o[idx].cpu().numpy(), v[idx].cpu().numpy(), sc.xyzmin, n, sc.voxel_size,
                                           sc.mask.cpu().numpy(), 1.0))
    from diver_gb300 import masked_intersect

    inter, hit, tns = masked_intersect(o[idx].contiguous(), v[idx].contiguous(), sc.xyzmin, sc.xyzmax, n, sc.voxel_size,
                                       sc.mask, 1.0)
    assert same_bits(inter.cpu().numpy(), oi) and same_bits(tns.cpu().numpy(), ot)


def test_full_frame_walks_stay_within_their_step_bound():
    """800x800 frames of the 256^3 scene through every walk (dense, masked
    count + emission, captured slot walk, octree first hit + march rounds,
    the one-launch real-time frame): no walk reaches its step bound."""
    from diver_gb300 import _native as N
    from diver_gb300 import dense_segments, masked_segments, scenes
    from diver_gb300.realtime import RealtimeModel, convert
    from diver_gb300.renderer import DIVeRField

    N.lib().dv_walk_cap_hits(1)
    sc = scenes.grid_scene(256, 32, device="cuda")
    c2w = scenes.sphere_cameras(1, 4.0, 3)[0]
    o, v = scenes.camera_rays(c2w, 800, 800, 960.0, "cuda")
    dense_segments(o, v, sc.xyzmin, sc.voxel_num, sc.voxel_size)
    masked_segments(o, v, sc.xyzmin, sc.voxel_num, sc.voxel_size, sc.mask, 1.0)
    field = DIVeRField.from_scene(sc, "cuda")
    field.segments(o[:4096].contiguous(), v[:4096].contiguous(), capacity=field.segment_capacity(4096))
    sd = {"voxels": sc.features}
    sd.update(sc.decoder.state_dict())
    model = RealtimeModel.from_serialized(convert(sd, sc.mask.float()), 256, sc.xyzmin, sc.voxel_size, "cuda")
    model.render_frame(c2w[:, 3].cuda(), v, mode="fused")
    model.render_frame(c2w[:, 3].cuda(), v, mode="loop")
    torch.cuda.synchronize()
    assert N.lib().dv_walk_cap_hits(1) == 0


def test_empty_and_all_miss_batches():
    from diver_gb300 import masked_intersect, masked_segments, ray_voxel_intersect

    mk = torch.ones(8, 8, 8, dtype=torch.bool, device="cuda")
    e = torch.zeros(0, 3, device="cuda")
    inter, hit, tns = ray_voxel_intersect(e, e, -1.0, 1.0, 8, 0.25)
    assert inter.shape == (0, 0, 3)
    o = torch.tensor([[5.0, 5.0, 5.0]] * 4, device="cuda")
    v = torch.tensor([[1.0, 0.0, 0.0]] * 4, device="cuda")  # pointing away
    inter, hit, tns = masked_intersect(o, v, -1.0, 1.0, 8, 0.25, mk, 1.0)
    assert inter.shape == (4, 0, 6) and hit.shape == (4, 0)
    sg = masked_segments(o, v, -1.0, 8, 0.25, mk, 1.0)
    assert sg.total == 0 and int(sg.offsets[-1]) == 0


def test_scan_matches_cumsum():
    from diver_gb300.ray_voxel_intersection import exclusive_scan

    for n in (1, 7, 2048, 2049, 1 << 20, 3_000_001):
        c = torch.randint(0, 1000, (n,), dtype=torch.int32, device="cuda")
        off = exclusive_scan(c)
        ref = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
        ref[1:] = torch.cumsum(c.long(), 0)
        assert torch.equal(off, ref), n


def test_bad_arguments_raise():
    from diver_gb300 import masked_intersect

    o = torch.zeros(4, 3, device="cuda")
    with pytest.raises(ValueError):
        masked_intersect(o, o, -1.0, 1.0, 8, 0.25, torch.ones(4, 4, 4, dtype=torch.bool, device="cuda"), 1.0)
    with pytest.raises(ValueError):
        masked_intersect(o.cpu(), o.cpu(), -1.0, 1.0, 8, 0.25, torch.ones(8, 8, 8, dtype=torch.bool), 1.0)


@pytest.mark.gpu
def test_camera_rays_on_device_match_reference_math():
    """dv_camera_rays vs the reference's torch ray generation
    (utils/dataset/ray_utils.py:5-55, restated in scenes.camera_rays): within
    2e-7 abs (the matmul and norm reduce in a different order)."""
    from diver_gb300 import scenes

    c2w = scenes.sphere_cameras(3, 4.0, 3)[2]
    o_ref, d_ref = scenes.camera_rays(c2w, 120, 160, 192.0, "cpu")
    o, d = scenes.camera_rays_device(c2w, 120, 160, 192.0, "cuda")
    assert torch.equal(o.cpu(), o_ref)
    assert (d.cpu() - d_ref).abs().max().item() <= 2e-7
    o2, d2 = scenes.camera_rays_device(c2w, 120, 160, 192.0, "cuda", 5000, 3000)  # a pixel range
    assert torch.equal(d2, d[5000:8000]) and torch.equal(o2, o[5000:8000])


@pytest.mark.gpu
@pytest.mark.parametrize("n_rays", [3000, 40001, 60000])
def test_masked_segments_both_writers_bit_exact(n_rays):
    """Small batches write segments per lane, large ones stage them per warp
    (masked_emit_staged_kernel, also with a partly filled last warp): both
    give the oracle's CSR lists bit for bit."""
    from diver_gb300 import masked_segments, scenes

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cpu")
    g = torch.Generator().manual_seed(n_rays)
    pick = torch.randint(0, o.shape[0], (n_rays,), generator=g)
    jitter = (torch.rand(n_rays, 3, generator=g) - 0.5) * 0.2
    v = v[pick] + jitter
    v = (v / v.norm(dim=1, keepdim=True)).contiguous()
    o = o[pick].contiguous()
    seg = masked_segments(o.cuda(), v.cuda(), sc.xyzmin, sc.voxel_num, sc.voxel_size, sc.mask.cuda(), 1.0)
    inter, num, tns = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, sc.voxel_num, sc.voxel_size, sc.mask.numpy(),
                                      1.0)
    ref = orc.csr_from_padded(inter, num)
    ref_t = orc.csr_from_padded(tns[..., None], num)[:, 0]
    assert same_bits(seg.seg.cpu().numpy(), ref)
    assert same_bits(seg.t.cpu().numpy(), ref_t)
    assert np.array_equal(seg.ray.cpu().numpy(), np.repeat(np.arange(n_rays), num))
