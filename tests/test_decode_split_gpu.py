"""GPU: the split-operand tensor-core decoder (form 'bf16s': FP32 values as
BF16 terms, FP32 accumulation) against the plain FP32 decoder, the reference's
own outputs and gradients (tests/golden/decode_ref.npz), FP64 central finite
differences and the FP64 oracle.

Tolerances (the FP32 form's): rgb 1e-5 abs, loss 1e-6; gradients within 1e-4
relative of the reference autograd and of FP64 central differences (both in
L2 over the sampled entries and per entry above 1 % of the largest); decoder
outputs per segment within 1e-5 of the plain FP32 kernel."""
import numpy as np
import pytest
import torch

from tests.test_decode_gpu import (check_forward_and_loss, check_gradients_vs_central_differences,
                                   check_gradients_vs_reference_autograd)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g(golden):
    return golden("decode_ref.npz")


@pytest.mark.parametrize("kind,channels", [("diver32", 32), ("diver64", 32), ("diver64", 64)])
def test_split_segments_match_fp32(kind, channels):
    from diver_gb300 import _native as N
    from diver_gb300 import scenes
    from diver_gb300.decoder import random_decoder
    from diver_gb300.renderer import KIND_ID, DIVeRField

    sc = scenes.small_scene("cpu")
    feats = scenes.features(65, channels, 0.05, 0, "cpu")
    dec = random_decoder(kind, channels, 2)
    dec.layers[dec.n_mlp1 - 1][1][0] += 0.6  # active density
    field = DIVeRField(feats.cuda(), dec, sc.mask.cuda(), sc.xyzmin, sc.voxel_size)
    o, v = scenes.small_view("cuda")
    seg = field.segments(o, v)
    k = KIND_ID[kind]
    W = 32 if kind == "diver32" else 64
    pe_feat = torch.empty(o.shape[0], 28, device="cuda")
    pe_out = torch.empty(o.shape[0], W, device="cuda")
    st = N.stream()
    N.call("dv_ray_pe", k, channels, N.ptr(field.params), o.shape[0], N.ptr(v), N.ptr(pe_feat), N.ptr(pe_out), st)
    ref = torch.empty(seg.total, 4, device="cuda")
    N.call("dv_decode_fwd", k, channels, N.ptr(field.params), N.ptr(field.voxels), 65, 65, 65, N.ptr(seg.seg),
           N.ptr(seg.ray), seg.total, None, N.ptr(pe_out), N.ptr(ref), st)
    tcw = field.tc_weights("bf16s")
    got = torch.empty_like(ref)
    tcw.decode(k, channels, field.voxels, seg, pe_out, got, st)
    # with a save buffer (training) the output is the same, bit for bit
    save = tcw.save_buffer(k, channels, seg.total, "cuda")
    got2 = torch.empty_like(ref)
    tcw.decode(k, channels, field.voxels, seg, pe_out, got2, st, None, save)
    torch.cuda.synchronize()
    assert int(tcw.err.item()) == 0
    err = (got - ref).abs().max(0).values.cpu().numpy()
    scale = ref.abs().max(0).values.cpu().numpy()
    assert err[0] <= 1e-5 * max(1.0, scale[0]), (err, scale)
    assert err[1:].max() <= 1e-5, (err, scale)
    assert torch.equal(got, got2)


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_split_forward_and_loss_match_reference(g, kind):
    check_forward_and_loss(g, kind, "bf16s")


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_split_gradients_match_reference_autograd(g, kind):
    check_gradients_vs_reference_autograd(g, kind, "bf16s")


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_split_gradients_match_fp64_central_differences(g, kind):
    rel = check_gradients_vs_central_differences(g, kind, "bf16s")
    print(f"SPLITFD kind={kind} rel_l2_vs_central_differences={rel:.2e}")


def test_split_training_on_the_small_scene_matches_fp64():
    """Many tiles (64^3 scene, 200x200 view, semi-opaque): the split form's
    grid and decoder gradients against an FP64 autograd backward of the
    oracle, and against the plain FP32 CUDA backward (relative L2)."""
    from diver_gb300 import scenes
    from diver_gb300.decoder import unpack_plain_grad
    from diver_gb300.renderer import DIVeRField
    from oracle import native as orc
    from oracle import torch_ref

    sc = scenes.small_scene("cpu")
    sc.decoder.layers[sc.decoder.n_mlp1 - 1][1][0] += 0.6
    o, v = scenes.small_view("cpu")
    tgt = torch.rand(o.shape[0], 3, generator=torch.Generator().manual_seed(1))
    out = {}
    for form in ("fp32", "bf16s"):
        field = DIVeRField.from_scene(sc, "cuda")
        rgb, reg = field(o.cuda(), v.cuda(), form=form)
        (torch.nn.functional.mse_loss(rgb, tgt.cuda()) + 1e-5 * reg).backward()
        torch.cuda.synchronize()
        out[form] = (field.voxels.grad.cpu().double(), field.params.grad.cpu().double())
    inter, num, _ = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, sc.voxel_num, sc.voxel_size, sc.mask.numpy(), 1.0)
    segs = torch.from_numpy(orc.csr_from_padded(inter, num)).double()
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    vox = sc.features.double().requires_grad_(True)
    layers = [(w.double().requires_grad_(True), b.double().requires_grad_(True)) for w, b in sc.decoder.layers]
    rgb, sigma, _ = torch_ref.forward(vox, layers, sc.decoder.n_mlp1, segs, ray, torch.from_numpy(num), v.double())
    (torch.nn.functional.mse_loss(rgb, tgt.double()) + 1e-5 * torch.log(1 + sigma ** 2 / 0.5).mean()).backward()
    ref_w = torch.cat([torch.cat([w.grad.reshape(-1), b.grad]) for w, b in layers])
    for form in ("fp32", "bf16s"):
        gv, gp = out[form]
        got_w = torch.cat([torch.cat([dw.reshape(-1), db]) for dw, db in
                           unpack_plain_grad(sc.decoder.kind, 32, gp.float())]).double()
        e_grid = ((gv - vox.grad).norm() / vox.grad.norm()).item()
        e_w = ((got_w - ref_w).norm() / ref_w.norm()).item()
        print(f"SPLITERR form={form} grid_rel_l2={e_grid:.2e} decoder_rel_l2={e_w:.2e}")
        assert e_grid <= 1e-5 and e_w <= 1e-5, (form, e_grid, e_w)
    for a, b in zip(out["bf16s"], out["fp32"]):
        assert ((a - b).norm() / b.norm()).item() <= 1e-5


def test_split_render_error_vs_fp64_oracle():
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField
    from oracle import native as orc
    from oracle import torch_ref

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cpu")
    field = DIVeRField.from_scene(sc, "cuda")
    with torch.no_grad():
        rgb, _ = field(o.cuda(), v.cuda(), form="bf16s")
    inter, num, _ = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, 64, sc.voxel_size, sc.mask.numpy(), 1.0)
    segs = torch.from_numpy(orc.csr_from_padded(inter, num)).double()
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    L = [(w.double(), b.double()) for w, b in sc.decoder.layers]
    ref, _, _ = torch_ref.forward(sc.features.double(), L, 3, segs, ray, torch.from_numpy(num), v.double())
    assert np.abs(rgb.cpu().numpy() - ref.numpy()).max() < 1e-5


def split_terms(x: torch.Tensor, n: int) -> list[torch.Tensor]:
    """FP32 values as n BF16 terms, each rounding what the previous ones left."""
    out, r = [], x.float()
    for _ in range(n):
        t = r.to(torch.bfloat16)
        out.append(t)
        r = r - t.float()
    return out


def test_weight_image_gather_matches_torch_conversions():
    """dv_tc_image (the one-launch weight refresh) against torch's own
    conversions, bit for bit: FP32, BF16, FP16 and the three-term split, with
    index 0 the zero entry and indices past the parameters reading 0."""
    from diver_gb300 import _native as N

    g = torch.Generator().manual_seed(3)
    params = (torch.randn(5000, generator=g) * torch.exp(torch.randn(5000, generator=g) * 4)).cuda()
    index = torch.randint(0, 5001, (70001,), generator=g)
    index[:7] = torch.tensor([0, 1, 5000, 5001, 9999, -3, 0])
    ext = torch.cat([params.new_zeros(1), params])
    ref = ext[index.clamp(0, 5000).cuda()]
    ref[(index > 5000) | (index < 0)] = 0
    index = index.cuda()
    n = index.numel()
    st = N.stream()
    for form, expect in ((0, [ref]), (1, [ref.to(torch.bfloat16)]), (2, [ref.half()]), (3, split_terms(ref, 3))):
        out = torch.full((len(expect) * n,), -1.0, dtype=expect[0].dtype, device="cuda")
        N.call("dv_tc_image", N.ptr(params), params.numel(), N.ptr(index), n, form, N.ptr(out), st)
        torch.cuda.synchronize()
        assert torch.equal(out.view(torch.int16 if out.element_size() == 2 else torch.int32),
                           torch.cat(expect).view(torch.int16 if out.element_size() == 2 else torch.int32)), form
    with pytest.raises(RuntimeError):
        N.call("dv_tc_image", N.ptr(params), params.numel(), N.ptr(index), n, 4, N.ptr(out), st)
