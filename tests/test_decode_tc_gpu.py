"""GPU: the tcgen05 decoder (BF16 / FP16 operands, FP32 accumulation) against
the plain FP32 decoder and the FP64 oracle.

Tolerances (stated): per-segment sigma and rgb vs FP32 within 3e-2 (BF16) /
4e-3 (FP16) abs; rendered rgb and alpha vs the FP64 oracle within 1e-3 (BF16)
/ 2e-4 (FP16) / 1e-5 (FP32) max abs."""
import numpy as np
import pytest
import torch

from oracle import native as orc
from oracle import torch_ref

pytestmark = pytest.mark.gpu
TOL_SEG = {"bf16": 3e-2, "fp16": 4e-3}
TOL_RGB = {"bf16": 1e-3, "fp16": 2e-4}


def small():
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cpu")
    return sc, o, v, DIVeRField.from_scene(sc, "cuda")


def test_kmajor_layout_is_a_permutation():
    from diver_gb300.decoder import _kmajor_index

    for N, K in ((16, 32), (48, 32), (80, 64), (64, 64)):
        idx = _kmajor_index(N, K)
        assert torch.equal(idx.sort().values, torch.arange(N * K))


@pytest.mark.parametrize("kind,channels", [("diver32", 32), ("diver64", 32), ("diver64", 64)])
@pytest.mark.parametrize("form", ["bf16", "fp16"])
def test_tc_segments_match_fp32(kind, channels, form):
    from diver_gb300 import masked_segments, scenes
    from diver_gb300.decoder import pack_plain, random_decoder
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    feats = scenes.features(65, channels, 0.05, 0, "cpu")
    dec = random_decoder(kind, channels, 2)
    dec.layers[dec.n_mlp1 - 1][1][0] += 0.6  # active density
    field = DIVeRField(feats.cuda(), dec, sc.mask.cuda(), sc.xyzmin, sc.voxel_size)
    o, v = scenes.small_view("cuda")
    seg = field.segments(o, v)
    from diver_gb300 import _native as N
    from diver_gb300.renderer import KIND_ID

    k = KIND_ID[kind]
    W = 32 if kind == "diver32" else 64
    pe_feat = torch.empty(o.shape[0], 28, device="cuda")
    pe_out = torch.empty(o.shape[0], W, device="cuda")
    st = N.stream()
    N.call("dv_ray_pe", k, channels, N.ptr(field.params), o.shape[0], N.ptr(v), N.ptr(pe_feat), N.ptr(pe_out), st)
    ref = torch.empty(seg.total, 4, device="cuda")
    N.call("dv_decode_fwd", k, channels, N.ptr(field.params), N.ptr(field.voxels), 65, 65, 65, N.ptr(seg.seg),
           N.ptr(seg.ray), seg.total, None, N.ptr(pe_out), N.ptr(ref), st)
    tcw = field.tc_weights(form)
    scale = ref.abs().max(0).values.cpu().numpy()
    # FP32 grid rows, then the 16-bit copy of the grid used for rendering
    for g16 in (None, field.grid16(form)):
        got = torch.empty_like(ref)
        tcw.decode(k, channels, field.voxels, seg, pe_out, got, st, g16)
        torch.cuda.synchronize()
        assert int(tcw.err.item()) == 0
        err = (got - ref).abs().max(0).values.cpu().numpy()
        assert err[0] <= TOL_SEG[form] * max(1.0, scale[0]), (err, scale, g16 is None)
        assert err[1:].max() <= TOL_SEG[form], (err, scale, g16 is None)


@pytest.mark.parametrize("form", ["bf16", "fp16"])
def test_tc_render_error_vs_fp64_oracle(form):
    sc, o, v, field = small()
    with torch.no_grad():
        rgb, _ = field(o.cuda(), v.cuda(), form=form)
    inter, num, _ = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, 64, sc.voxel_size, sc.mask.numpy(), 1.0)
    segs = torch.from_numpy(orc.csr_from_padded(inter, num)).double()
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    L = [(w.double(), b.double()) for w, b in sc.decoder.layers]
    ref, _, _ = torch_ref.forward(sc.features.double(), L, 3, segs, ray, torch.from_numpy(num), v.double())
    err = np.abs(rgb.cpu().numpy() - ref.numpy()).max()
    assert err <= TOL_RGB[form], err


# Stated tolerances for the tensor-core training forms: gradients within these
# relative L2 errors of the FP32 backward, per tensor.  BF16: tcgen05 forward
# and backward (FP32 accumulation); FP16: tcgen05 forward, FP32 backward.
TOL_GRAD = {"bf16": 3e-2, "fp16": 5e-3}


@pytest.mark.parametrize("form", ["bf16", "fp16"])
def test_tc_backward_matches_fp32_backward(form, golden):
    from diver_gb300 import masked_segments
    from diver_gb300.decoder import pack_plain
    from diver_gb300.renderer import TcWeights, render_segments
    from tests.test_decode_gpu import decoder_from_golden

    g = golden("decode_ref.npz")
    dec = decoder_from_golden(g, "diver32")
    o = torch.from_numpy(g["o_hit"]).cuda()
    d = torch.from_numpy(g["d_hit"]).cuda()
    seg = masked_segments(o, d, -1.5, 12, 0.25, torch.from_numpy(g["mask"]).cuda(), 1.0)
    tgt = torch.from_numpy(g["target"]).cuda()
    grads = {}
    for f in ("fp32", form):
        vox = torch.from_numpy(g["voxels"]).cuda().requires_grad_(True)
        params = pack_plain(dec).cuda().requires_grad_(True)
        tc = None if f == "fp32" else TcWeights.from_decoder(dec, "cuda", bf16=(f == "bf16"))
        rgb, reg = render_segments(vox, params, seg, d, "diver32", True, tc)
        (torch.nn.functional.mse_loss(rgb, tgt) + 1e-5 * reg).backward()
        torch.cuda.synchronize()
        if tc is not None:
            assert int(tc.err.item()) == 0
        grads[f] = (vox.grad.clone(), params.grad.clone())
    for a, b in zip(grads[form], grads["fp32"]):
        rel = ((a - b).norm() / b.norm()).item()
        assert rel <= TOL_GRAD[form], rel


def test_tc_backward_on_the_small_scene_runs_full_tiles():
    """Many tiles (64^3 scene, 200x200 view): tensor-core grads vs FP32 grads."""
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cuda")
    tgt = torch.rand(o.shape[0], 3, generator=torch.Generator().manual_seed(1)).cuda()
    out = {}
    for form in ("fp32", "bf16"):
        field = DIVeRField.from_scene(sc, "cuda")
        rgb, reg = field(o, v, form=form)
        (torch.nn.functional.mse_loss(rgb, tgt) + 1e-5 * reg).backward()
        out[form] = (field.voxels.grad.clone(), field.params.grad.clone())
    for a, b in zip(out["bf16"], out["fp32"]):
        assert ((a - b).norm() / b.norm()).item() <= TOL_GRAD["bf16"]


def test_tc_backward_from_saved_layers_matches_recompute():
    """The forward's saved layer inputs reproduce the recomputed forward: the
    two backward modes agree to FP32 atomic-accumulation order (1e-6 of the
    largest gradient magnitude)."""
    from diver_gb300 import _native as N
    from diver_gb300.renderer import KIND_ID

    sc, o, v, field = small()
    sc.decoder.layers[sc.decoder.n_mlp1 - 1][1][0] += 0.6
    from diver_gb300.renderer import DIVeRField

    field = DIVeRField.from_scene(sc, "cuda")
    o, v = o.cuda(), v.cuda()
    seg = field.segments(o, v)
    k, C, B, S = KIND_ID["diver32"], 32, o.shape[0], seg.total
    st = N.stream()
    tw = field.tc_weights("bf16")
    pe_feat = torch.empty(B, 28, device="cuda")
    pe_out = torch.empty(B, 32, device="cuda")
    N.call("dv_ray_pe", k, C, N.ptr(field.params), B, N.ptr(v), N.ptr(pe_feat), N.ptr(pe_out), st)
    out4 = torch.empty(S, 4, device="cuda")
    save = tw.save_buffer(k, C, S, "cuda")
    tw.decode(k, C, field.voxels, seg, pe_out, out4, st, None, save)
    out4_ref = torch.empty_like(out4)
    tw.decode(k, C, field.voxels, seg, pe_out, out4_ref, st)
    assert torch.equal(out4, out4_ref)
    rgb = torch.empty(B, 3, device="cuda")
    N.call("dv_composite_fwd", B, N.ptr(seg.offsets), N.ptr(out4), 1, N.ptr(rgb), None, None, st)
    g_rgb = (torch.rand(B, 3, generator=torch.Generator().manual_seed(3)) - 0.5).cuda()
    d4 = torch.empty_like(out4)
    N.call("dv_composite_bwd", B, N.ptr(seg.offsets), N.ptr(out4), N.ptr(rgb), N.ptr(g_rgb), 1e-5 / B, None,
           N.ptr(d4), st)
    grads = []
    for sv in (save, None):
        gv = torch.zeros_like(field.voxels)
        gp = torch.zeros_like(field.params)
        assert tw.backward(k, field.voxels, seg, pe_feat, pe_out, d4, gv, gp, st, sv, out4)
        torch.cuda.synchronize()
        assert int(tw.err.item()) == 0
        grads.append((gv, gp))
    for a, b in zip(*grads):
        assert (a - b).abs().max().item() <= 1e-6 * a.abs().max().item()


def _oracle_rgb_alpha(sc, o, v, xyzmin, n, vs):
    inter, num, _ = orc.masked_walk(o.cpu().numpy(), v.cpu().numpy(), xyzmin, n, vs, sc.mask.cpu().numpy(), 1.0)
    segs = torch.from_numpy(orc.csr_from_padded(inter, num)).double()
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    L = [(w.double().cpu(), b.double().cpu()) for w, b in sc.decoder.layers]
    rgb, sigma, mask = torch_ref.forward(sc.features.cpu(), L, sc.decoder.n_mlp1, segs, ray,
                                         torch.from_numpy(num), v.double().cpu(), dtype=torch.float64)
    color = torch.zeros(sigma.shape + (3,), dtype=torch.float64)
    _, weight = torch_ref.render(color, sigma, mask, False)
    return rgb.numpy(), weight.sum(1).numpy()


# Error of each decoder form against the FP64 oracle, per scene (stated bounds):
# max-abs rgb, PSNR of the rendering against the FP64 rendering, max-abs alpha
# (accumulated opacity 1 - T).
ERR_BOUNDS = {"fp32": 1e-5, "bf16": 1e-3, "fp16": 2e-4}


@pytest.mark.parametrize("scene", ["small", "grid256", "grid256x64"])
def test_render_error_metrics_vs_fp64(scene):
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    if scene == "small":
        sc = scenes.small_scene("cpu")
        o, v = scenes.small_view("cpu")
    else:
        # grid256: the differentiation scene (DIVeR32, 32 channels); grid256x64: the precision
        # scene (64-channel features, DIVeR64) on a spiral camera
        wide = scene == "grid256x64"
        sc = scenes.grid_scene(256, 64, "diver64", device="cpu") if wide else scenes.grid_scene(256, 32, "diver32",
                                                                                                device="cpu")
        cam = scenes.spiral_cameras(200, 4.0)[37] if wide else scenes.sphere_cameras(100, 4.0, 3)[0]
        o, v = scenes.camera_rays(cam, 800, 800, 960.0, "cpu")
        n = 1024 if wide else 2048
        pick = torch.arange(0, o.shape[0], 313)[:n]  # a fixed spread-out subset of the frame
        o, v = o[pick].contiguous(), v[pick].contiguous()
    sc.decoder.layers[sc.decoder.n_mlp1 - 1][1][0] += 0.6  # density above zero: a visible, semi-opaque scene
    ref_rgb, ref_alpha = _oracle_rgb_alpha(sc, o, v, sc.xyzmin, sc.voxel_num, sc.voxel_size)
    field = DIVeRField.from_scene(sc, "cuda")
    oc, vc = o.cuda(), v.cuda()
    for form in ("fp32", "bf16", "fp16"):
        with torch.no_grad():
            field.white_back = True
            rgb_w, _ = field(oc, vc, form=form)
            field.white_back = False
            rgb_b, _ = field(oc, vc, form=form)
        rgb = rgb_w.cpu().double().numpy()
        alpha = 1.0 - (rgb_w - rgb_b).cpu().double().numpy()[:, 0]
        e_rgb = float(np.abs(rgb - ref_rgb).max())
        mse = float(((rgb - ref_rgb) ** 2).mean())
        psnr = float("inf") if mse == 0 else -10.0 * np.log10(mse)
        e_alpha = float(np.abs(alpha - ref_alpha).max())
        print(f"ERRMETRIC scene={scene} form={form} max_abs_rgb={e_rgb:.3e} psnr_vs_fp64={psnr:.1f}dB "
              f"max_abs_alpha={e_alpha:.3e} mean_alpha={ref_alpha.mean():.3f}")
        assert e_rgb <= ERR_BOUNDS[form], (form, e_rgb)
        assert e_alpha <= ERR_BOUNDS[form], (form, e_alpha)


def test_inference_render_keeps_no_layer_tiles(monkeypatch):
    """Without autograd the tensor-core forward must not keep its layer tiles
    (for a 800x800 frame that buffer would be ~36 GB of writes)."""
    from diver_gb300 import renderer

    sc, o, v, field = small()

    def refuse(*args, **kwargs):
        raise AssertionError("layer-tile buffer requested by an inference render")

    monkeypatch.setattr(renderer.TcWeights, "save_buffer", refuse)
    with torch.no_grad():
        rgb, _ = field(o.cuda(), v.cuda(), form="bf16")
    torch.cuda.synchronize()
    assert torch.isfinite(rgb).all()


def test_bounded_wait_reports_a_timeout_and_completes_after_arrival():
    """Failure detection without a fault: a completion wait that nothing
    satisfies gives up after its poll limit and says so; the context stays
    usable (the next call on it works)."""
    from diver_gb300 import _native as N

    status = torch.full((2,), -1, dtype=torch.int32, device="cuda")
    N.call("dv_wait_selftest", 1000, N.ptr(status), N.stream())
    torch.cuda.synchronize()
    assert status.tolist() == [1, 0]
    assert torch.ones(4, device="cuda").sum().item() == 4.0
