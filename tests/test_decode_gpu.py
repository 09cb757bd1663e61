"""GPU: integrator, plain-FP32 decoder, compositing and the hand-written
backward against the reference's own outputs (tests/golden/decode_ref.npz),
the FP64 oracle and FP64 central finite differences.

Tolerances: forward features 1e-6 abs, rgb 1e-5 abs (FP32 plain form);
gradients 1e-4 relative to the reference autograd and to FP64 central
differences."""
import numpy as np
import pytest
import torch

from oracle import integrate as oint
from oracle import native as orc
from oracle import torch_ref

pytestmark = pytest.mark.gpu
KINDS = {"diver32": 3, "diver64": 2}


@pytest.fixture(scope="module")
def g(golden):
    return golden("decode_ref.npz")


def decoder_from_golden(g, kind):
    from diver_gb300.decoder import Decoder

    n1 = KINDS[kind]
    sd = {}
    for i in range(n1):
        sd[f"mlp1.{2 * i}.weight"] = torch.from_numpy(g[f"{kind}/mlp1.{2 * i}.weight"])
        sd[f"mlp1.{2 * i}.bias"] = torch.from_numpy(g[f"{kind}/mlp1.{2 * i}.bias"])
    for i in range(2):
        sd[f"mlp2.{2 * i}.weight"] = torch.from_numpy(g[f"{kind}/mlp2.{2 * i}.weight"])
        sd[f"mlp2.{2 * i}.bias"] = torch.from_numpy(g[f"{kind}/mlp2.{2 * i}.bias"])
    return Decoder.from_state_dict(kind, sd)


def test_integrate_matches_reference(g):
    from diver_gb300.integrator import integrate

    vox = torch.from_numpy(g["voxels"]).cuda()
    seg = torch.from_numpy(g["seg"]).cuda()
    f = integrate(vox, seg[:, :3], seg[:, 3:])  # strided halves of one [S,6] tensor
    assert np.abs(f.cpu().numpy() - g["feature"]).max() < 1e-6
    f64 = oint.integrate(g["voxels"], g["seg"][:, :3], g["seg"][:, 3:])
    assert np.abs(f.cpu().numpy() - f64).max() < 1e-6
    f2 = integrate(vox, seg[:, :3].contiguous(), seg[:, 3:].contiguous())
    assert torch.equal(f, f2)


def test_integrate_backward_matches_autograd(g):
    from diver_gb300.integrator import integrate

    vox = torch.from_numpy(g["voxels"]).cuda().requires_grad_(True)
    seg = torch.from_numpy(g["seg"]).cuda()
    up = torch.randn(seg.shape[0], vox.shape[-1], generator=torch.Generator().manual_seed(3)).cuda()
    (integrate(vox, seg[:, :3], seg[:, 3:]) * up).sum().backward()
    v64 = torch.from_numpy(g["voxels"]).double().requires_grad_(True)
    s64 = torch.from_numpy(g["seg"])
    (torch_ref.integrate(v64, s64[:, :3], s64[:, 3:]) * up.cpu().double()).sum().backward()
    ref = v64.grad.numpy()
    assert np.abs(vox.grad.cpu().numpy() - ref).max() < 1e-5 * max(1.0, np.abs(ref).max())


def run_field(g, kind, form="fp32"):
    """Forward + backward of the golden case through render_segments with the
    given decoder form ('fp32' plain kernels, or a tensor-core form)."""
    from diver_gb300 import masked_segments
    from diver_gb300.decoder import pack_plain
    from diver_gb300.renderer import TcWeights, render_segments

    dec = decoder_from_golden(g, kind)
    vox = torch.from_numpy(g["voxels"]).cuda().requires_grad_(True)
    params = pack_plain(dec).cuda().requires_grad_(True)
    tc = None if form == "fp32" else TcWeights.from_decoder(dec, "cuda", mode=form)
    o = torch.from_numpy(g["o_hit"]).cuda()
    d = torch.from_numpy(g["d_hit"]).cuda()
    seg = masked_segments(o, d, -1.5, 12, 0.25, torch.from_numpy(g["mask"]).cuda(), 1.0)
    rgb, reg = render_segments(vox, params, seg, d, kind, True, tc)
    loss = torch.nn.functional.mse_loss(rgb, torch.from_numpy(g["target"]).cuda()) + 1e-5 * reg
    loss.backward()
    torch.cuda.synchronize()
    if tc is not None:
        assert int(tc.err.item()) == 0
    return rgb, reg, loss, vox, params, seg


def check_forward_and_loss(g, kind, form="fp32"):
    rgb, reg, loss, *_ = run_field(g, kind, form)
    assert np.abs(rgb.detach().cpu().numpy() - g[f"{kind}/rgb"]).max() < 1e-5
    assert abs(loss.item() - float(g[f"{kind}/loss"])) < 1e-6


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_forward_and_loss_match_reference(g, kind):
    check_forward_and_loss(g, kind)


def check_gradients_vs_reference_autograd(g, kind, form="fp32"):
    from diver_gb300.decoder import unpack_plain_grad

    _, _, _, vox, params, _ = run_field(g, kind, form)
    gv = vox.grad.reshape(-1, vox.shape[-1]).cpu().numpy()
    rows = g[f"{kind}/grad_voxels_rows"]
    ref = g[f"{kind}/grad_voxels"]
    scale = np.abs(ref).max()
    assert np.abs(gv[rows] - ref).max() <= 1e-4 * scale
    assert np.abs(np.delete(gv, rows, 0)).max() == 0
    grads = unpack_plain_grad(kind, 32, params.grad.cpu())
    n1 = KINDS[kind]
    for i, (dw, db) in enumerate(grads):
        name = f"mlp1.{2 * i}" if i < n1 else f"mlp2.{2 * (i - n1)}"
        rw, rb = g[f"{kind}/grad/{name}.weight"], g[f"{kind}/grad/{name}.bias"]
        s = max(np.abs(rw).max(), np.abs(rb).max(), 1e-12)
        assert np.abs(dw.numpy() - rw).max() <= 1e-4 * s, name
        assert np.abs(db.numpy() - rb).max() <= 1e-4 * s, name


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_gradients_match_reference_autograd(g, kind):
    check_gradients_vs_reference_autograd(g, kind)


def check_gradients_vs_central_differences(g, kind, form="fp32"):
    """Central differences of the FP64 oracle loss (same segments) for sampled
    feature entries and decoder weights: relative error <= 1e-4."""
    from diver_gb300.decoder import unpack_plain_grad

    _, _, _, vox, params, seg = run_field(g, kind, form)
    gv = vox.grad.cpu().double()
    gp = unpack_plain_grad(kind, 32, params.grad.cpu())
    dec = decoder_from_golden(g, kind)
    L = [(w.double(), b.double()) for w, b in dec.layers]
    V = torch.from_numpy(g["voxels"]).double()
    segs = seg.seg.cpu().double()
    ray = seg.ray.cpu().long()
    counts = seg.counts.cpu()
    dirs = torch.from_numpy(g["d_hit"]).double()
    tgt = torch.from_numpy(g["target"]).double()
    n1 = KINDS[kind]

    def parts(V_, L_):
        rgb, sigma, _ = torch_ref.forward(V_, L_, n1, segs, ray, counts, dirs)
        mse = torch.nn.functional.mse_loss(rgb, tgt).item()
        reg = torch.log(1 + sigma ** 2 / 0.5).mean().item()
        return np.array([mse, 1e-5 * reg])

    def central(Vp, Lp, Vm, Lm):
        # difference each loss term on its own: the tiny sparsity term would
        # otherwise be lost in the rounding of the much larger MSE
        return float(((parts(Vp, Lp) - parts(Vm, Lm)) / (2 * h)).sum())

    h = 1e-6
    gen = torch.Generator().manual_seed(11)
    got, fd = [], []
    flat = gv.reshape(-1)
    nz = torch.nonzero(flat.abs() > 1e-3 * flat.abs().max())[:, 0]
    for idx in nz[torch.randperm(nz.numel(), generator=gen)[:12]].tolist():
        Vp, Vm = V.clone(), V.clone()
        Vp.view(-1)[idx] += h
        Vm.view(-1)[idx] -= h
        fd.append(central(Vp, L, Vm, L))
        got.append(flat[idx].item())
    for li in range(len(L)):
        w, b = L[li]
        dw = gp[li][0].double()
        for _ in range(3):
            i = torch.randint(0, w.shape[0], (1,), generator=gen).item()
            j = torch.randint(0, w.shape[1], (1,), generator=gen).item()
            Lp = [(x.clone(), y.clone()) for x, y in L]
            Lm = [(x.clone(), y.clone()) for x, y in L]
            Lp[li][0][i, j] += h
            Lm[li][0][i, j] -= h
            fd.append(central(V, Lp, V, Lm))
            got.append(dw[i, j].item())
    got, fd = np.array(got), np.array(fd)
    rel = np.linalg.norm(got - fd) / np.linalg.norm(fd)
    assert rel < 1e-4, rel
    big = np.abs(fd) > 1e-2 * np.abs(fd).max()
    assert (np.abs(got - fd)[big] <= 1e-4 * np.abs(fd)[big] + 1e-9).all()
    return rel


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_gradients_match_fp64_central_differences(g, kind):
    check_gradients_vs_central_differences(g, kind)


def test_render_small_scene_matches_fp64_oracle():
    """Full 200x200 view of the 64^3 scene through DIVeRField: FP32 plain form
    vs the FP64 oracle, max abs rgb <= 1e-5."""
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    o, v = scenes.small_view("cpu")
    field = DIVeRField.from_scene(sc, "cuda")
    with torch.no_grad():
        rgb, _ = field(o.cuda(), v.cuda())
    inter, num, _ = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, 64, sc.voxel_size, sc.mask.numpy(), 1.0)
    segs = torch.from_numpy(orc.csr_from_padded(inter, num)).double()
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    L = [(w.double(), b.double()) for w, b in sc.decoder.layers]
    ref, _, _ = torch_ref.forward(sc.features.double(), L, 3, segs, ray, torch.from_numpy(num), v.double())
    assert np.abs(rgb.cpu().numpy() - ref.numpy()).max() < 1e-5
