"""GPU: the one-launch training loss (renderer.l2_loss: dv_l2_loss_fwd/bwd)
against torch's mse_loss + l_s * reg, values and gradients, and the
sparsity-term mean (dv_reg_mean) against the per-ray terms.

Tolerances (stated): loss within 1e-6 relative (the sums run in another
order), gradients within 1e-6 relative to their largest magnitude."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("B", [1, 777, 4096])
def test_l2_loss_matches_torch(B):
    from diver_gb300.renderer import l2_loss

    g = torch.Generator().manual_seed(B)
    rgb0 = torch.rand(B, 3, generator=g).cuda()
    tgt = torch.rand(B, 3, generator=g).cuda()
    reg0 = torch.rand((), generator=g).cuda()
    l_s = 1e-3
    outs = []
    for fn in (lambda r, s: l2_loss(r, s, tgt, l_s),
               lambda r, s: torch.nn.functional.mse_loss(r, tgt) + l_s * s):
        rgb = rgb0.clone().requires_grad_(True)
        reg = reg0.clone().requires_grad_(True)
        loss = fn(rgb, reg)
        (loss * 3.0).backward()
        outs.append((loss.detach(), rgb.grad, reg.grad))
    (a, ga, ra), (b, gb, rb) = outs
    assert abs(a.item() - b.item()) <= 1e-6 * abs(b.item())
    assert (ga - gb).abs().max().item() <= 1e-6 * gb.abs().max().item()
    assert abs(ra.item() - rb.item()) <= 1e-6 * abs(rb.item())


def test_reg_mean_with_device_and_host_maximum():
    from diver_gb300 import _native as N

    B = 3000
    reg = torch.rand(B, generator=torch.Generator().manual_seed(5)).cuda()
    mean = torch.empty((), device="cuda")
    inv = torch.empty(1, device="cuda")
    for m_dev, m_host, m in ((torch.tensor([37], dtype=torch.int32, device="cuda"), 0.0, 37.0),
                             (torch.tensor([0], dtype=torch.int32, device="cuda"), 0.0, 1.0),
                             (None, 12.0, 12.0)):
        N.call("dv_reg_mean", B, N.ptr(reg), N.ptr(m_dev), m_host, N.ptr(mean), N.ptr(inv), N.stream())
        torch.cuda.synchronize()
        ref = reg.double().sum().item() / (B * m)
        assert abs(mean.item() - ref) <= 1e-6 * ref
        assert inv.item() == pytest.approx(1.0 / m, rel=1e-7)
