"""Implicit-stage integrator (utils/integrator.py:3-59) against the
reference's own integrate_mlp + ImplicitMLP (golden fixture made by
tests/golden/make_implicit_golden.py).

Stated tolerance: features within 1e-5 relative to their largest magnitude,
MLP parameter gradients within 1e-4 relative L2 (FP32 arithmetic; the table
gradient is accumulated with atomics).  The MLP itself is the oracle's
restatement of ImplicitMLP, standing in for the caller's module."""
import numpy as np
import pytest
import torch

from oracle import torch_ref


def test_oracle_implicit_mlp_matches_reference_weights_shapes(golden):
    g = golden("implicit_ref.npz")
    N, C, D, W, ENC = (int(x) for x in g["meta"][:5])
    assert g["w:pts_linears.0.weight"].shape == (W, 3 + 6 * ENC)
    assert g["w:feature_linear.weight"].shape == (C, W)


@pytest.mark.gpu
def test_integrate_mlp_matches_reference(golden):
    from diver_gb300.integrator import integrate_mlp

    g = golden("implicit_ref.npz")
    N, C, D, W, ENC = (int(x) for x in g["meta"][:5])
    skips = [int(x) for x in g["meta"][5:]]
    params = {k[2:]: torch.from_numpy(g[k]).cuda().requires_grad_(True) for k in g.files if k.startswith("w:")}
    seg = torch.from_numpy(g["seg"]).cuda()
    feat = integrate_mlp(lambda x: torch_ref.implicit_mlp(x, params, D, skips, ENC), N + 1, C, seg[:, :3], seg[:, 3:])
    ref = torch.from_numpy(g["feature"])
    assert (feat.detach().cpu() - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
    G = torch.cos(torch.arange(feat.numel(), dtype=torch.float32) * 0.37).reshape(feat.shape).cuda()
    (feat * G).sum().backward()
    for name, p in params.items():
        r = torch.from_numpy(g["g:" + name])
        got = p.grad.cpu()
        assert ((got - r).norm() / r.norm()).item() <= 1e-4, name


def test_oracle_restatement_reproduces_reference(golden):
    """The oracle's ImplicitMLP evaluated at every vertex, integrated as a dense
    grid, gives the reference's integrate_mlp features."""
    g = golden("implicit_ref.npz")
    N, C, D, W, ENC = (int(x) for x in g["meta"][:5])
    skips = [int(x) for x in g["meta"][5:]]
    params = {k[2:]: torch.from_numpy(g[k]).double() for k in g.files if k.startswith("w:")}
    n = N + 1
    z, y, x = torch.meshgrid(*[torch.arange(n)] * 3, indexing="ij")
    pts = torch.stack([z, y, x], -1).reshape(-1, 3).double() / (n * 0.5) - 1.0
    grid = torch_ref.implicit_mlp(pts, params, D, skips, ENC).reshape(n, n, n, C)
    seg = torch.from_numpy(g["seg"])
    feat = torch_ref.integrate(grid, seg[:, :3], seg[:, 3:], dtype=torch.float64)
    ref = torch.from_numpy(g["feature"]).double()
    assert (feat - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
