"""CPU: the integrate / decode / render / loss oracle restatements against
fixtures from the reference's own Python modules (tests/golden/decode_ref.npz,
made by tests/golden/make_golden.py)."""
import numpy as np
import pytest
import torch

from oracle import integrate as oint
from oracle import native as orc
from oracle import torch_ref

KINDS = {"diver32": 3, "diver64": 2}  # kind -> number of mlp1 layers


@pytest.fixture(scope="module")
def g(golden):
    return golden("decode_ref.npz")


def layers(g, kind):
    n1 = KINDS[kind]
    L = [(torch.from_numpy(g[f"{kind}/mlp1.{2 * i}.weight"]), torch.from_numpy(g[f"{kind}/mlp1.{2 * i}.bias"])) for i in range(n1)]
    L += [(torch.from_numpy(g[f"{kind}/mlp2.{2 * i}.weight"]), torch.from_numpy(g[f"{kind}/mlp2.{2 * i}.bias"])) for i in range(2)]
    return L


def test_integrate_oracle_matches_reference(g):
    seg = g["seg"]
    f64 = oint.integrate(g["voxels"], seg[:, :3], seg[:, 3:])
    assert np.abs(f64 - g["feature"]).max() < 2e-7
    f32 = oint.integrate(g["voxels"], seg[:, :3], seg[:, 3:], dtype=np.float32)
    assert np.abs(f32 - g["feature"]).max() < 2e-7
    tr = torch_ref.integrate(torch.from_numpy(g["voxels"]), torch.from_numpy(seg[:, :3]), torch.from_numpy(seg[:, 3:]))
    assert np.array_equal(tr.numpy(), g["feature"])  # same torch ops, same inputs


def test_corner_weights_reproduce_integral_and_sum_to_one(g):
    seg = g["seg"]
    w = oint.corner_weights(seg[:, :3], seg[:, 3:])
    assert np.abs(w.sum(1) - 1).max() < 1e-12
    pmin, pmax = oint.corner_index(seg[:, :3], seg[:, 3:], g["voxels"].shape[0])
    vox = g["voxels"].astype(np.float64)
    f = np.zeros((seg.shape[0], vox.shape[-1]))
    for j in range(8):
        x = np.where(j & 1, pmax[:, 0], pmin[:, 0])
        y = np.where(j & 2, pmax[:, 1], pmin[:, 1])
        z = np.where(j & 4, pmax[:, 2], pmin[:, 2])
        f += w[:, j:j + 1] * vox[z, y, x]
    assert np.abs(f - g["feature"]).max() < 2e-7


def test_constant_field_integrates_to_itself():
    vox = np.full((5, 5, 5, 4), 0.37, np.float32)
    seg = np.array([[0.2, 1.0, 3.3, 1.0, 0.4, 3.9], [2.0, 2.0, 2.0, 3.0, 2.5, 2.1]], np.float32)
    f = oint.integrate(vox, seg[:, :3], seg[:, 3:])
    assert np.abs(f - np.float64(np.float32(0.37))).max() < 1e-12


def test_linear_field_gives_midpoint_value():
    # f(x,y,z) = ax + by + cz + d is integrated exactly: the mean equals f(midpoint)
    n = 6
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    vox = (0.3 * x - 0.2 * y + 0.7 * z + 0.1)[..., None].astype(np.float64)
    rng = np.random.default_rng(0)
    base = rng.integers(0, n - 1, (50, 3))
    p0 = (base + rng.uniform(0, 1, (50, 3))).astype(np.float32)
    p1 = (base + rng.uniform(0, 1, (50, 3))).astype(np.float32)
    f = oint.integrate(vox, p0, p1)[:, 0]
    mid = (p0.astype(np.float64) + p1) / 2
    assert np.abs(f - (0.3 * mid[:, 0] - 0.2 * mid[:, 1] + 0.7 * mid[:, 2] + 0.1)).max() < 1e-9


@pytest.mark.parametrize("kind", ["diver32", "diver64"])
def test_torch_ref_forward_loss_and_grads_match_reference(g, kind):
    vox = torch.from_numpy(g["voxels"]).clone().requires_grad_(True)
    L = [(w.clone().requires_grad_(True), b.clone().requires_grad_(True)) for w, b in layers(g, kind)]
    o, d = g["o_hit"], g["d_hit"]
    inter, num, _ = orc.masked_walk(o, d, -1.5, 12, 0.25, g["mask"], 1.0)
    seg = torch.from_numpy(orc.csr_from_padded(inter, num))
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    rgb, sigma, mask = torch_ref.forward(vox, L, KINDS[kind], seg, ray, torch.from_numpy(num), torch.from_numpy(d))
    assert torch.equal(mask, torch.from_numpy(g[f"{kind}/mask"]))
    assert (rgb.detach().numpy() - g[f"{kind}/rgb"]).__abs__().max() < 1e-6
    assert (sigma.detach().numpy() - g[f"{kind}/sigma"]).__abs__().max() < 1e-6
    loss = torch_ref.loss(rgb, torch.from_numpy(g["target"]), sigma)
    assert abs(loss.item() - float(g[f"{kind}/loss"])) < 1e-6
    loss.backward()
    gv = vox.grad.reshape(-1, vox.shape[-1]).numpy()
    rows = g[f"{kind}/grad_voxels_rows"]
    assert np.abs(gv[rows] - g[f"{kind}/grad_voxels"]).max() < 1e-8
    assert np.abs(np.delete(gv, rows, 0)).max() == 0
    n1 = KINDS[kind]
    for i, (w, b) in enumerate(L):
        name = f"mlp1.{2 * i}" if i < n1 else f"mlp2.{2 * (i - n1)}"
        assert np.abs(w.grad.numpy() - g[f"{kind}/grad/{name}.weight"]).max() < 1e-7
        assert np.abs(b.grad.numpy() - g[f"{kind}/grad/{name}.bias"]).max() < 1e-7
