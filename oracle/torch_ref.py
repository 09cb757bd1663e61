"""ORACLE — test infrastructure only.  torch restatement of the reference's
training/offline decode path, used for reference gradients (autograd, float32
or float64), as the timed CPU baseline, and (on CUDA tensors, fed by the
reference's own traversal kernels) as the reference's GPU path in bench.py's
reference arm:

  integrate     utils/integrator.py:62-112
  pos_enc       model/mlps.py:6-18 (L = 4 bands)
  mlp           model/mlps.py:21-30 (Linear/ReLU stack)
  decode        model/diver.py:270-290 (mlp1 -> sigma, hidden; PE; mlp2; sigmoid)
  render        model/diver.py:295-319 (relu, 1-exp, shifted cumprod, white back)
  loss          train.py:84-85,109-113 (MSE + l_s * mean(log(1 + sigma^2 / 0.5)))
  implicit_mlp  model/mlps.py:34-81 (PE of the vertex position, Linear+ReLU
                layers with the encoded input re-joined before the skip layers,
                a final Linear)

Segment lists come in the CSR form (offsets, seg [S,6], ray [S]); the padded
[B, M] layout of the reference is rebuilt here the way DIVeR.forward scatters
with its boolean mask, so the arithmetic is the reference's.
"""
from __future__ import annotations

import math

import torch


def integrate(voxels: torch.Tensor, coord_i: torch.Tensor, coord_o: torch.Tensor, per_axis: bool = False,
              dtype: torch.dtype | None = None) -> torch.Tensor:
    """per_axis: clamp each axis to its own vertex count (grids that are not
    cubic); the reference clamps every axis with voxels.shape[-2].  dtype:
    arithmetic type when it differs from the grid's (the corner rows are
    gathered first, then converted, so a large FP32 grid needs no FP64 copy)."""
    n, c = voxels.shape[-2:]
    pmin = torch.min((coord_i + 1e-4).long(), (coord_o + 1e-4).long())
    xmin, ymin, zmin = pmin.split(1, dim=-1)
    if per_axis:
        nz, ny, nx = voxels.shape[:3]
        hi = torch.tensor([nx - 1, ny - 1, nz - 1], device=coord_i.device)
        xmax, ymax, zmax = torch.minimum(pmin + 1, hi).split(1, dim=-1)
    else:
        xmax, ymax, zmax = (pmin + 1).clamp_max(n - 1).split(1, dim=-1)
    corners = [voxels[zmin, ymin, xmin], voxels[zmin, ymin, xmax], voxels[zmin, ymax, xmin], voxels[zmin, ymax, xmax],
               voxels[zmax, ymin, xmin], voxels[zmax, ymin, xmax], voxels[zmax, ymax, xmin], voxels[zmax, ymax, xmax]]
    dt = dtype or voxels.dtype
    F = torch.stack(corners, 0).reshape(2, 2, 2, -1, c).to(dt)  # [z][y][x]
    P = torch.stack([coord_i - pmin, coord_o - pmin], 0).permute(0, 2, 1).to(dt)  # [2][xyz][S]
    A = P.sum(0).prod(0) / 12 + P.prod(1).sum(0) / 6
    X = F[1] - F[0]
    X = X[0] - X[1]
    X = X[0] - X[1]
    feat = A[:, None] * X
    P_roll = P[:, [1, 2, 0]]
    B = (P * P_roll).sum(0) / 3 + (P * P_roll[[1, 0]]).sum(0) / 6
    Y = F[0, 0, 0, None] - F[[0, 0, 1], [1, 1, 0], 0] - F[[0, 1, 0], 0, [1, 0, 1]] + F[[0, 1, 1], [1, 1, 0], [1, 0, 1]]
    feat = feat + torch.einsum("dk,dkc->kc", B, Y)
    Cm = P.sum(0) / 2
    Z = F[[0, 0, 1], [0, 1, 0], [1, 0, 0]] - F[0, 0, 0, None]
    feat = feat + torch.einsum("dk,dkc->kc", Cm, Z)
    return feat + F[0, 0, 0]


def pos_enc(x: torch.Tensor, L: int = 4) -> torch.Tensor:
    out = [x]
    for l in range(L):
        out.append(torch.sin((2 ** l * math.pi) * x))
        out.append(torch.cos((2 ** l * math.pi) * x))
    return torch.cat(out, -1)


def mlp(x: torch.Tensor, layers) -> torch.Tensor:
    for i, (w, b) in enumerate(layers):
        x = torch.nn.functional.linear(x, w, b)
        if i + 1 < len(layers):
            x = torch.relu(x)
    return x


def decode(layers, n_mlp1: int, feature: torch.Tensor, dirs: torch.Tensor):
    """(sigma_raw [S], color [S,3]) for per-segment features and directions."""
    x = mlp(feature, layers[:n_mlp1])
    sigma, x = x[:, 0], x[:, 1:]
    x = torch.cat([x, pos_enc(dirs)], -1)
    color = torch.sigmoid(mlp(x, layers[n_mlp1:]))
    return sigma, color


def scatter_padded(values: torch.Tensor, counts: torch.Tensor, fill=0.0):
    """CSR values [S, ...] -> padded [B, M, ...] and mask [B, M] (ray-major order)."""
    B = counts.numel()
    M = int(counts.max().item()) if B else 0
    mask = torch.arange(M, device=counts.device)[None, :] < counts[:, None].long()
    out = torch.full((B, M) + tuple(values.shape[1:]), fill, dtype=values.dtype, device=values.device)
    out = out.clone()
    out[mask] = values
    return out, mask


def render(color: torch.Tensor, sigma: torch.Tensor, mask: torch.Tensor, white_back: bool = True):
    sigma = torch.relu(sigma)
    alpha = 1 - torch.exp(-sigma * mask)
    shifted = torch.nn.functional.pad(1 - alpha[None, :, :-1], (1, 0), value=1)[0]
    weight = alpha * torch.cumprod(shifted, -1)
    rgb = (weight[:, :, None] * color).sum(1)
    if white_back:
        rgb = rgb + (1 - weight.sum(1, keepdim=True))
    return rgb, weight


def forward(voxels, layers, n_mlp1, seg, seg_ray, counts, dirs, white_back=True, per_axis=False, dtype=None):
    """Full decode path over CSR segments: returns rgb [B,3], sigma [B,M], mask [B,M]."""
    feat = integrate(voxels, seg[:, :3], seg[:, 3:], per_axis, dtype)
    s, c = decode(layers, n_mlp1, feat, dirs[seg_ray.long()])
    counts = counts.to(feat.device)
    sigma, mask = scatter_padded(s, counts)
    color, _ = scatter_padded(c, counts)
    rgb, _ = render(color, sigma, mask, white_back)
    return rgb, sigma, mask


def loss(rgb, target, sigma, l_s=1e-5):
    return torch.nn.functional.mse_loss(rgb, target) + l_s * torch.log(1 + sigma ** 2 / 0.5).mean()


def implicit_mlp(x: torch.Tensor, params: dict, depth: int, skips, enc: int) -> torch.Tensor:
    """params: 'pts_linears.{i}.weight/bias' (i < depth) and 'feature_linear.weight/bias'."""
    points = pos_enc(x, enc)
    p = points
    for i in range(depth):
        if i in skips:
            p = torch.cat([points, p], 1)
        p = torch.relu(torch.nn.functional.linear(p, params[f"pts_linears.{i}.weight"], params[f"pts_linears.{i}.bias"]))
    return torch.nn.functional.linear(p, params["feature_linear.weight"], params["feature_linear.bias"])
