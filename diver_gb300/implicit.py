"""The implicit grid of DIVeR's coarse stage (model/mlps.py:34-81): an MLP from
a vertex position to its feature vector, queried at the unique corners of the
segments by integrator.integrate_mlp.

Same architecture and constructor arguments as the reference's ImplicitMLP
(depth D, width C, skip layers S that re-join the encoded input, output
dimension, PE bands), so its state dict loads unchanged.  Its layers are plain
GEMMs (cuBLAS through torch, BF16 under autocast); the corner deduplication
and the integral around it are this package's kernels.
"""
from __future__ import annotations

import math

import torch
from torch import nn


class ImplicitMLP(nn.Module):
    def __init__(self, D: int, C: int, S, dim_out: int, dim_enc: int):
        super().__init__()
        self.D, self.C, self.skips, self.dim_out, self.enc = D, C, list(S), dim_out, dim_enc
        self.input_ch = dim_enc * 2 * 3 + 3
        self.pts_linears = nn.ModuleList(
            [nn.Linear(self.input_ch, C)]
            + [nn.Linear(C + self.input_ch if i in self.skips else C, C) for i in range(1, D)])
        self.feature_linear = nn.Linear(C, dim_out)

    def encode(self, x: torch.Tensor) -> torch.Tensor:
        out = [x]
        for l in range(self.enc):
            out.append(torch.sin((2 ** l * math.pi) * x))
            out.append(torch.cos((2 ** l * math.pi) * x))
        return torch.cat(out, -1)

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        pts = self.encode(x)
        h = pts
        for i, lin in enumerate(self.pts_linears):
            if i in self.skips:
                h = torch.cat([pts, h], 1)
            h = torch.relu(lin(h))
        return self.feature_linear(h)
