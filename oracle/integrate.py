"""ORACLE — test infrastructure only.  numpy restatement of the reference's
closed-form segment integral `integrate(voxels, coord_i, coord_o)`
(utils/integrator.py:62-112), in float64 (default) or float32.

The integrated feature is the mean of the trilinear interpolant of the 8
corner vectors along the segment, written as the reference writes it:
  A * X + sum_d B_d * Y_d + sum_d C_d * Z_d + F000
with A, B, C moments of the local coordinates and X, Y, Z the trilinear
coefficients (differences of corner vectors).
"""
from __future__ import annotations

import numpy as np


def corner_index(coord_i: np.ndarray, coord_o: np.ndarray, n_vert):
    """pmin and the clamped upper corner (utils/integrator.py:75-79)."""
    ci = np.asarray(coord_i, np.float32)
    co = np.asarray(coord_o, np.float32)
    eps = np.float32(1e-4)
    pmin = np.minimum((ci + eps).astype(np.int64), (co + eps).astype(np.int64))
    nv = np.asarray(n_vert, np.int64).reshape(-1)
    pmax = np.minimum(pmin + 1, nv - 1 if nv.size == 3 else nv[0] - 1)
    return pmin, pmax


def integrate(voxels: np.ndarray, coord_i: np.ndarray, coord_o: np.ndarray, dtype=np.float64) -> np.ndarray:
    voxels = np.asarray(voxels)
    n = voxels.shape[-2]  # the reference clamps every axis with voxels.shape[-2]
    pmin, pmax = corner_index(coord_i, coord_o, n)
    x0, y0, z0 = pmin[:, 0], pmin[:, 1], pmin[:, 2]
    x1, y1, z1 = pmax[:, 0], pmax[:, 1], pmax[:, 2]

    def F(z, y, x):
        return voxels[z, y, x].astype(dtype)

    f000, f001, f010, f011 = F(z0, y0, x0), F(z0, y0, x1), F(z0, y1, x0), F(z0, y1, x1)
    f100, f101, f110, f111 = F(z1, y0, x0), F(z1, y0, x1), F(z1, y1, x0), F(z1, y1, x1)
    # f{z}{y}{x}
    P0 = np.asarray(coord_i, np.float32).astype(dtype) - pmin.astype(dtype)
    P1 = np.asarray(coord_o, np.float32).astype(dtype) - pmin.astype(dtype)
    if dtype == np.float32:
        P0 = (np.asarray(coord_i, np.float32) - pmin).astype(np.float32)
        P1 = (np.asarray(coord_o, np.float32) - pmin).astype(np.float32)
    Ps = P0 + P1
    A = Ps.prod(1) / 12 + (P0.prod(1) + P1.prod(1)) / 6
    X = (f100 - f000 - f110 + f010) - (f101 - f001 - f111 + f011)
    feat = A[:, None] * X
    # pairs (x,y), (y,z), (z,x)
    roll = [1, 2, 0]
    B = (P0 * P0[:, roll] + P1 * P1[:, roll]) / 3 + (P0 * P1[:, roll] + P1 * P0[:, roll]) / 6
    Yxy = f000 - f010 - f001 + f011
    Yyz = f000 - f010 - f100 + f110
    Yzx = f000 - f100 - f001 + f101
    feat = feat + B[:, 0:1] * Yxy + B[:, 1:2] * Yyz + B[:, 2:3] * Yzx
    Cm = Ps / 2
    feat = feat + Cm[:, 0:1] * (f001 - f000) + Cm[:, 1:2] * (f010 - f000) + Cm[:, 2:3] * (f100 - f000)
    return feat + f000


def corner_weights(coord_i, coord_o, dtype=np.float64):
    """Per-corner weights w[S, 8] (bit 0 = x, bit 1 = y, bit 2 = z) of the same
    integral; the gradient of the feature with respect to each corner vector."""
    pmin, _ = corner_index(coord_i, coord_o, 1 << 30)
    P0 = np.asarray(coord_i, np.float32).astype(dtype) - pmin
    P1 = np.asarray(coord_o, np.float32).astype(dtype) - pmin
    Ix, Iy, Iz = [(P0[:, d] + P1[:, d]) / 2 for d in range(3)]

    def I2(a, b):
        return (P0[:, a] * P0[:, b] + P1[:, a] * P1[:, b]) / 3 + (P0[:, a] * P1[:, b] + P1[:, a] * P0[:, b]) / 6

    Ixy, Iyz, Ixz = I2(0, 1), I2(1, 2), I2(0, 2)
    Ixyz = (P0 + P1).prod(1) / 12 + (P0.prod(1) + P1.prod(1)) / 6
    w = np.empty((P0.shape[0], 8), dtype)
    w[:, 7] = Ixyz
    w[:, 3] = Ixy - Ixyz
    w[:, 5] = Ixz - Ixyz
    w[:, 6] = Iyz - Ixyz
    w[:, 1] = Ix - Ixy - Ixz + Ixyz
    w[:, 2] = Iy - Ixy - Iyz + Ixyz
    w[:, 4] = Iz - Ixz - Iyz + Ixyz
    w[:, 0] = 1 - Ix - Iy - Iz + Ixy + Iyz + Ixz - Ixyz
    return w
