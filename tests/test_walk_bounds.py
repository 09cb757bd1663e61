"""CPU: every walk is bounded.  Rays whose direction is zero or has a
non-finite component are misses (the reference kernels would never leave
their loop on them); every other ray leaves the grid within nx + ny + nz + 3
steps, one grid plane per step, so the step bound the walks carry is never
reached.  Checked on the C restatement of the walks (oracle/dda.c), which
mirrors the CUDA kernels' checks line for line; such rays are never sent to
a GPU."""
import numpy as np
import pytest

from oracle import native as orc

N = 16
XYZMIN, VS = -1.5, 3.0 / N
BAD_DIRS = np.array([
    [0.0, 0.0, 0.0],
    [np.nan, 0.0, 1.0],
    [np.nan, np.nan, np.nan],
    [np.inf, 0.0, 0.0],
    [0.3, -np.inf, 0.1],
    [1.0, np.nan, 0.0],
], np.float32)


def _origins(k):
    inside = np.full((k, 3), 0.1, np.float32)
    outside = np.full((k, 3), -4.0, np.float32)
    return np.concatenate([inside, outside])


@pytest.mark.timeout(60)
def test_degenerate_directions_are_misses_in_every_walk():
    orc.walk_cap_hits(reset=True)
    o = _origins(len(BAD_DIRS))
    v = np.concatenate([BAD_DIRS, BAD_DIRS])
    mask = np.ones((N, N, N), bool)
    _, num, tns = orc.dense_walk(o, v, XYZMIN, N, VS)
    assert (num == 0).all() and (tns == -1).all()
    _, num, _ = orc.masked_walk(o, v, XYZMIN, N, VS, mask, 1.0)
    assert (num == 0).all()
    _, num, _ = orc.masked_walk_grid(o, v, [XYZMIN] * 3, (N, N, N // 2), VS, np.ones((N // 2, N, N), bool))
    assert (num == 0).all()
    # real-time path: first hit through the octree, then one round of the march
    NR = 64
    B = len(v)
    coords = np.zeros((8, B, 6), np.float32)
    finish = np.zeros(B, np.uint8)
    rgba = np.zeros((B, 4), np.float32)
    octree = np.ones(1 + 64 + 4096, bool)
    orc.aabb(coords, v, np.array([NR / 2, NR / 2, NR / 2], np.float32), finish, rgba, octree, NR)
    assert finish.all() and (coords[7, :, 3] == -1).all()
    finish[:] = 0  # the march also refuses them on its own
    coords[7, :, 3:6] = NR / 2
    orc.ray_march(coords, v, np.ones((NR, NR, NR), bool), finish, NR)
    assert (coords[0, :, 0] == -1).all()
    assert orc.walk_cap_hits(reset=True) == 0


def test_valid_rays_stay_within_the_step_bound():
    """Random origins inside and outside the grid, random directions
    (including axis-parallel ones and components down to 1e-30): the
    number of recorded points of the dense walk (1 + steps inside) never
    exceeds 3N + 3, and no walk reaches its bound."""
    rng = np.random.default_rng(0)
    B = 4000
    o = rng.uniform(-3.0, 3.0, (B, 3)).astype(np.float32)
    v = rng.normal(size=(B, 3)).astype(np.float32)
    v[:400, 1:] = 0.0  # along x
    v[400:800, 0] = 0.0  # in the yz plane
    v[800:1200, 2] = 1e-30
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    orc.walk_cap_hits(reset=True)
    _, num, _ = orc.dense_walk(o, v, XYZMIN, N, VS)
    assert num.max() <= 3 * N + 3
    _, mnum, _ = orc.masked_walk(o, v, XYZMIN, N, VS, np.ones((N, N, N), bool), 1.0)
    assert (mnum <= np.maximum(num - 1, 0)).all()
    assert orc.walk_cap_hits(reset=True) == 0
