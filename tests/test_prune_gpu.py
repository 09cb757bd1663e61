"""GPU: occupancy extraction (prune.py:86-145) against the oracle.

Stated tolerance: alpha_map within 1e-6 abs of the FP64-accumulated oracle
restatement of the reference (weights of torch_ref.render, np.maximum.at at the
segment's voxel, boundary band `pad` excluded); the thresholded masks agree
except where the oracle's value is within 1e-5 of the threshold."""
import numpy as np
import pytest
import torch

from oracle import native as orc
from oracle import torch_ref

pytestmark = pytest.mark.gpu


def _oracle_alpha(sc, o, v, pad):
    n = sc.voxel_num
    inter, num, _ = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, n, sc.voxel_size, sc.mask.numpy(), 1.0)
    segs = torch.from_numpy(orc.csr_from_padded(inter, num))
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    L = [(w.double(), b.double()) for w, b in sc.decoder.layers]
    feat = torch_ref.integrate(sc.features, segs[:, :3].double(), segs[:, 3:].double(), dtype=torch.float64)
    sigma, color = torch_ref.decode(L, sc.decoder.n_mlp1, feat, v.double()[ray])
    sig_p, mask = torch_ref.scatter_padded(sigma, torch.from_numpy(num))
    col_p, _ = torch_ref.scatter_padded(color, torch.from_numpy(num))
    _, weight = torch_ref.render(col_p, sig_p, mask, True)
    w = weight[mask].numpy()
    c = torch.minimum((segs[:, :3] + np.float32(1e-4)).long(), (segs[:, 3:] + np.float32(1e-4)).long()).numpy()
    keep = ((c >= pad) & (c <= n - 1 - pad)).all(1)
    idx = c[keep, 0] + c[keep, 1] * n + c[keep, 2] * n * n
    alpha = np.zeros(n ** 3)
    np.maximum.at(alpha, idx, w[keep])
    return alpha.reshape(n, n, n)


@pytest.mark.parametrize("pad", [0, 2])
def test_alpha_map_matches_oracle(pad):
    from diver_gb300 import scenes
    from diver_gb300.prune import extract_alpha_map, prune_mask, rays_hitting
    from diver_gb300.renderer import DIVeRField

    sc = scenes.small_scene("cpu")
    sc.decoder.layers[sc.decoder.n_mlp1 - 1][1][0] += 0.6
    o, v = scenes.small_view("cpu")
    field = DIVeRField.from_scene(sc, "cuda")
    rays = torch.cat([o, v], 1).cuda()
    alpha = extract_alpha_map(field, rays, batch=4000, pad=pad)
    ref = _oracle_alpha(sc, o, v, pad)
    got = alpha.cpu().double().numpy()
    assert np.abs(got - ref).max() <= 1e-6
    assert (ref > 0).sum() > 100  # the view covers a real part of the grid
    mask = prune_mask(alpha, 1e-2).cpu().numpy()
    differ = mask != (ref > 1e-2)
    assert np.all(np.abs(ref[differ] - 1e-2) < 1e-5)
    # bias sampling: rays that cross the pruned grid, vs the oracle walk over that mask
    hit = rays_hitting(field, o.cuda(), v.cuda(), torch.from_numpy(ref > 1e-2).cuda()).cpu().numpy()
    _, num, _ = orc.masked_walk(o.numpy(), v.numpy(), sc.xyzmin, sc.voxel_num, sc.voxel_size, ref > 1e-2, 1.0)
    assert np.array_equal(hit, num > 0)
