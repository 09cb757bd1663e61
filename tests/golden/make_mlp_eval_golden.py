"""Makes tests/golden/mlp_eval_ref.npz: outputs of the reference's own
real-time decoder kernels (utils/mlp_evaluation{,64}/src/mlp_eval.cu, built by
oracle/ref_kernels.build_mlp_eval_cubins with the texture reference patched
into a plain array) on a GB300, for the real-time loop of eval_rt.py:106-122.

Scene: the 64^3 sphere scene converted to the serialized real-time form
(DIVeR32, and DIVeR64 over 32 channels), density bias raised by BIAS so that
rays need several march rounds and some terminate.
Frame: rows 392..407 of an 800x800 view (the reference kernel assumes images
800 pixels wide).  The octree first hit and the 8-hit march of every round run
in the C restatement of the reference traversal kernels (oracle/dda.c, pinned
bit-exact to them); every round's decode is the reference kernel's.  Stored
per decoder: rgba after the first round and after the last, the finish flags,
the number of rounds.

Run on a GPU machine from the repository root, after the cubins exist:
    python tests/golden/make_mlp_eval_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

ROWS = (392, 408)
W = 800
BIAS = 0.3  # added to the density output's bias: semi-transparent, several march rounds


def scene(kind):
    """Same construction as tests/test_realtime.small_realtime, without the
    product loader: flat params, index map and masks as eval_rt.py:52-82 builds them."""
    from diver_gb300 import scenes
    from diver_gb300.decoder import random_decoder
    from diver_gb300.ray_march import build_octree_levels
    from diver_gb300.realtime import convert

    sc = scenes.small_scene("cpu")
    dec = random_decoder(kind, 32, 2)
    dec.layers[dec.n_mlp1 - 1][1][0] += BIAS
    sd = {"voxels": sc.features}
    sd.update(dec.state_dict())
    ser = convert(sd, sc.mask.float())
    n = 64
    nv = n + 1
    inds = ser["i"].long()
    ii, rem = inds // (nv * nv), inds % (nv * nv)
    jj, kk = rem // nv, rem % nv
    masks = torch.zeros(n, n, n, dtype=torch.bool)
    mm = ser["m"].bool()
    masks[ii[mm], jj[mm], kk[mm]] = True
    vmap = torch.zeros(nv, nv, nv, dtype=torch.int32)
    vmap[ii, jj, kk] = torch.arange(inds.numel(), dtype=torch.int32)
    return sc, ser, masks, vmap, build_octree_levels(masks)


def strip_rays():
    from diver_gb300 import scenes

    c2w = scenes.sphere_cameras(1, 4.0, 3)[0]
    _, v = scenes.camera_rays(c2w, W, W, 960.0, "cpu")
    v = v.reshape(W, W, 3)[ROWS[0]:ROWS[1]].reshape(-1, 3).contiguous()
    return c2w, v


def run(kind, width, rk):
    from oracle import native as orc

    sc, ser, masks, vmap, octs = scene(kind)
    c2w, v = strip_rays()
    B = v.shape[0]
    center = ((c2w[:, 3].float() - sc.xyzmin) / sc.voxel_size).numpy().astype(np.float32)
    coords = np.zeros((8, B, 6), np.float32)
    rgba = np.zeros((B, 4), np.float32)
    fin = np.zeros(B, np.uint8)
    vn = v.numpy()
    orc.aabb(coords, vn, center, fin, rgba, octs.numpy(), 64)
    dev = torch.device("cuda")
    vmap_d = vmap.to(dev).contiguous()
    rk.upload_weight(width, ser["p"], vmap_d)
    feats = ser["f"].float().to(dev).contiguous()
    v_d = v.to(dev)
    rgba_d = torch.from_numpy(rgba).to(dev)
    fin_d = torch.from_numpy(fin).to(dev)
    first = None
    r = 0
    mask_np = masks.numpy()
    while not fin.all() and r < 3 * 64:
        orc.ray_march(coords, vn, mask_np, fin, 64)
        rk.mlp_eval(width, rgba_d, torch.from_numpy(coords).to(dev), feats, v_d, fin_d)
        rgba = rgba_d.cpu().numpy()
        fin = fin_d.cpu().numpy()
        if first is None:
            first = rgba.copy()
        r += 1
    return {f"{kind}/rgba_round1": first, f"{kind}/rgba": rgba, f"{kind}/finish": fin,
            f"{kind}/rounds": np.int32(r)}


def main():
    from oracle.ref_kernels import UNITS, RefKernels

    rk = RefKernels(list(UNITS) + ["mlp_eval32", "mlp_eval64"])
    out = {"rows": np.array(ROWS, np.int32), "width": np.int32(W), "density_bias": np.float32(BIAS)}
    out.update(run("diver32", 32, rk))
    out.update(run("diver64", 64, rk))
    dst = ROOT / "tests" / "golden" / "mlp_eval_ref.npz"
    np.savez_compressed(dst, **out)
    for k in ("diver32", "diver64"):
        print(k, "rounds", int(out[f"{k}/rounds"]), "finished", float(out[f"{k}/finish"].mean()),
              "mean alpha", float(1 - out[f"{k}/rgba"][:, 3].mean()))
    print("wrote", dst)


if __name__ == "__main__":
    main()
