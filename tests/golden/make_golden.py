"""Generates tests/golden/decode_ref.npz and tests/golden/convert_ref.npz from
the DIVeR reference's own Python code (CPU), where the reference tree is
present:
    python tests/golden/make_golden.py [reference_root]

decode_ref.npz   utils.integrator.integrate on traversal segments, and the
                 reference DIVeR module's forward + render + training loss and
                 its autograd gradients (model/diver.py, train.py:84-113) for
                 DIVeR32 and DIVeR64 decoders.  The reference's CUDA traversal
                 extension is replaced by the C oracle (oracle/dda.c), which
                 the traversal fixtures pin bit-exactly to the reference's
                 kernels.
convert_ref.npz  the serialized real-time model written by the reference's
                 convert.py (run as a script on a synthetic checkpoint) for
                 DIVeR32 (voxel_dim 32) and DIVeR64 (voxel_dim 64).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile
import types
from argparse import Namespace
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.dont_write_bytecode = True
sys.path.insert(0, str(ROOT))

N, C = 12, 32
XYZMIN, VS = -1.5, 3.0 / 12


def scene(rng):
    import torch

    vox = rng.normal(0, 0.05, (N + 1, N + 1, N + 1, C)).astype(np.float32)
    cen = (np.arange(N) + 0.5) * VS + XYZMIN
    z, y, x = np.meshgrid(cen, cen, cen, indexing="ij")
    mask = np.zeros((N, N, N), bool)
    for _ in range(4):
        c = rng.uniform(-0.8, 0.8, 3)
        r = rng.uniform(0.4, 0.8)
        mask |= (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 <= r * r
    return torch.from_numpy(vox), torch.from_numpy(mask)


def rays(rng, count):
    o = rng.normal(size=(count, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * 3.5
    tgt = rng.uniform(-0.9, 0.9, (count, 3))
    d = tgt - o
    d = d / np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def install_traversal_stub():
    """utils.ray_voxel_intersection backed by the C oracle, returning what the
    reference's autograd Functions return (utils/ray_voxel_intersection/__init__.py:40-43,75-79)."""
    import torch

    from oracle import native as orc

    stub = types.ModuleType("utils.ray_voxel_intersection")

    def masked_intersect(o, v, xyzmin, xyzmax, voxel_num, voxel_size, mask, mask_scale):
        inter, num, tns = orc.masked_walk(o.numpy(), v.numpy(), xyzmin, voxel_num, voxel_size, mask.numpy(), mask_scale)
        i, m, t = orc.trim(inter, num, tns)
        return torch.from_numpy(i.copy()), torch.from_numpy(m.copy()), torch.from_numpy(t.copy())

    def ray_voxel_intersect(o, v, xyzmin, xyzmax, voxel_num, voxel_size):
        inter, num, tns = orc.dense_walk(o.numpy(), v.numpy(), xyzmin, voxel_num, voxel_size)
        i, m, t = orc.trim(inter, num, tns)
        return torch.from_numpy(i.copy()), torch.from_numpy(m.copy()), torch.from_numpy(t.copy())

    stub.masked_intersect = masked_intersect
    stub.ray_voxel_intersect = ray_voxel_intersect
    sys.modules["utils.ray_voxel_intersection"] = stub


def hparams(kind):
    mp, mv = ([32, 2, 33], [32, 1]) if kind == "diver32" else ([64, 1, 65], [64, 1])
    return Namespace(voxel_num=N, voxel_dim=C, grid_size=N * VS, mask_scale=1.0, white_back=True, implicit=False,
                     fine=1, mlp_point=mp, mlp_view=mv, dir_encode=4)


def make_decode(ref_root: Path, out: Path):
    import torch

    sys.path.insert(0, str(ref_root))
    install_traversal_stub()
    from model.diver import DIVeR
    from utils.integrator import integrate

    from oracle import native as orc

    rng = np.random.default_rng(1234)
    vox, mask = scene(rng)
    o, d = rays(rng, 160)
    data = {"voxels": vox.numpy(), "mask": mask.numpy(), "o": o, "d": d}
    # integrate on the masked segments of all rays
    inter, num, _ = orc.masked_walk(o, d, XYZMIN, N, VS, mask.numpy(), 1.0)
    seg = orc.csr_from_padded(inter, num)
    data["seg"] = seg
    data["feature"] = integrate(vox, torch.from_numpy(seg[:, :3]), torch.from_numpy(seg[:, 3:])).numpy()
    # DIVeR forward/render/loss/backward
    hit = num > 0
    o_h, d_h = o[hit][:96], d[hit][:96]
    target = rng.uniform(0, 1, (o_h.shape[0], 3)).astype(np.float32)
    data.update(o_hit=o_h, d_hit=d_h, target=target)
    for kind, seed in (("diver32", 7), ("diver64", 8)):
        torch.manual_seed(seed)
        model = DIVeR(hparams(kind))
        with torch.no_grad():
            model.voxels.copy_(vox)
            model.voxel_mask.copy_(mask)
            # a positive density bias so both the density and the colour
            # branches carry gradient (default init can leave sigma <= 0)
            model.mlp1[-1].bias[0] += 0.6
        color, sigma, m, ts = model(torch.from_numpy(o_h), torch.from_numpy(d_h))
        rgb, weight = model.render(color, sigma, m)
        loss_c = torch.nn.functional.mse_loss(rgb, torch.from_numpy(target))
        loss = loss_c + 1e-5 * torch.log(1 + sigma ** 2 / 0.5).mean()
        loss.backward()
        sd = {k: v.detach().numpy() for k, v in model.state_dict().items() if k.startswith("mlp")}
        for k, v in sd.items():
            data[f"{kind}/{k}"] = v
        data[f"{kind}/rgb"] = rgb.detach().numpy()
        data[f"{kind}/sigma"] = sigma.detach().numpy()
        data[f"{kind}/color"] = color.detach().numpy()
        data[f"{kind}/weight"] = weight.detach().numpy()
        data[f"{kind}/mask"] = m.numpy()
        data[f"{kind}/ts"] = ts.numpy()
        data[f"{kind}/loss"] = np.float32(loss.item())
        gv = model.voxels.grad.numpy().reshape(-1, C)
        rows = np.nonzero(np.abs(gv).sum(1) > 0)[0]
        data[f"{kind}/grad_voxels_rows"] = rows.astype(np.int64)
        data[f"{kind}/grad_voxels"] = gv[rows]
        for name, p in model.named_parameters():
            if name.startswith("mlp"):
                data[f"{kind}/grad/{name}"] = p.grad.numpy()
    np.savez_compressed(out, **data)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


def make_convert(ref_root: Path, out: Path):
    import torch

    from diver_gb300.decoder import random_decoder

    rng = np.random.default_rng(99)
    data = {}
    for kind, vdim in (("diver32", 32), ("diver64", 64)):
        dec = random_decoder(kind, vdim, 5)
        vox = torch.from_numpy(rng.normal(0, 0.05, (N + 1, N + 1, N + 1, vdim)).astype(np.float32))
        alpha = torch.from_numpy(rng.uniform(0, 0.02, (N, N, N)).astype(np.float32))
        sd = {"model.voxels": vox}
        sd.update({f"model.{k}": v for k, v in dec.state_dict().items()})
        with tempfile.TemporaryDirectory() as tmp:
            tmp = Path(tmp)
            torch.save({"state_dict": sd}, tmp / "last.ckpt")
            torch.save(alpha, tmp / "alpha_map.pt")
            env = dict(os.environ, PYTHONDONTWRITEBYTECODE="1")
            subprocess.run([sys.executable, str(ref_root / "convert.py"), "--checkpoint_path", str(tmp / "last.ckpt"),
                            "--serialize", "1"], check=True, cwd=tmp, env=env)
            ser = torch.load(tmp / "serialize.pth", map_location="cpu")
        data[f"{kind}/voxels"] = vox.numpy()
        data[f"{kind}/alpha"] = alpha.numpy()
        for k, v in dec.state_dict().items():
            data[f"{kind}/{k}"] = v.numpy()
        for k in ("f", "i", "m", "p"):
            data[f"{kind}/ser_{k}"] = ser[k].numpy()
    np.savez_compressed(out, **data)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("DIVER_REFERENCE"):
        sys.exit("usage: make_golden.py <reference tree> (or set DIVER_REFERENCE)")
    ref = Path(sys.argv[1]) if len(sys.argv) > 1 else Path(os.environ["DIVER_REFERENCE"])
    make_decode(ref, HERE / "decode_ref.npz")
    make_convert(ref, HERE / "convert_ref.npz")
