"""Generates tests/golden/implicit_ref.npz from the DIVeR reference's own
implicit stage (utils/integrator.py:integrate_mlp over model/mlps.py's
ImplicitMLP, CPU), where the reference tree is present:
    python tests/golden/make_implicit_golden.py [reference_root]

Segments come from the C oracle's masked walk (pinned to the reference's
traversal kernels) on a 16^3 grid; the MLP is small (depth 4, width 64, a skip
at layer 2, 2 PE bands, 32 output channels) with seeded weights.  Stored: the
weights, the segments, the integrated features and the gradients of
sum(features * G), G = cos(0.37 k) over the flattened features, with respect
to every MLP parameter.
"""
from __future__ import annotations

import importlib.util
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.dont_write_bytecode = True
sys.path.insert(0, str(ROOT))

N, C, D, W, SKIPS, ENC = 16, 32, 4, 64, [2], 2


def load(path, name):
    spec = importlib.util.spec_from_file_location(name, path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main(ref_root: Path):
    import torch

    from oracle import native as orc

    mlps = load(ref_root / "model" / "mlps.py", "ref_mlps")
    integ = load(ref_root / "utils" / "integrator.py", "ref_integrator")
    torch.manual_seed(0)
    mlp = mlps.ImplicitMLP(D, W, SKIPS, C, ENC)
    rng = np.random.default_rng(7)
    vs, xyzmin = 3.0 / N, -1.5
    mask = rng.random((N, N, N)) < 0.5
    B = 150
    o = np.tile(np.array([[0.2, -3.5, 0.4]], np.float32), (B, 1))
    d = rng.normal(size=(B, 3)).astype(np.float32) * np.float32(0.25) + np.array([0.0, 1.0, 0.0], np.float32)
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    inter, num, _ = orc.masked_walk(o, d.astype(np.float32), xyzmin, N, vs, mask, 1.0)
    seg = orc.csr_from_padded(inter, num).astype(np.float32)
    ci, co = torch.from_numpy(seg[:, :3]), torch.from_numpy(seg[:, 3:])
    feat = integ.integrate_mlp(mlp, N + 1, C, ci, co)
    G = torch.cos(torch.arange(feat.numel(), dtype=torch.float32) * 0.37).reshape(feat.shape)
    (feat * G).sum().backward()
    out = {"seg": seg, "feature": feat.detach().numpy(),
           "meta": np.array([N, C, D, W, ENC] + SKIPS, np.int64)}
    for name, p in mlp.named_parameters():
        out["w:" + name] = p.detach().numpy()
        out["g:" + name] = p.grad.numpy()
    np.savez_compressed(HERE / "implicit_ref.npz", **out)
    print(f"implicit_ref.npz: {seg.shape[0]} segments")


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("DIVER_REFERENCE"):
        sys.exit("usage: make_implicit_golden.py <reference tree> (or set DIVER_REFERENCE)")
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(os.environ["DIVER_REFERENCE"]))
