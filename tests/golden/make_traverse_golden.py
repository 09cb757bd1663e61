"""Generates tests/golden/traverse_ref.npz: inputs and outputs of the
reference's own CUDA traversal kernels (ray_voxel_intersect_kernel,
masked_intersect_kernel, aabb_intersect_kernel<N>, ray_march_kernel<N>).

Run on a machine with a GB300 after `oracle.ref_kernels.build_cubins()` has
compiled the reference sources (the cubins travel in oracle/_ref/):
    python tests/golden/make_traverse_golden.py [out.npz]

Inputs are generated with numpy (seeded) and stored in the file, so the
tests never regenerate them.  Outputs are stored compacted (per-ray counts
plus concatenated rows) to keep the file small.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))


def sphere_mask(n, xyzmin, vs, count, rng, r_lo=0.15, r_hi=0.4):
    c = (np.arange(n) + 0.5) * vs + xyzmin
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    m = np.zeros((n, n, n), bool)
    for _ in range(count):
        ctr = rng.uniform(-1, 1, 3)
        r = rng.uniform(r_lo, r_hi)
        m |= (x - ctr[0]) ** 2 + (y - ctr[1]) ** 2 + (z - ctr[2]) ** 2 <= r * r
    return m


def maxpool(m, s):
    n = m.shape[0] // s
    return m.reshape(n, s, n, s, n, s).any(axis=(1, 3, 5))


def look_at(eye):
    back = eye / np.linalg.norm(eye)
    up = np.array([0.0, 0.0, 1.0])
    right = np.cross(up, back)
    right /= np.linalg.norm(right)
    return np.stack([right, np.cross(back, right), back], 1), eye


def camera(eye, H, W, focal):
    R, t = look_at(np.asarray(eye, np.float64))
    i, j = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)
    d = np.stack([(i - W / 2) / focal, -(j - H / 2) / focal, -np.ones_like(i)], -1).reshape(-1, 3)
    d = d @ R.T
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    return np.repeat(t[None], d.shape[0], 0).astype(np.float32), d.astype(np.float32)


def special_rays(rng, xyzmin, vs, n):
    lo, hi = xyzmin, xyzmin + n * vs
    O, D = [], []

    def add(o, d):
        d = np.asarray(d, np.float64)
        O.append(np.asarray(o, np.float32))
        D.append((d / np.linalg.norm(d)).astype(np.float32))

    for _ in range(32):  # origin inside the grid
        add(rng.uniform(lo, hi, 3), rng.normal(size=3))
    for ax in range(3):  # axis-aligned, from outside and from inside
        for sgn in (1, -1):
            for inside in (0, 1):
                for _ in range(2):
                    o = rng.uniform(lo, hi, 3)
                    if not inside:
                        o[ax] = lo - 0.5 if sgn > 0 else hi + 0.5
                    d = np.zeros(3)
                    d[ax] = sgn
                    add(o, d)
    for _ in range(24):  # one zero direction component
        d = rng.normal(size=3)
        d[rng.integers(3)] = 0.0
        o = -d / np.linalg.norm(d) * 3.0 + rng.uniform(-0.3, 0.3, 3)
        add(o, d)
    for _ in range(32):  # exact grid points, diagonal directions (ties between axes)
        k = rng.integers(0, n + 1, 3)
        o = xyzmin + vs * k
        d = rng.choice([-1.0, 1.0], 3) * np.array([1.0, 1.0, rng.choice([1.0, 0.5])])
        add(o, d)
    for _ in range(16):  # grazing the far faces
        o = rng.uniform(lo, hi, 3)
        ax = rng.integers(3)
        o[ax] = hi
        d = rng.normal(size=3)
        d[ax] = 0.0
        add(o - d * 3, d)
    for _ in range(16):  # starting on a face
        o = rng.uniform(lo, hi, 3)
        ax = rng.integers(3)
        o[ax] = lo if rng.integers(2) else hi
        add(o, rng.normal(size=3))
    for _ in range(16):  # misses
        o = rng.normal(size=3)
        o = o / np.linalg.norm(o) * 4.0
        t = np.cross(o, rng.normal(size=3))
        add(o, t)
    while len(O) < 256:  # random chords
        a = rng.normal(size=3)
        a = a / np.linalg.norm(a) * 4.0
        b = rng.uniform(lo, hi, 3)
        add(a, b - a)
    return np.stack(O), np.stack(D)


def compact(rows, num):
    rows = rows.cpu().numpy()
    num = num.cpu().numpy()
    return np.concatenate([rows[b, :num[b]] for b in range(len(num))], 0), num


def main(out: Path):
    import torch

    from oracle.ref_kernels import RefKernels

    rng = np.random.default_rng(20240611)
    ref = RefKernels()
    data = {}

    # --- dense / masked walks, N = 64 ---------------------------------------
    n, xyzmin, vs = 64, -1.5, 3.0 / 64
    mask64 = sphere_mask(n, xyzmin, vs, 8, rng)
    o_cam, d_cam = camera(np.array([2.3, -2.9, 1.6]), 200, 200, 240.0)
    pick = rng.choice(o_cam.shape[0], 768, replace=False)
    o_sp, d_sp = special_rays(rng, xyzmin, vs, n)
    o = np.concatenate([o_cam[pick], o_sp]).astype(np.float32)
    d = np.concatenate([d_cam[pick], d_sp]).astype(np.float32)
    data.update(walk_o=o, walk_v=d, walk_n=n, walk_xyzmin=xyzmin, walk_vs=vs, mask64=np.packbits(mask64))
    ot, dt = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    inter, num, tns = ref.dense(ot, dt, xyzmin, -xyzmin, float(n), vs)
    data["dense_row0"] = inter[:, 0].cpu().numpy()
    data["dense_pts"], data["dense_num"] = compact(inter, num)
    data["dense_tns"], _ = compact(tns, num)
    for tag, scale in (("m1", 1.0), ("m05", 0.5), ("m025", 0.25)):
        m = mask64 if scale == 1.0 else maxpool(mask64, int(round(1 / scale)))
        mt = torch.from_numpy(m.copy()).cuda()
        inter, num, tns = ref.masked(ot, dt, xyzmin, -xyzmin, float(n), vs, mt, scale)
        data[f"masked_{tag}_seg"], data[f"masked_{tag}_num"] = compact(inter, num)
        data[f"masked_{tag}_tns"], _ = compact(tns, num)

    # --- octree first hit + 8-hit march, N = 128 and 256 ---------------------
    for N, side in ((128, 32), (256, 16)):
        vsN = 3.0 / N
        m = sphere_mask(N, -1.5, vsN, 8, rng)
        octs = np.concatenate([maxpool(m, s).reshape(-1) for s in (64, 16, 4)])
        eye = np.array([3.1, 2.2, -1.3]) if N == 128 else np.array([-2.5, 2.9, 1.1])
        o_c, d_c = camera(eye, side, side, 1.2 * side)
        center = ((eye.astype(np.float32) - np.float32(-1.5)) / np.float32(vsN)).astype(np.float32)
        B = d_c.shape[0]
        vt = torch.from_numpy(d_c).cuda().contiguous()
        coords = torch.zeros(8, B, 6, device="cuda")
        rgba = torch.zeros(B, 4, device="cuda")
        finish = torch.zeros(B, dtype=torch.bool, device="cuda")
        ref.aabb(coords, vt, torch.from_numpy(center).cuda(), finish, rgba, torch.from_numpy(octs).cuda(), N)
        data[f"oct{N}_mask"] = np.packbits(m)
        data[f"oct{N}_v"] = d_c
        data[f"oct{N}_center"] = center
        data[f"oct{N}_resume"] = coords[7, :, 3:].cpu().numpy()
        data[f"oct{N}_finish"] = finish.cpu().numpy()
        data[f"oct{N}_rgba"] = rgba.cpu().numpy()
        hits = [[] for _ in range(B)]
        mt = torch.from_numpy(m.copy()).cuda()
        rounds = 0
        while not bool(finish.all()) and rounds < 4 * N:
            active = (~finish).cpu().numpy()
            ref.march(coords, vt, mt, finish, N)
            c = coords.cpu().numpy()
            for b in np.nonzero(active)[0]:
                for h in range(8):
                    if c[h, b, 0] < 0:
                        break
                    hits[b].append(c[h, b])
            # the decoder's finishing rule without transmittance (mlp_eval.cu:67-70)
            finish |= (coords[:, :, 0] < 0).any(0)
            rounds += 1
        data[f"oct{N}_hit_num"] = np.array([len(h) for h in hits], np.int32)
        data[f"oct{N}_hits"] = np.concatenate([np.asarray(h, np.float32).reshape(-1, 6) for h in hits], 0)
        data[f"oct{N}_rounds"] = rounds
    np.savez_compressed(out, **data)
    print(f"wrote {out} ({out.stat().st_size} bytes)")


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).with_name("traverse_ref.npz"))
