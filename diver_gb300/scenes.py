"""Seeded synthetic scenes standing in for the reference's datasets.

NeRF-synthetic, Tanks&Temples and BlendedMVS are not available, so scenes are
generated with the shapes, sizes and value distributions of the reference's
configurations (configs/nerf_synthetic_fine*.py, configs/tnt_fine.py):

  small   64^3 x 32, bbox [-1.5,1.5]^3, 8-sphere occupancy, one 200x200 view
  train   256^3 x 32 (257^3 corners), grid_size 2.8, 16-blob occupancy (~60%),
          100 cameras at 800x800, batches of rays that hit occupied voxels
  rt64    the same 256^3 scene with 64-channel features and a DIVeR64 decoder,
          200 spiral cameras at 800x800

Seeds: features 0, occupancy 1, decoder 2, cameras 3, batches/targets 4;
scene k of a multi-scene set adds 100*k.  Cameras follow the reference's
pinhole convention (utils/dataset/ray_utils.py:5-55): pixel centres at +0.5,
x right, y up, looking down -z, unit directions.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import torch

from .decoder import Decoder, random_decoder


@dataclass
class Scene:
    name: str
    voxel_num: int
    channels: int
    xyzmin: float | tuple
    voxel_size: float
    features: torch.Tensor  # [N+1, N+1, N+1, C] float32, [z][y][x][c]
    mask: torch.Tensor  # [M, M, M] bool, [z][y][x]
    mask_scale: float
    decoder: Decoder
    white_back: bool = True

    @property
    def xyzmax(self) -> float:
        return self.xyzmin + self.voxel_num * self.voxel_size if not isinstance(self.xyzmin, tuple) else None

    @property
    def dims(self):
        return (self.features.shape[2] - 1, self.features.shape[1] - 1, self.features.shape[0] - 1)

    def to(self, device) -> "Scene":
        return Scene(self.name, self.voxel_num, self.channels, self.xyzmin, self.voxel_size,
                     self.features.to(device), self.mask.to(device), self.mask_scale,
                     self.decoder.to(device), self.white_back)


def _gen(seed: int, device) -> torch.Generator:
    return torch.Generator(device=device).manual_seed(seed)


def voxel_centres(n: int, xyzmin: float, vs: float, device) -> torch.Tensor:
    c = xyzmin + (torch.arange(n, device=device, dtype=torch.float32) + 0.5) * vs
    z, y, x = torch.meshgrid(c, c, c, indexing="ij")
    return torch.stack([x, y, z], -1)  # [z][y][x][xyz]


def sphere_union_mask(n, xyzmin, vs, count, seed, device, r_lo=0.15, r_hi=0.4, span=1.0):
    g = _gen(seed, "cpu")
    centres = (torch.rand(count, 3, generator=g) * 2 - 1) * span
    radii = r_lo + torch.rand(count, generator=g) * (r_hi - r_lo)
    p = voxel_centres(n, xyzmin, vs, device)
    m = torch.zeros(n, n, n, dtype=torch.bool, device=device)
    for c, r in zip(centres.to(device), radii.to(device)):
        m |= ((p - c) ** 2).sum(-1) <= r * r
    return m


def blob_mask(n, xyzmin, vs, count, seed, device, occupancy=0.6):
    """Sum of Gaussian blobs thresholded at 0.5, scaled so ~`occupancy` of voxels are set."""
    g = _gen(seed, "cpu")
    centres = (torch.rand(count, 3, generator=g) * 2 - 1) * 0.8
    sig = 0.25 + torch.rand(count, generator=g) * 0.35
    amp = 0.5 + torch.rand(count, generator=g)
    p = voxel_centres(n, xyzmin, vs, device)
    f = torch.zeros(n, n, n, device=device)
    for c, s, a in zip(centres.to(device), sig.to(device), amp.to(device)):
        f += a * torch.exp(-((p - c) ** 2).sum(-1) / (2 * s * s))
    sub = f[::4, ::4, ::4].reshape(-1).float().cpu()
    q = torch.kthvalue(sub, max(1, int(round((1 - occupancy) * sub.numel())))).values.item()
    return (f * (0.5 / max(q, 1e-12))) > 0.5


def features(n_vert: int, channels: int, std: float, seed: int, device) -> torch.Tensor:
    g = _gen(seed, device)
    return torch.randn(n_vert, n_vert, n_vert, channels, generator=g, device=device, dtype=torch.float32) * std


# --- cameras ------------------------------------------------------------------

def pixel_directions(H: int, W: int, focal: float, device="cpu") -> torch.Tensor:
    """Camera-space directions, reference utils/dataset/ray_utils.py:5-29."""
    xs = torch.linspace(0.5, W - 1 + 0.5, W, device=device)
    ys = torch.linspace(0.5, H - 1 + 0.5, H, device=device)
    j, i = torch.meshgrid(ys, xs, indexing="ij")
    return torch.stack([(i - W / 2) / focal, -(j - H / 2) / focal, -torch.ones_like(i)], -1)


def look_at(eye: torch.Tensor) -> torch.Tensor:
    """3x4 camera-to-world matrix of a camera at `eye` looking at the origin, z up."""
    eye = eye.float()
    back = eye / eye.norm()
    up = torch.tensor([0.0, 0.0, 1.0])
    if torch.cross(up, back, dim=0).norm() < 1e-6:
        up = torch.tensor([0.0, 1.0, 0.0])
    right = torch.cross(up, back, dim=0)
    right = right / right.norm()
    cam_up = torch.cross(back, right, dim=0)
    return torch.stack([right, cam_up, back, eye], 1)


def camera_rays(c2w: torch.Tensor, H: int, W: int, focal: float, device="cpu"):
    """(rays_o [H*W,3], rays_d [H*W,3]) as reference utils/dataset/ray_utils.py:32-55."""
    dirs = pixel_directions(H, W, focal, device)
    c2w = c2w.to(device)
    d = dirs @ c2w[:, :3].t()
    d = d / torch.norm(d, dim=-1, keepdim=True)
    o = c2w[:, 3].expand(d.shape)
    return o.reshape(-1, 3).contiguous(), d.reshape(-1, 3).contiguous()


def camera_rays_device(c2w: torch.Tensor, H: int, W: int, focal: float, device="cuda", first: int = 0,
                       count: int | None = None):
    """camera_rays generated on the device in one kernel (dv_camera_rays), for
    pixels [first, first + count) of the row-major image (all by default)."""
    import ctypes

    from . import _native as N

    n = H * W - first if count is None else int(count)
    m = (ctypes.c_float * 12)(*[float(x) for x in c2w.float().reshape(-1).tolist()])
    o = torch.empty(n, 3, device=device)
    d = torch.empty(n, 3, device=device)
    N.call("dv_camera_rays", H, W, float(focal), ctypes.addressof(m), int(first), n, N.ptr(o), N.ptr(d),
           N.stream(torch.device(device)))
    return o, d


def sphere_cameras(count: int, radius: float, seed: int) -> list[torch.Tensor]:
    g = _gen(seed, "cpu")
    v = torch.randn(count, 3, generator=g)
    v = v / v.norm(dim=-1, keepdim=True) * radius
    return [look_at(e) for e in v]


def spiral_cameras(count: int, radius: float, elev_lo=-30.0, elev_hi=30.0, turns=2.0) -> list[torch.Tensor]:
    cams = []
    for k in range(count):
        f = k / max(count - 1, 1)
        az = 2 * math.pi * turns * f
        el = math.radians(elev_lo + (elev_hi - elev_lo) * f)
        eye = torch.tensor([radius * math.cos(el) * math.cos(az), radius * math.cos(el) * math.sin(az), radius * math.sin(el)])
        cams.append(look_at(eye))
    return cams


# --- configurations -------------------------------------------------------------

def small_scene(device="cpu", seed_offset: int = 0) -> Scene:
    """64^3 x 32, bbox [-1.5,1.5]^3, union of 8 spheres, DIVeR32."""
    n, vs, xyzmin = 64, 3.0 / 64, -1.5
    s = seed_offset
    return Scene("small", n, 32, xyzmin, vs,
                 features(n + 1, 32, 0.05, 0 + s, device),
                 sphere_union_mask(n, xyzmin, vs, 8, 1 + s, device),
                 1.0, random_decoder("diver32", 32, 2 + s).to(device))


def small_view(device="cpu", seed_offset: int = 0):
    """One 200x200 camera on a radius-4 sphere, focal 240."""
    c2w = sphere_cameras(1, 4.0, 3 + seed_offset)[0]
    return camera_rays(c2w, 200, 200, 240.0, device)


def grid_scene(n=256, channels=32, kind="diver32", device="cpu", seed_offset: int = 0, occupancy=0.6,
               grid_size=2.8) -> Scene:
    """n^3 grid over [-grid_size/2, grid_size/2]^3, 16-blob occupancy (~60%)."""
    vs = grid_size / n
    xyzmin = -grid_size / 2
    s = seed_offset
    std = 0.02
    return Scene(f"grid{n}x{channels}", n, channels, xyzmin, vs,
                 features(n + 1, channels, std, 0 + s, device),
                 blob_mask(n, xyzmin, vs, 16, 1 + s, device, occupancy),
                 1.0, random_decoder(kind, channels, 2 + s).to(device))


def ellipsoid_mask(dims, xyzmin, vs, count, seed, device, occupancy=0.25):
    """Union of `count` axis-aligned ellipsoids (centres in the box, semi-axes
    U(0.05, 0.5)), uniformly rescaled so ~`occupancy` of the voxels are set."""
    nx, ny, nz = dims
    g = _gen(seed, "cpu")
    lo = torch.tensor(xyzmin)
    hi = lo + torch.tensor([nx, ny, nz], dtype=torch.float32) * vs
    centres = lo + torch.rand(count, 3, generator=g) * (hi - lo)
    axes = 0.05 + torch.rand(count, 3, generator=g) * 0.45
    cx = xyzmin[0] + (torch.arange(nx, device=device) + 0.5) * vs
    cy = xyzmin[1] + (torch.arange(ny, device=device) + 0.5) * vs
    cz = xyzmin[2] + (torch.arange(nz, device=device) + 0.5) * vs
    z, y, x = torch.meshgrid(cz, cy, cx, indexing="ij")

    def build(scale):
        m = torch.zeros(nz, ny, nx, dtype=torch.bool, device=device)
        for c, a in zip(centres.to(device), (axes * scale).to(device)):
            m |= ((x - c[0]) / a[0]) ** 2 + ((y - c[1]) / a[1]) ** 2 + ((z - c[2]) / a[2]) ** 2 <= 1.0
        return m

    s_lo, s_hi = 0.2, 4.0
    for _ in range(12):  # bisection on a common scale of the semi-axes
        mid = 0.5 * (s_lo + s_hi)
        if build(mid).float().mean().item() < occupancy:
            s_lo = mid
        else:
            s_hi = mid
    return build(0.5 * (s_lo + s_hi))


def wide_scene(device="cpu", dims=(320, 320, 160), seed_offset: int = 0) -> Scene:
    """bbox [-1,1] x [-1,1] x [-0.5,0.5], voxel 1/160, 24-ellipsoid occupancy (~25%), DIVeR32."""
    nx, ny, nz = dims
    vs = 1.0 / 160
    xyzmin = (-1.0, -1.0, -0.5)
    s = seed_offset
    g = _gen(0 + s, device)
    feats = torch.randn(nz + 1, ny + 1, nx + 1, 32, generator=g, device=device, dtype=torch.float32) * 0.02
    return Scene("wide", nx, 32, xyzmin, vs, feats, ellipsoid_mask(dims, xyzmin, vs, 24, 1 + s, device), 1.0,
                 random_decoder("diver32", 32, 2 + s).to(device))


def ellipse_cameras(count=150, a=3.0, b=2.0, z=0.8) -> list[torch.Tensor]:
    cams = []
    for k in range(count):
        th = 2 * math.pi * k / count
        cams.append(look_at(torch.tensor([a * math.cos(th), b * math.sin(th), z])))
    return cams


def training_batches(scene: Scene, count: int, batch: int, device, seed: int = 4, cameras: int = 100,
                     size: int = 800, focal: float = 960.0, count_fn=None):
    """`count` batches (o, d, target) of `batch` rays drawn from `cameras`
    sphere cameras (radius 4) at size x size pixels, kept only where the ray
    crosses at least one occupied voxel of the scene (cubic grids); targets
    U[0, 1].  count_fn(o, d) -> per-ray counts of occupied segments (int
    tensor on `device`); by default the CUDA masked walk (dv_masked_count)."""
    if count_fn is None:
        from . import _native as N

        m8 = scene.mask.view(torch.uint8)

        def count_fn(o, d):
            num = torch.empty(d.shape[0], dtype=torch.int32, device=device)
            N.call("dv_masked_count", d.shape[0], scene.xyzmin, float(scene.voxel_num), scene.voxel_size, 1.0,
                   N.ptr(o), N.ptr(d), N.ptr(m8), N.ptr(num), None, None, N.stream(device))
            return num

    cams = sphere_cameras(cameras, 4.0, 3)
    dirs_cam = pixel_directions(size, size, focal, device).reshape(-1, 3)
    g = torch.Generator(device=device).manual_seed(seed)
    gc = torch.Generator().manual_seed(seed)
    out = []
    while len(out) < count:
        c2w = cams[int(torch.randint(0, cameras, (1,), generator=gc))].to(device)
        pick = torch.randint(0, dirs_cam.shape[0], (3 * batch,), generator=g, device=device)
        d = dirs_cam[pick] @ c2w[:, :3].t()
        d = (d / d.norm(dim=-1, keepdim=True)).contiguous()
        o = c2w[:, 3].expand(d.shape).contiguous()
        num = count_fn(o, d)
        keep = torch.nonzero(num > 0)[:, 0]
        if keep.numel() < batch:
            continue
        keep = keep[:batch]
        tgt = torch.rand(batch, 3, generator=g, device=device)
        out.append((o[keep].contiguous(), d[keep].contiguous(), tgt))
    return out


def reference_octree(mask: torch.Tensor) -> torch.Tensor:
    from .ray_march import build_octree_levels

    return build_octree_levels(mask)
