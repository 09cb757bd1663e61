"""ORACLE — test infrastructure only.  The reference's own CUDA traversal
kernels, compiled from the reference sources in place and run through the
CUDA driver API, to produce the traversal fixtures in tests/golden/.

  build_cubins(root)  nvcc -cubin of utils/ray_voxel_intersection/src/
                  ray_voxel_intersect.cu and utils/ray_march/src/ray_march.cu
                  with the reference's default nvcc flags (no fast math,
                  default -fmad=true) into oracle/_ref/*.cubin.  Needs the
                  reference tree; oracle/ref_shim/ supplies a stand-in for its
                  torch-dependent cuda_utils.h.
  build_mlp_eval_cubins(root)
                  the reference's real-time decoder kernels
                  (utils/mlp_evaluation{,64}/src/mlp_eval.cu) for the same
                  checker role.  They use a texture reference (removed in
                  CUDA 12), so the recipe patches a temporary copy before
                  compiling it: the voxel index map becomes a plain int array
                  read with the texture's clamp addressing
                  (`c_voxel_map_ptr`, `c_voxel_map_n`), and the host wrappers
                  (texture binding, ATen streams) are left out.  The kernel's
                  arithmetic (__expf, __sinf/__cosf, the weight polynomial,
                  the skip and termination thresholds) is untouched.  Only the
                  cubin is kept, in oracle/_ref/.
  RefKernels      loads the cubins (libcuda via ctypes) and launches
                  ray_voxel_intersect_kernel, masked_intersect_kernel,
                  aabb_intersect_kernel<N>, ray_march_kernel<N> and the
                  patched mlp_eval_kernel with the launch shapes of the
                  reference wrappers.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
UNITS = {
    "ray_voxel_intersect": "utils/ray_voxel_intersection/src/ray_voxel_intersect.cu",
    "ray_march": "utils/ray_march/src/ray_march.cu",
}


def reference_root(root: str | os.PathLike | None = None) -> Path | None:
    """The reference source tree: `root`, else $DIVER_REFERENCE, else None."""
    r = root if root is not None else os.environ.get("DIVER_REFERENCE")
    return Path(r) if r else None


def build_cubins(root: str | os.PathLike | None = None, force: bool = False) -> list[Path]:
    """Compiles the reference kernels when the reference sources are present
    (tree `root` or $DIVER_REFERENCE)."""
    out = []
    ref = reference_root(root)
    if ref is None:
        return out
    for name, rel in UNITS.items():
        src = ref / rel
        dst = OUT / f"{name}.cubin"
        if not src.exists():
            continue
        if dst.exists() and not force and dst.stat().st_mtime >= src.stat().st_mtime:
            out.append(dst)
            continue
        OUT.mkdir(parents=True, exist_ok=True)
        inc = src.parent.parent / "include"
        cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
               "-I", str(HERE / "ref_shim"), "-I", str(inc), str(src), "-o", str(dst)]
        r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError(f"reference cubin build failed for {rel}:\n{r.stdout.decode(errors='replace')}")
        out.append(dst)
    return out


MLP_UNITS = {
    "mlp_eval32": "utils/mlp_evaluation/src/mlp_eval.cu",
    "mlp_eval64": "utils/mlp_evaluation64/src/mlp_eval.cu",
}
# The texture reference of the voxel index map becomes a plain device array
# with the texture's addressing: unnormalised integer coordinates, point
# sampling, every coordinate clamped to [0, n - 1].
_MAP_DECL = """__device__ const int* c_voxel_map_ptr;  // index map [n][n][n], x fastest
__device__ int c_voxel_map_n;
__device__ __forceinline__ int c_voxel_map_at(int x, int y, int z) {
  const int m = c_voxel_map_n - 1;
  x = min(max(x, 0), m);
  y = min(max(y, 0), m);
  z = min(max(z, 0), m);
  return c_voxel_map_ptr[((long long)z * c_voxel_map_n + y) * c_voxel_map_n + x];
}
"""


def patch_mlp_eval(src: str) -> str:
    """The reference mlp_eval.cu with its texture reference replaced by a plain
    array (see the module docstring) and its host wrappers removed."""
    import re

    decl = re.search(r"^static texture\s*<int,\s*3,\s*cudaReadModeElementType>\s*c_voxel_map;.*$", src, re.M)
    if decl is None or "tex3D(c_voxel_map," not in src or "void mlp_eval_wrapper(" not in src:
        raise RuntimeError("unexpected mlp_eval.cu layout: the patch anchors are missing")
    src = src[:decl.start()] + _MAP_DECL + src[decl.end():]
    src = src.replace("tex3D(c_voxel_map,", "c_voxel_map_at(")
    return src[:src.index("void mlp_eval_wrapper(")]


def build_mlp_eval_cubins(root: str | os.PathLike | None = None, force: bool = False) -> list[Path]:
    """Patched reference real-time decoder kernels -> oracle/_ref/mlp_eval{32,64}.cubin
    (only where the reference sources are present)."""
    import tempfile

    out = []
    ref = reference_root(root)
    if ref is None:
        return out
    for name, rel in MLP_UNITS.items():
        src = ref / rel
        dst = OUT / f"{name}.cubin"
        if not src.exists():
            continue
        if dst.exists() and not force and dst.stat().st_mtime >= max(src.stat().st_mtime, Path(__file__).stat().st_mtime):
            out.append(dst)
            continue
        OUT.mkdir(parents=True, exist_ok=True)
        with tempfile.TemporaryDirectory() as tmp:
            patched = Path(tmp) / "mlp_eval_patched.cu"
            patched.write_text(patch_mlp_eval(src.read_text()))
            inc = src.parent.parent / "include"
            cmd = ["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                   "-I", str(HERE / "ref_shim"), "-I", str(inc), str(patched), "-o", str(dst)]
            r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
        if r.returncode != 0:
            raise RuntimeError(f"patched reference cubin build failed for {rel}:\n{r.stdout.decode(errors='replace')}")
        out.append(dst)
    return out


class _Driver:
    def __init__(self):
        self.cu = C.CDLL("libcuda.so.1")

    def check(self, res, what):
        if res != 0:
            raise RuntimeError(f"{what} failed with CUresult {res}")


class RefKernels:
    """The reference traversal kernels, launched on torch's current stream."""

    def __init__(self, units=None):
        import torch

        torch.zeros(1, device="cuda")  # make the primary context current
        self.d = _Driver()
        self.mods = {}
        self.funcs = {}
        for name in (units or UNITS):
            path = OUT / f"{name}.cubin"
            if not path.exists():
                raise FileNotFoundError(f"{path} missing: build it with oracle.ref_kernels.build_cubins() where the reference sources are present")
            mod = C.c_void_p()
            self.d.check(self.d.cu.cuModuleLoad(C.byref(mod), str(path).encode()), f"cuModuleLoad({path.name})")
            self.mods[name] = mod
            cnt = C.c_uint()
            self.d.check(self.d.cu.cuModuleGetFunctionCount(C.byref(cnt), mod), "cuModuleGetFunctionCount")
            arr = (C.c_void_p * cnt.value)()
            self.d.check(self.d.cu.cuModuleEnumerateFunctions(arr, cnt, mod), "cuModuleEnumerateFunctions")
            for f in arr:
                nm = C.c_char_p()
                self.d.check(self.d.cu.cuFuncGetName(C.byref(nm), C.c_void_p(f)), "cuFuncGetName")
                self.funcs[(name, nm.value.decode())] = C.c_void_p(f)

    def _func(self, needle: str, extra: str = "", unit: str | None = None):
        for (u, k), f in self.funcs.items():
            if needle in k and extra in k and (unit is None or u == unit):
                return f
        raise KeyError(f"kernel {needle} {extra} not in {list(self.funcs)}")

    def _set_global(self, unit: str, name: str, data: bytes):
        g = C.c_void_p()
        size = C.c_size_t()
        self.d.check(self.d.cu.cuModuleGetGlobal_v2(C.byref(g), C.byref(size), self.mods[unit], name.encode()),
                     f"cuModuleGetGlobal({name})")
        if size.value != len(data):
            raise ValueError(f"{name}: {len(data)} bytes for a {size.value}-byte symbol")
        buf = C.create_string_buffer(data, len(data))
        self.d.check(self.d.cu.cuMemcpyHtoD_v2(g, buf, C.c_size_t(len(data))), f"cuMemcpyHtoD({name})")

    def _launch(self, f, grid, block, args):
        import torch

        holders = []
        ptrs = (C.c_void_p * len(args))()
        for i, a in enumerate(args):
            if isinstance(a, torch.Tensor):
                h = C.c_void_p(a.data_ptr())
            elif isinstance(a, float):
                h = C.c_float(a)
            else:
                h = C.c_int(int(a))
            holders.append(h)
            ptrs[i] = C.cast(C.byref(h), C.c_void_p)
        st = C.c_void_p(torch.cuda.current_stream().cuda_stream)
        bx, by = block if isinstance(block, tuple) else (block, 1)
        self.d.check(self.d.cu.cuLaunchKernel(f, grid, 1, 1, bx, by, 1, 0, st, ptrs, None), "cuLaunchKernel")
        torch.cuda.synchronize()

    def dense(self, o, v, xyzmin, xyzmax, voxel_num, voxel_size):
        """ray_voxel_intersect wrapper semantics (ray_voxel_intersect.cpp:13-42)."""
        import torch

        B = o.shape[0]
        max_n = int(float(voxel_num) * 3)
        inter = torch.zeros(B, max_n, 3, device="cuda")
        num = torch.zeros(B, dtype=torch.int32, device="cuda")
        tns = torch.full((B, max_n), -1.0, device="cuda")
        self._launch(self._func("ray_voxel_intersect_kernel"), (B + 1023) // 1024, 1024,
                     [B, max_n, float(xyzmin), float(xyzmax), float(voxel_num), float(voxel_size), o, v, inter, num, tns])
        return inter, num, tns

    def masked(self, o, v, xyzmin, xyzmax, voxel_num, voxel_size, mask, mask_scale):
        import torch

        B = o.shape[0]
        max_n = int(float(voxel_num) * 3)
        inter = torch.zeros(B, max_n, 6, device="cuda")
        num = torch.zeros(B, dtype=torch.int32, device="cuda")
        tns = torch.full((B, max_n), -1.0, device="cuda")
        self._launch(self._func("masked_intersect_kernel"), (B + 1023) // 1024, 1024,
                     [B, max_n, float(xyzmin), float(xyzmax), float(voxel_num), float(voxel_size), float(mask_scale),
                      o, v, mask, inter, num, tns])
        return inter, num, tns

    def aabb(self, o, v, center, finish, rgba, octrees, N):
        import torch

        g = C.c_void_p()
        size = C.c_size_t()
        self.d.check(self.d.cu.cuModuleGetGlobal_v2(C.byref(g), C.byref(size), self.mods["ray_march"], b"c_center"),
                     "cuModuleGetGlobal(c_center)")
        c = center.detach().float().cpu().contiguous()
        self.d.check(self.d.cu.cuMemcpyHtoD_v2(g, C.c_void_p(c.data_ptr()), C.c_size_t(12)), "cuMemcpyHtoD")
        B = v.numel() // 3
        self._launch(self._func("aabb_intersect_kernel", f"ILi{N}E"), (B + 1023) // 1024, 1024,
                     [B, o, v, finish, rgba, octrees])

    def march(self, o, v, mask, finish, N):
        B = v.numel() // 3
        self._launch(self._func("ray_march_kernel", f"ILi{N}E"), 256, 1024, [B, o, v, mask, finish])

    def upload_weight(self, width: int, params, voxel_map):
        """upload_weight semantics (mlp_eval.cu:264-295): the flat params into
        the kernel's __constant__ array, the [n][n][n] int32 index map (a CUDA
        tensor the caller keeps alive) as the kernel's map."""
        import numpy as np

        unit = f"mlp_eval{width}"
        p = np.ascontiguousarray(params.detach().cpu().numpy(), np.float32)
        self._set_global(unit, "params_cache", p.tobytes())
        self._set_global(unit, "c_voxel_map_ptr", np.array([voxel_map.data_ptr()], np.uint64).tobytes())
        self._set_global(unit, "c_voxel_map_n", np.array([voxel_map.shape[0]], np.int32).tobytes())

    def mlp_eval(self, width: int, rgba, coords, voxels, v, finish):
        """mlp_eval_wrapper's launch (mlp_eval.cu:234-253): 1024 blocks of 16 x 24
        threads over an image 800 pixels wide; in place on rgba and finish."""
        B = v.numel() // 3
        self._launch(self._func("mlp_eval_kernel", unit=f"mlp_eval{width}"), 1024, (16, 24),
                     [B, coords, voxels, v, rgba, finish])
