#!/usr/bin/env python
"""Benchmark of the DIVeR hot path on GB300.

Default workload (one step): one training forward + backward over a batch of
4096 rays of the 256^3 x 32-channel DIVeR32 scene (257^3 corner features,
~60% occupancy), rays drawn from 100 cameras at 800x800 among rays that hit
occupied voxels, MSE + sparsity loss, gradients for the feature grid and the
decoder.  Inputs are synthetic (seeded), with the shapes of the reference's
NeRF-synthetic fine configuration.  Also reported: full-frame render
(800x800) rays/s and p50/p99 frame latency on the same scene.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the reference algorithm on the host cores (the CPU
oracle: C traversal + torch CPU integrate/decoder/render/loss with autograd),
on bounded samples of the same workload.
"""
from __future__ import annotations

import argparse
import math
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mrays/s render & train fwd+bwd, p50/p99 frame ms; fused BF16 vs plain FP32 @ tol"
BATCH = 4096
L_S = 1e-5
# Algorithmic work of the decode kernels (the roofline's numerator), DIVeR32 over
# 32 channels, per launch of S segments of R rays touching U distinct corner rows:
#   FLOPs   forward 10,176 per segment (2 x multiply-adds of the torch-form decoder
#           incl. the per-segment PE part), backward 2 x that (input + weight grads)
#   bytes   compulsory HBM bytes: corner rows U x 128 B (read by a forward,
#           read-modify-written once by a backward's gradient accumulation), the
#           segment record + ray id (28 B), out4 / d4 (16 B each), the per-ray PE
#           rows (pe_feat 112 B, pe_out 128 B), and the 320 B of BF16 layer tiles per
#           segment that the tensor-core forward saves and its backward reads back
ROW_BYTES = 32 * 4
FLOP_FWD_SEG = 10176


def alg_work(kernel, S, U, R):
    """(FLOPs, bytes) of one launch."""
    if kernel == "dv_decode_bwd_tc":
        return 2 * FLOP_FWD_SEG * S, 2 * U * ROW_BYTES + S * (28 + 16 + 16 + 320) + R * (112 + 128)
    if kernel == "dv_decode_bwd":
        return 2 * FLOP_FWD_SEG * S, 3 * U * ROW_BYTES + S * (28 + 16) + R * (112 + 128)
    if kernel == "dv_decode_fwd_tc":
        return FLOP_FWD_SEG * S, U * ROW_BYTES + S * (28 + 16 + 320) + R * 128
    if kernel == "dv_decode_fwd":
        return FLOP_FWD_SEG * S, U * ROW_BYTES + S * (28 + 16) + R * 128
    return 0, 0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per segment of the
# dominant kernels, from one ncu capture of the captured training step of this
# workload (profiles/decode_bwd_tc_train.md); the roofline's `traffic` is this
# times the segments of a launch.
TRAFFIC_PER_SEG = {"dv_decode_bwd_tc": 1302.35, "dv_decode_fwd_tc": 810.52}
OUR_LAUNCHES_PER_STEP = 10  # count, 3 x scan, segments, ray_pe, decode_fwd(_tc), composite_fwd, composite_bwd,
#                             decode_bwd(_tc)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=100)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--frames", type=int, default=8)
    p.add_argument("--no-render", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--requests", type=int, default=24)
    p.add_argument("--no-extra", action="store_true", help="skip the wide-grid, 64-channel and real-time sections")
    p.add_argument("--form", default="bf16", choices=["fp32", "bf16", "fp16"],
                   help="decoder form of the headline training step (the FP32 form is always timed too)")
    return p.parse_args()


def dist_setup(n):
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def _reduce_device() -> str:
    """Where the timing reductions live: the GPU for NCCL, the host for gloo."""
    import torch.distributed as dist

    return "cuda" if dist.get_backend() == "nccl" else "cpu"


def allreduce_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], device=_reduce_device(), dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], device=_reduce_device(), dtype=torch.float64)
    dist.all_reduce(t)
    return float(t.item())


class Clocks:
    """nvidia-smi samples (every 50 ms) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-lms", "50", "-i", str(self.index)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            # wait for the sampler's first line (taken before the region, not kept) so that the
            # samples that follow all fall inside the timed region
            import select

            if select.select([self.proc.stdout], [], [], 5.0)[0]:
                self.proc.stdout.readline()
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# --- workload ------------------------------------------------------------------

def train_scene(device):
    from diver_gb300 import scenes

    return scenes.grid_scene(256, 32, "diver32", device=device)


def make_batches(scene, count, device, seed=4):
    """`count` batches of BATCH rays from 100 cameras at 800x800 (focal 960),
    kept only where the ray crosses at least one occupied voxel."""
    from diver_gb300 import scenes

    return scenes.training_batches(scene, count, BATCH, device, seed)


def unique_corner_rows(seg, n):
    """Distinct grid rows (corner vertices) that the segments' integrals read,
    on a cubic grid of n vertices per side (the corner rule of the decode kernels)."""
    import torch

    lo = torch.minimum((seg.seg[:, :3] + 1e-4).long(), (seg.seg[:, 3:] + 1e-4).long()).clamp_(0, n - 1)
    rows = []
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                x = (lo[:, 0] + dx).clamp_max(n - 1)
                y = (lo[:, 1] + dy).clamp_max(n - 1)
                z = (lo[:, 2] + dz).clamp_max(n - 1)
                rows.append((z * n + y) * n + x)
    return int(torch.unique(torch.cat(rows)).numel())


def train_step(field, o, d, tgt, form="fp32"):
    import torch

    rgb, reg = field(o, d, form=form)
    loss = torch.nn.functional.mse_loss(rgb, tgt) + L_S * reg
    gv, gp = torch.autograd.grad(loss, [field.voxels, field.params])
    return loss, gv, gp


def frame_rays(scene, k, device):
    from diver_gb300 import scenes

    cams = scenes.sphere_cameras(100, 4.0, 3)
    return scenes.camera_rays(cams[k % 100], 800, 800, 960.0, device)


# --- our arm -------------------------------------------------------------------

def run_ours(args, rank, world, local):
    import torch

    import diver_gb300.renderer as R
    from diver_gb300.renderer import DIVeRField

    dev = torch.device("cuda", local)
    scene = train_scene(dev)
    field = DIVeRField.from_scene(scene, dev)
    batches = make_batches(scene, args.warmup + args.steps, dev)
    from diver_gb300.graphs import TrainStepGraph

    forms, graphs = {}, {}
    for form in ("fp32", args.form) if args.form != "fp32" else ("fp32",):
        # eager pipeline, with per-kernel CUDA events
        for i in range(args.warmup):
            train_step(field, *batches[i], form=form)
        torch.cuda.synchronize()
        R.KERNEL_EVENTS = {}
        barrier(world)
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record()
            for i in range(args.steps):
                o, d, tgt = batches[args.warmup + i]
                train_step(field, o, d, tgt, form=form)
            end.record()
            torch.cuda.synchronize()
        barrier(world)
        kms = {k: [s.elapsed_time(e) for s, e in v] for k, v in R.KERNEL_EVENTS.items()}
        R.KERNEL_EVENTS = None
        forms[form] = (start.elapsed_time(end), kms, clk.summary())
        # the same step captured once in a CUDA graph and replayed
        step = TrainStepGraph(field, *batches[0], form=form, l_s=L_S)
        for i in range(args.warmup):
            step(*batches[i])
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        with Clocks(local) as clk:
            start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            start.record()
            for i in range(args.steps):
                step(*batches[args.warmup + i])
            end.record()
            torch.cuda.synchronize()
        barrier(world)
        graphs[form] = (start.elapsed_time(end), clk.summary())
        if form != args.form:
            del step
    tform = args.form
    ms, clocks = graphs[tform]
    kernel_ms = forms[tform][1]
    # segments per step (for the roofline): recount with the same traversal
    seg_counts, corner_rows = [], []
    for i in range(args.steps):
        seg = field.segments(*batches[args.warmup + i][:2])
        seg_counts.append(seg.total)
        corner_rows.append(unique_corner_rows(seg, field.voxels.shape[0]))
        del seg
    ms_max = allreduce_max(ms, world)
    rays = allreduce_sum(float(BATCH * args.steps), world)
    value = rays / (ms_max * 1e-3) / 1e6
    train_forms = {}
    for f in forms:
        train_forms[f] = {"eager": {"Mrays_per_s": rays / (allreduce_max(forms[f][0], world) * 1e-3) / 1e6,
                                    "ms_per_step": forms[f][0] / args.steps},
                          "graph": {"Mrays_per_s": rays / (allreduce_max(graphs[f][0], world) * 1e-3) / 1e6,
                                    "ms_per_step": graphs[f][0] / args.steps}}
    if "fp32" in forms and tform != "fp32":
        train_forms["speedup_vs_fp32"] = {m: train_forms[tform][m]["Mrays_per_s"] / train_forms["fp32"][m]["Mrays_per_s"]
                                          for m in ("eager", "graph")}
    # ---- e2e: pinned host inputs, H2D + D2H inside the timed region ----
    # a training loop's pattern: each step's loss is copied to a pinned host
    # slot and read on the host while the next step runs (one step in flight)
    host = [tuple(t.cpu().pin_memory() for t in b) for b in batches[args.warmup:]]
    loss_host = [torch.empty(1, pin_memory=True) for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    losses = []
    torch.cuda.synchronize()
    barrier(world)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for i, (o_h, d_h, g_h) in enumerate(host):
        loss, _, _ = step(o_h, d_h, g_h)  # H2D copies into the graph's inputs, replay
        loss_host[i % 2].copy_(loss.reshape(1), non_blocking=True)
        copied[i % 2].record()
        if i > 0:
            copied[(i - 1) % 2].synchronize()
            losses.append(loss_host[(i - 1) % 2].item())
    copied[(len(host) - 1) % 2].synchronize()
    losses.append(loss_host[(len(host) - 1) % 2].item())
    t1.record()
    torch.cuda.synchronize()
    if len(losses) != len(host) or not all(math.isfinite(x) for x in losses):
        raise RuntimeError("end-to-end training loop produced a non-finite or missing loss")
    e2e_ms = allreduce_max(t0.elapsed_time(t1), world)
    e2e_val = rays / (e2e_ms * 1e-3) / 1e6
    # ---- render: full frames, forward only, per decoder form ----
    render = None
    if not args.no_render:
        render = {"resolution": [800, 800], "forms": {}}
        with torch.no_grad(), Clocks(local) as rclk:
            for form in ("fp32", "bf16", "fp16"):
                times = []
                for k in range(2 + args.frames):
                    o, d = frame_rays(scene, k, dev)
                    torch.cuda.synchronize()
                    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    s.record()
                    field(o, d, form=form)
                    e.record()
                    torch.cuda.synchronize()
                    if k >= 2:
                        times.append(s.elapsed_time(e))
                times.sort()
                p50 = statistics.median(times)
                p99 = times[min(len(times) - 1, int(round(0.99 * (len(times) - 1))))]
                render["forms"][form] = {"Mrays_per_s": 640000 / (p50 * 1e-3) / 1e6, "p50_ms": p50, "p99_ms": p99,
                                         "frames": len(times)}
        f = render["forms"]
        render["bf16_speedup_vs_fp32"] = f["bf16"]["Mrays_per_s"] / f["fp32"]["Mrays_per_s"]
        render["clocks"] = rclk.summary()
    extra = None
    if not args.no_extra and world == 1:
        del field, step
        torch.cuda.empty_cache()
        extra = {"wide_train": run_wide_train(args, dev), "rt64_render": run_rt64_render(args, dev),
                 "realtime_frame": run_realtime(args, dev), "prune": run_prune(args, dev),
                 "implicit": run_implicit(args, dev)}
        torch.cuda.empty_cache()
    # ---- serving: 4 resident scenes, Poisson arrivals at 200 req/s ----
    serving = None
    if not args.no_serving and world == 1:
        serving = run_serving(args, dev)
    # ---- roofline of the dominant kernel ----
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    tot = {k: sum(v) for k, v in kernel_ms.items()}
    dom = max(tot, key=tot.get)
    avg_ms = tot[dom] / len(kernel_ms[dom])
    S_mean = statistics.mean(seg_counts)
    U_mean = statistics.mean(corner_rows)
    flops, nbytes = alg_work(dom, S_mean, U_mean, BATCH)
    hbm = peaks.get("hbm_gbs", 6800.0)
    tensor = peaks.get("bf16_tflops_sustained", 1700.0)
    t_bytes, t_flops = nbytes / (hbm * 1e9), flops / (tensor * 1e12)
    sec = avg_ms * 1e-3
    if t_bytes >= t_flops:
        roofline = {"kernel": dom, "bound": "hbm", "achieved": nbytes / sec / 1e9, "peak": hbm, "unit": "GB/s",
                    "frac": nbytes / sec / 1e9 / hbm,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peaks else "fallback"}
    else:
        roofline = {"kernel": dom, "bound": "tensor", "achieved": flops / sec / 1e12, "peak": tensor,
                    "unit": "TFLOP/s", "frac": flops / sec / 1e12 / tensor,
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (measured)" if peaks else "fallback"}
    roofline.update({
        "traffic": TRAFFIC_PER_SEG[dom] * S_mean if dom in TRAFFIC_PER_SEG else None,
        "algorithmic_bytes": nbytes, "algorithmic_flops": flops,
        "tensor_frac": flops / sec / 1e12 / tensor, "hbm_frac": nbytes / sec / 1e9 / hbm,
        "avg_launch_ms": avg_ms, "segments_per_launch": S_mean, "corner_rows_per_launch": U_mean,
        "kernel_share": {k: v / sum(tot.values()) for k, v in tot.items()}})
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {"fp32": "f32", "bf16": "bf16", "fp16": "f16"}[tform],
        "data": "synthetic: seeded 256^3x32 grid N(0,0.02^2), 16-blob occupancy ~60%, 100 cameras 800x800, "
                "targets U[0,1]",
        "config": {"workload": "train fwd+bwd, DIVeR32, 256^3 x 32 features, batch 4096 rays that hit occupied voxels",
                   "global_batch": BATCH * world,
                   "form": ("plain FP32" if tform == "fp32" else f"tcgen05 {tform.upper()} decoder fwd+bwd, FP32 accumulation, "
                            "FP32 integration/compositing/weight-gradient accumulation")
                           + "; the whole step captured once in a CUDA graph and replayed (diver_gb300.graphs)",
                   "parallelism": f"replicas x{world}",
                   "l2": "inputs larger than L2 (2.2 GB grid), a fresh batch every step"},
        "e2e": {"value": e2e_val, "unit": "Mrays/s", "h2d_bytes_per_step": BATCH * 9 * 4, "d2h_bytes_per_step": 4},
        "gpu_launches": OUR_LAUNCHES_PER_STEP * args.steps,
        "roofline": roofline,
        "train_forms": train_forms,
        "configs": extra,
        "render": render,
        "serving": serving,
        "segments_per_step": statistics.mean(seg_counts),
    }
    line["clocks"] = clocks
    if rank == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(scene, batches[args.warmup], sample=256, repeats=3)
    return line


def _time_steps(fn, warmup, steps):
    import torch

    for _ in range(warmup):
        fn(0)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for i in range(steps):
        fn(i)
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / steps


def run_wide_train(args, dev):
    """Wide grid 320x320x160 x 32 (bbox [-1,1]^2 x [-0.5,0.5], 24 ellipsoids ~25%),
    150 cameras on an ellipse (a=3, b=2, z=0.8) at 1920x1080, batch 8192 rays
    that hit occupied voxels; training fwd+bwd per form."""
    import torch

    from diver_gb300 import _native as N
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.wide_scene(dev)
    field = DIVeRField(sc.features, sc.decoder, sc.mask, sc.xyzmin, sc.voxel_size)
    cams = scenes.ellipse_cameras(150)
    dirs_cam = scenes.pixel_directions(1080, 1920, 1.2 * 1920, dev).reshape(-1, 3)
    g = torch.Generator(device=dev).manual_seed(4)
    gc = torch.Generator().manual_seed(4)
    B = 8192
    batches = []
    while len(batches) < 8:
        c2w = cams[int(torch.randint(0, 150, (1,), generator=gc))].to(dev)
        pick = torch.randint(0, dirs_cam.shape[0], (4 * B,), generator=g, device=dev)
        d = dirs_cam[pick] @ c2w[:, :3].t()
        d = (d / d.norm(dim=-1, keepdim=True)).contiguous()
        o = c2w[:, 3].expand(d.shape).contiguous()
        seg = field.segments(o, d)
        keep = torch.nonzero(seg.counts > 0)[:, 0]
        if keep.numel() >= B:
            keep = keep[:B]
            batches.append((o[keep].contiguous(), d[keep].contiguous(), torch.rand(B, 3, generator=g, device=dev)))
    from diver_gb300.graphs import TrainStepGraph

    out = {"grid": list(sc.dims), "occupancy": float(sc.mask.float().mean()), "batch": B,
           "form": "the step captured in a CUDA graph (eager in `eager_ms_per_step`)"}
    for form in ("fp32", "bf16"):
        eager = _time_steps(lambda i: train_step(field, *batches[i % 8], form=form), 2, 8)
        step = TrainStepGraph(field, *batches[0], form=form, l_s=L_S)
        ms = _time_steps(lambda i: step(*batches[i % 8]), 3, 16)
        del step
        out[form] = {"ms_per_step": ms, "Mrays_per_s": B / (ms * 1e-3) / 1e6, "eager_ms_per_step": eager}
    out["bf16_speedup_vs_fp32"] = out["bf16"]["Mrays_per_s"] / out["fp32"]["Mrays_per_s"]
    return out


def run_rt64_render(args, dev):
    """256^3 x 64-channel scene with a DIVeR64 decoder: full 800x800 frames from
    spiral cameras (radius 4, elevation -30..30 deg) per decoder form."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.grid_scene(256, 64, "diver64", device=dev)
    field = DIVeRField.from_scene(sc, dev)
    cams = scenes.spiral_cameras(200, 4.0)
    rays = [scenes.camera_rays(cams[k * 40], 800, 800, 960.0, dev) for k in range(4)]
    out = {}
    with torch.no_grad():
        for form in ("fp32", "bf16", "fp16"):
            ms = _time_steps(lambda i: field(*rays[i % 4], form=form), 1, 4)
            out[form] = {"frame_ms": ms, "Mrays_per_s": 640000 / (ms * 1e-3) / 1e6}
    out["bf16_speedup_vs_fp32"] = out["bf16"]["Mrays_per_s"] / out["fp32"]["Mrays_per_s"]
    return out


def run_realtime(args, dev):
    """Real-time path (eval_rt.py): the 256^3 x 32 scene converted to the serialized
    form (sparse feature table of occupied voxels' corners), octree first hit, then
    rounds of 8-hit march + fused decoder with early termination, 800x800."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.realtime import RealtimeModel, convert

    sc = scenes.grid_scene(256, 32, "diver32", device=dev)
    sd = {"voxels": sc.features}
    sd.update(sc.decoder.state_dict())
    ser = convert(sd, sc.mask.float())
    model = RealtimeModel.from_serialized(ser, 256, sc.xyzmin, sc.voxel_size, dev)
    cams = scenes.sphere_cameras(100, 4.0, 3)
    frames = []
    for k in range(3):
        _, d = scenes.camera_rays(cams[k], 800, 800, 960.0, dev)
        frames.append((cams[k][:, 3], d))
    rounds = []

    def frame_loop(i):
        _, r = model.render_frame(*frames[i % 3], fused=False)
        rounds.append(r)

    def frame_fused(i):
        model.render_frame(*frames[i % 3])

    ms_loop = _time_steps(frame_loop, 1, 3)
    ms = _time_steps(frame_fused, 3, 10)
    return {"frame_ms": ms, "Mrays_per_s": 640000 / (ms * 1e-3) / 1e6, "form": "one launch per frame",
            "host_loop": {"frame_ms": ms_loop, "rounds": rounds[-1],
                          "form": "aabb_intersect + rounds of ray_march / mlp_eval (the reference's loop)"},
            "features": int(ser["f"].shape[0])}


def run_prune(args, dev):
    """Occupancy extraction (prune.py:86-145) on the 256^3 x 32 DIVeR32 scene:
    alpha map over 4 training views at 800x800 (2.56 M rays, batches of 65,536),
    then the pruned mask at 1e-2 and the bias-sampling ray selection."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.prune import extract_alpha_map, prune_mask, rays_hitting
    from diver_gb300.renderer import DIVeRField

    sc = scenes.grid_scene(256, 32, "diver32", device=dev)
    field = DIVeRField.from_scene(sc, dev)
    cams = scenes.sphere_cameras(100, 4.0, 3)
    rays = torch.cat([torch.cat(scenes.camera_rays(cams[k], 800, 800, 960.0, dev), 1) for k in range(4)], 0)
    extract_alpha_map(field, rays[:65536], batch=65536)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    alpha = extract_alpha_map(field, rays, batch=65536)
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e)
    mask = prune_mask(alpha)
    s.record()
    hit = rays_hitting(field, rays[:, :3], rays[:, 3:6], mask)
    e.record()
    torch.cuda.synchronize()
    return {"rays": int(rays.shape[0]), "alpha_map_ms": ms, "Mrays_per_s": rays.shape[0] / (ms * 1e-3) / 1e6,
            "kept_voxels": float(mask.float().mean().item()), "bias_sampling_ms": s.elapsed_time(e),
            "rays_kept": float(hit.float().mean().item())}


def run_implicit(args, dev):
    """Implicit stage (utils/integrator.py:3-59 + model/mlps.py:34-81): one
    forward + backward of integrate_mlp over the segments of a 4096-ray training
    batch of the 256^3 scene, ImplicitMLP(8, 512, [4], 32, 10) under BF16
    autocast (its GEMMs are cuBLAS), gradients for the MLP."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.implicit import ImplicitMLP
    from diver_gb300.integrator import integrate_mlp
    from diver_gb300.renderer import DIVeRField

    sc = scenes.grid_scene(256, 32, "diver32", device=dev)
    field = DIVeRField.from_scene(sc, dev)
    o, d, _ = make_batches(sc, 1, dev)[0]
    seg = field.segments(o, d)
    del field
    torch.manual_seed(0)
    mlp = ImplicitMLP(8, 512, [4], 32, 10).to(dev)
    G = torch.randn(seg.total, 32, device=dev)
    uniq = {}

    def step(i):
        with torch.autocast("cuda", dtype=torch.bfloat16):
            f = integrate_mlp(mlp, 257, 32, seg.seg[:, :3], seg.seg[:, 3:])
        grads = torch.autograd.grad((f * G).sum(), list(mlp.parameters()))
        return grads

    ms = _time_steps(step, 2, 5)
    from diver_gb300.integrator import corner_rows

    U = int(torch.unique(corner_rows(seg.seg[:, :3], seg.seg[:, 3:], 257)).numel())
    flops = 2 * 3 * U * (63 * 512 + 6 * 512 * 512 + (512 + 63) * 512 + 512 * 32)  # fwd + 2x bwd
    return {"segments": seg.total, "unique_corners": U, "ms_per_step": ms,
            "Mseg_per_s": seg.total / (ms * 1e-3) / 1e6, "mlp_tflops": flops / (ms * 1e-3) / 1e12,
            "mlp": "ImplicitMLP(8, 512, [4], 32, 10), BF16 autocast (cuBLAS)"}


def run_serving(args, dev):
    """Two 256^3x32 DIVeR32 and two 256^3x64 DIVeR64 scenes (different seeds) under a
    60 GB HBM budget; requests: scene id, a random camera on a radius-4 sphere and a
    resolution from {200^2, 400^2, 800^2, 1280x720, 1920x1080}, Poisson arrivals at
    200 req/s; BF16 tensor-core decoder."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField
    from diver_gb300.serving import GpuRenderer, Request, Residency, latency_summary, serve

    specs = [("d32a", 32, "diver32", 0), ("d32b", 32, "diver32", 1), ("d64a", 64, "diver64", 2),
             ("d64b", 64, "diver64", 3)]
    res = Residency(60 << 30)
    for name, ch, kind, k in specs:
        nbytes = 257 ** 3 * ch * 4 + 256 ** 3
        res.register(name, nbytes, lambda ch=ch, kind=kind, k=k: DIVeRField.from_scene(
            scenes.grid_scene(256, ch, kind, device=dev, seed_offset=100 * k), dev))
    for name, *_ in specs:  # load everything before the clock starts
        res.acquire(name)
        res.release(name)
    g = torch.Generator().manual_seed(4)
    sizes = [(200, 200), (400, 400), (800, 800), (720, 1280), (1080, 1920)]
    t = 0.0
    reqs = []
    for i in range(args.requests):
        t += float(torch.empty(1).exponential_(200.0, generator=g))
        name = specs[int(torch.randint(0, 4, (1,), generator=g))][0]
        H, W = sizes[int(torch.randint(0, 5, (1,), generator=g))]
        v = torch.randn(3, generator=g)
        c2w = scenes.look_at(v / v.norm() * 4.0)
        reqs.append(Request(i, name, c2w, H, W, 1.2 * W, arrival=t))
    torch.cuda.synchronize()
    done = serve(reqs, res, GpuRenderer("bf16"), realtime=True, max_rays_in_flight=1 << 23, chunk_rays=1 << 19)
    torch.cuda.synchronize()
    out = latency_summary(done)
    out.update({"scenes": len(specs), "arrival_rate_per_s": 200, "hbm_budget_gb": 60, "form": "bf16",
                "resident_gb": res.used / 1e9})
    return out


# --- CPU reference path (oracle port) ------------------------------------------

def cpu_sample_step(feat_cpu, mask_np, scene, layers, o, d, tgt):
    import numpy as np
    import torch

    from oracle import native as orc
    from oracle import torch_ref

    inter, num, _ = orc.masked_walk(o, d, scene.xyzmin, scene.voxel_num, scene.voxel_size, mask_np, 1.0)
    seg = torch.from_numpy(orc.csr_from_padded(inter, num))
    ray = torch.from_numpy(np.repeat(np.arange(len(num)), num))
    V = feat_cpu.requires_grad_(True)
    L = [(w.requires_grad_(True), b.requires_grad_(True)) for w, b in layers]
    rgb, sigma, _ = torch_ref.forward(V, L, 3, seg, ray, torch.from_numpy(num), torch.from_numpy(d))
    loss = torch_ref.loss(rgb, torch.from_numpy(tgt), sigma)
    loss.backward()
    V.grad = None
    return loss.item()


def cpu_baseline(scene, batch, sample=256, repeats=3):
    import torch

    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    feat = scene.features.detach().cpu()
    mask_np = scene.mask.cpu().numpy()
    layers = [(w.detach().cpu().clone(), b.detach().cpu().clone()) for w, b in scene.decoder.layers]
    o, d, tgt = (x[:sample].cpu().numpy() for x in batch)
    cpu_sample_step(feat, mask_np, scene, layers, o, d, tgt)
    ts = []
    for _ in range(repeats):
        t = time.perf_counter()
        cpu_sample_step(feat, mask_np, scene, layers, o, d, tgt)
        ts.append(time.perf_counter() - t)
    sec = statistics.median(ts)
    return {"value": sample / sec / 1e6, "unit": "Mrays/s", "cores": cores, "kind": "port",
            "sample": f"{sample} rays of one training batch, fwd+bwd (C traversal + torch CPU integrate/decoder/render/"
                      f"loss/autograd), median of {repeats}"}


def run_reference(args, rank, world):
    import torch

    if rank != 0:
        return None
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else torch.device("cpu")
    scene = train_scene(dev)
    batches = make_batches(scene, 1, dev) if dev.type == "cuda" else None
    feat = scene.features.detach().cpu()
    mask_np = scene.mask.cpu().numpy()
    layers = [(w.detach().cpu().clone(), b.detach().cpu().clone()) for w, b in scene.decoder.layers]
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    sample = 256
    o, d, tgt = (x.cpu().numpy() for x in batches[0])
    for i in range(args.warmup):
        cpu_sample_step(feat, mask_np, scene, layers, o[:sample], d[:sample], tgt[:sample])
    t = time.perf_counter()
    for i in range(args.steps):
        j = (i * sample) % (BATCH - sample)
        cpu_sample_step(feat, mask_np, scene, layers, o[j:j + sample], d[j:j + sample], tgt[j:j + sample])
    sec = time.perf_counter() - t
    value = sample * args.steps / sec / 1e6
    return {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "impl": "reference",
        "data": "synthetic: same scene and batches as the GPU arm",
        "config": {"workload": "train fwd+bwd, DIVeR32, 256^3 x 32 features, batch 4096 rays that hit occupied voxels",
                   "global_batch": BATCH, "form": "reference algorithm on host cores", "parallelism": "cpu"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"{sample} rays per step of the training workload (C traversal restatement + "
                                   f"torch CPU integrate/decoder/render/loss/autograd)"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_ours(args, rank, world, local)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
