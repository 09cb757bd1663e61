#!/usr/bin/env python
"""Benchmark of the DIVeR hot path on GB300.

Default workload (one step): one training forward + backward over a batch of
4096 rays of the 256^3 x 32-channel DIVeR32 scene (257^3 corner features,
~60% occupancy), rays drawn from 100 cameras at 800x800 among rays that hit
occupied voxels, MSE + sparsity loss, gradients for the feature grid and the
decoder.  The headline form is 'bf16s': the tensor-core decoder with split
BF16 operands, whose gradients are FP32-grade (the plain FP32 form and the
single-term BF16 form are timed beside it).  Inputs are synthetic (seeded),
with the shapes of the reference's NeRF-synthetic fine configuration.  Also
reported: full-frame renders (800x800) per decoder form with p50/p99 frame
latency, the wide-grid training, the 64-channel DIVeR64 frames, the real-time
frame, occupancy extraction, the implicit stage and the serving loop.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
    python bench.py --profile train|render ...   (profiling drivers, see below)

The timed region is K steps between a barrier and a device synchronisation;
it is repeated until at least --min-region-s seconds have been timed (the
clocks are sampled over all repeats) and `value` comes from the median
region.

`--impl reference` times the reference algorithm on the host cores (the CPU
oracle: C traversal + torch CPU integrate/decoder/render/loss with autograd)
on the same 4096-ray batches, built without this repository's CUDA library,
and, on the same GPU, the reference's own traversal kernels (built from its
sources) with its torch decode path on CUDA tensors.
"""
from __future__ import annotations

import argparse
import json
import math
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
FORM_NAMES = {"fp32": "plain FP32 decoder",
              "bf16": "tcgen05 BF16 decoder (one BF16 term per operand)",
              "fp16": "tcgen05 FP16 decoder",
              "bf16s": "tcgen05 decoder with split BF16 operands (three terms, six products per layer; two-term "
                       "weight gradients): FP32-grade gradients"}
DTYPES = {"fp32": "f32", "bf16": "bf16", "fp16": "f16", "bf16s": "bf16x3 (split f32)"}
# Algorithmic work of the decode kernels (the roofline's numerator), DIVeR32 over
# 32 channels, per launch of S segments of R rays touching U distinct corner rows:
#   FLOPs   forward 10,176 per segment (2 x multiply-adds of the torch-form decoder
#           incl. the per-segment PE part), backward 2 x that (input + weight grads);
#           the split-operand kernels issue six (three) tensor-core products per
#           product counted here, which is not algorithmic work
#   bytes   compulsory HBM bytes: the corner rows U x 128 B (read by a forward,
#           read-modify-written once by a backward's gradient accumulation) and the
#           rays, 24 B in and 16 B out each; segment lists, layer tiles and other
#           intermediates are not compulsory
ROW_BYTES = 32 * 4
FLOP_FWD_SEG = 10176
FWD_KERNELS = ("dv_decode_fwd", "dv_decode_fwd_tc", "dv_decode_fwd_tc_split")
BWD_KERNELS = ("dv_decode_bwd", "dv_decode_bwd_tc", "dv_decode_bwd_tc_split")


def alg_work(kernel, S, U, R):
    """(FLOPs, bytes) of one launch."""
    if kernel in BWD_KERNELS:
        return 2 * FLOP_FWD_SEG * S, 2 * U * ROW_BYTES + R * 40
    if kernel in FWD_KERNELS:
        return FLOP_FWD_SEG * S, U * ROW_BYTES + R * 40
    return 0, 0


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per segment of the
# decode kernels in the captured 4096-ray training step, from ncu captures of
# `python bench.py --profile train --form <form>`: the single-term BF16 kernels
# on the 256^3 grid, the split-operand forward on the 128^3 grid of the same
# scene family (557,787 segments; its traffic is per-segment: the rays'
# segments, the corner rows and the saved record); the roofline's `traffic`
# is this times the segments of a launch.  The split backward has no entry:
# its current form has no ncu section capture (the roofline reports null).
TRAFFIC_PER_SEG = {"dv_decode_bwd_tc": 1302.35, "dv_decode_fwd_tc": 810.52, "dv_decode_fwd_tc_split": 997.2}
# Kernels of this library per captured training step: row clear, three weight
# image gathers, ray PE, slot walk, 3 scan kernels, slot compaction, decoder
# forward, compositing forward, sparsity mean, loss, loss gradients,
# compositing backward, decoder backward (which also marks the rows the next
# step's clear zeroes).
OUR_LAUNCHES_PER_STEP = 17


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--form", default="bf16s", choices=["fp32", "bf16", "fp16", "bf16s"],
                   help="decoder form of the headline training step (fp32, bf16 and bf16s are always timed)")
    p.add_argument("--min-region-s", type=float, default=1.0,
                   help="repeat the K-step timed region until this many seconds are timed")
    p.add_argument("--frames", type=int, default=100, help="800x800 frames per form (render section)")
    p.add_argument("--rt64-frames", type=int, default=200, help="spiral frames of the 64-channel scene per 16-bit form")
    p.add_argument("--requests", type=int, default=500)
    p.add_argument("--no-render", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-serving", action="store_true")
    p.add_argument("--no-extra", action="store_true", help="skip the wide-grid, 64-channel and real-time sections")
    p.add_argument("--no-reference-gpu", action="store_true", help="reference arm: skip the GPU timings")
    # profiling drivers (no JSON line): a short run whose profiled part sits
    # between cudaProfilerStart/Stop (ncu --profile-from-start off)
    p.add_argument("--profile", choices=["train", "render"], default=None)
    p.add_argument("--profiled", type=int, default=3, help="--profile train: profiled replays")
    p.add_argument("--timed", type=int, default=20, help="--profile train: timed replays printed afterwards")
    p.add_argument("--grid", type=int, default=256, help="--profile: n^3 grid of the scene family")
    p.add_argument("--size", type=int, default=800, help="--profile render: image size")
    p.add_argument("--forms", default="fp32,bf16", help="--profile render: decoder forms")
    p.add_argument("--repeat", type=int, default=2, help="--profile render: frames per form")
    p.add_argument("--channels", type=int, default=32, help="--profile render: feature channels")
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


def pct(sorted_vals, p):
    return sorted_vals[min(len(sorted_vals) - 1, int(round(p * (len(sorted_vals) - 1))))]


def timed_regions(fn, steps, world, min_s, clk_index=None):
    """Times regions of `steps` calls fn(i) (i = 0..steps-1), each between a
    barrier and a device synchronisation on both sides, max over ranks;
    repeated until `min_s` seconds are timed.  Returns (region ms list, clocks
    summary or None)."""
    import torch

    def one():
        barrier(world)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for i in range(steps):
            fn(i)
        e.record()
        torch.cuda.synchronize()
        barrier(world)
        return allreduce_max(s.elapsed_time(e), world)

    first = one()  # untimed calibration region
    reps = int(min(500, max(1, math.ceil(min_s * 1e3 / max(first, 1e-3)))))
    reps = int(allreduce_max(float(reps), world))
    clk = Clocks(clk_index) if clk_index is not None else None
    if clk:
        clk.__enter__()
    times = [one() for _ in range(reps)]
    if clk:
        clk.__exit__(None, None, None)
    return times, (clk.summary() if clk else None)


def region_stats(times, steps):
    st = sorted(times)
    med = statistics.median(st)
    return {"regions": len(st), "steps_per_region": steps, "median_ms": med, "min_ms": st[0], "max_ms": st[-1],
            "spread": (st[-1] - st[0]) / med if med > 0 else None}


# --- workload ------------------------------------------------------------------

def train_scene(device):
    from diver_gb300 import scenes

    return scenes.grid_scene(256, 32, "diver32", device=device)


def make_batches(scene, count, device, seed=4, count_fn=None):
    """`count` batches of BATCH rays from 100 cameras at 800x800 (focal 960),
    kept only where the ray crosses at least one occupied voxel."""
    from diver_gb300 import scenes

    return scenes.training_batches(scene, count, BATCH, device, seed, count_fn=count_fn)


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

    from diver_gb300.renderer import l2_loss

    rgb, reg = field(o, d, form=form)
    loss = l2_loss(rgb, reg, tgt, L_S)
    gv, gp = torch.autograd.grad(loss, [field.voxels, field.params])
    return loss, gv, gp


def frame_rays(scene, k, device):
    from diver_gb300 import scenes

    cams = scenes.sphere_cameras(100, 4.0, 3)
    return scenes.camera_rays(cams[k % 100], 800, 800, 960.0, device)


def e2e_loop(step, host, world, min_s):
    """End-to-end training loop through the captured step: every step's inputs
    copied from pinned host memory, its loss copied to a pinned host slot and
    read on the host while the next step runs (one step in flight).  Timed in
    regions of len(host) steps like the headline."""
    import torch

    loss_host = [torch.empty(1, pin_memory=True) for _ in range(2)]
    copied = [torch.cuda.Event() for _ in range(2)]
    bad = []

    def region_fn(i):
        o_h, d_h, g_h = host[i]
        loss, _, _ = step(o_h, d_h, g_h)  # H2D copies into the graph's inputs, replay
        loss_host[i % 2].copy_(loss.reshape(1), non_blocking=True)
        copied[i % 2].record()
        if i > 0:
            copied[(i - 1) % 2].synchronize()
            if not math.isfinite(loss_host[(i - 1) % 2].item()):
                bad.append(i - 1)
        if i == len(host) - 1:
            copied[i % 2].synchronize()
            if not math.isfinite(loss_host[i % 2].item()):
                bad.append(i)

    times, _ = timed_regions(region_fn, len(host), world, min_s)
    if bad:
        raise RuntimeError("end-to-end training loop produced a non-finite loss")
    return times


# --- our arm -------------------------------------------------------------------

def run_ours(args, rank, world, local):
    import torch

    import diver_gb300.renderer as R
    from diver_gb300.graphs import TrainStepGraph
    from diver_gb300.renderer import DIVeRField

    dev = torch.device("cuda", local)
    scene = train_scene(dev)
    field = DIVeRField.from_scene(scene, dev)
    batches = make_batches(scene, args.warmup + args.steps, dev)
    timed = batches[args.warmup:]
    tform = args.form
    order = ["fp32", "bf16", "bf16s"] + ([tform] if tform not in ("fp32", "bf16", "bf16s") else [])
    order = [f for f in order if f != tform] + [tform]  # the headline form last: its graph stays for e2e
    train_forms, kernel_ms, clocks, regions = {}, {}, None, None
    step = None
    e2e = {}
    for form in order:
        # eager pipeline, with per-kernel CUDA events
        for i in range(args.warmup):
            train_step(field, *batches[i], form=form)
        torch.cuda.synchronize()
        R.KERNEL_EVENTS = {}
        eager, _ = timed_regions(lambda i: train_step(field, *timed[i], form=form), args.steps, world, 0.0)
        kms = {k: [s.elapsed_time(e) for s, e in v] for k, v in R.KERNEL_EVENTS.items()}
        R.KERNEL_EVENTS = None
        # the same step captured once in a CUDA graph and replayed
        step = TrainStepGraph(field, *batches[0], form=form, l_s=L_S)
        for i in range(args.warmup):
            step(*batches[i])
        torch.cuda.synchronize()
        times, clk = timed_regions(lambda i: step(*timed[i]), args.steps, world, args.min_region_s, local)
        rays = allreduce_sum(float(BATCH * args.steps), world)
        rs = region_stats(times, args.steps)
        train_forms[form] = {
            "graph": {"Mrays_per_s": rays / (rs["median_ms"] * 1e-3) / 1e6, "ms_per_step": rs["median_ms"] / args.steps,
                      "regions": rs},
            "eager": {"Mrays_per_s": rays / (statistics.median(eager) * 1e-3) / 1e6,
                      "ms_per_step": statistics.median(eager) / args.steps},
            "clocks": clk}
        if form in (tform, "fp32"):
            host = [tuple(t.cpu().pin_memory() for t in b) for b in timed]
            et = e2e_loop(step, host, world, args.min_region_s)
            e2e[form] = {"value": rays / (statistics.median(et) * 1e-3) / 1e6, "unit": "Mrays/s",
                         "h2d_bytes_per_step": BATCH * 9 * 4, "d2h_bytes_per_step": 4,
                         "regions": region_stats(et, args.steps)}
            train_forms[form]["e2e"] = e2e[form]
        if form == tform:
            kernel_ms, clocks, regions = kms, clk, rs
        else:
            del step
            torch.cuda.empty_cache()
    for f in train_forms:
        if f != "fp32" and "fp32" in train_forms:
            train_forms[f]["speedup_vs_fp32"] = {m: train_forms[f][m]["Mrays_per_s"] / train_forms["fp32"][m]["Mrays_per_s"]
                                                 for m in ("eager", "graph")}
    # segments per step (for the roofline): recount with the same traversal
    seg_counts, corner_rows = [], []
    for i in range(args.steps):
        seg = field.segments(*timed[i][:2])
        seg_counts.append(seg.total)
        corner_rows.append(unique_corner_rows(seg, field.voxels.shape[0]))
        del seg
    value = train_forms[tform]["graph"]["Mrays_per_s"]
    ms_step = regions["median_ms"] / args.steps
    # ---- render: full frames, forward only, per decoder form ----
    render = None
    if not args.no_render:
        render = run_render(args, scene, field, dev)
    extra = None
    if not args.no_extra and world == 1:
        del field, step
        torch.cuda.empty_cache()
        extra = {"wide_train": run_wide_train(args, dev), "rt64_render": run_rt64_render(args, dev),
                 "realtime_frame": run_realtime(args, dev), "prune": run_prune(args, dev),
                 "implicit": run_implicit(args, dev)}
        torch.cuda.empty_cache()
    # ---- serving: 4 resident scenes, Poisson arrivals ----
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
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if peaks else "fallback"}
    else:
        roofline = {"kernel": dom, "bound": "tensor", "achieved": flops / sec / 1e12, "peak": tensor,
                    "unit": "TFLOP/s", "frac": flops / sec / 1e12 / tensor,
                    "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained (of measured)" if peaks else "fallback"}
    roofline.update({
        "traffic": TRAFFIC_PER_SEG[dom] * S_mean if dom in TRAFFIC_PER_SEG else None,
        "algorithmic_bytes": nbytes, "algorithmic_flops": flops,
        "tensor_frac": flops / sec / 1e12 / tensor, "hbm_frac": nbytes / sec / 1e9 / hbm,
        "avg_launch_ms": avg_ms, "segments_per_launch": S_mean, "corner_rows_per_launch": U_mean,
        "timing": "CUDA events around each launch on its stream, eager pipeline, mean over the K timed steps",
        "kernel_share": {k: v / sum(tot.values()) for k, v in tot.items()}})
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": DTYPES[tform],
        "data": "synthetic: seeded 256^3x32 grid N(0,0.02^2), 16-blob occupancy ~60%, 100 cameras 800x800, "
                "targets U[0,1]",
        "config": train_config(world),
        "form": FORM_NAMES[tform] + "; FP32 integration, compositing and gradient accumulation; the whole step "
                "captured once in a CUDA graph and replayed (diver_gb300.graphs)",
        "timed_region": regions,
        "e2e": e2e[tform],
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
        line["cpu_baseline"] = cpu_baseline(scene, timed[0], sample=256, repeats=3)
    return line


def train_config(world):
    return {"workload": "train fwd+bwd, DIVeR32, 256^3 x 32 features, batch 4096 rays that hit occupied voxels",
            "global_batch": BATCH * world, "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (2.2 GB grid), a fresh batch every step"}


def run_render(args, scene, field, dev):
    """Full 800x800 frames of the training scene from the 100 sphere cameras
    (two untimed frames first), forward only, per decoder form: Mrays/s from
    the median frame, p50 / p99 frame latency."""
    import torch

    out = {"resolution": [800, 800], "forms": {}}
    with torch.no_grad(), Clocks(dev.index or 0) as rclk:
        for form in ("fp32", "bf16", "fp16", "bf16s"):
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
            out["forms"][form] = {"Mrays_per_s": 640000 / (p50 * 1e-3) / 1e6, "p50_ms": p50, "p99_ms": pct(times, 0.99),
                                  "frames": len(times)}
    f = out["forms"]
    out["bf16_speedup_vs_fp32"] = f["bf16"]["Mrays_per_s"] / f["fp32"]["Mrays_per_s"]
    out["clocks"] = rclk.summary()
    return out


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


def _frame_times(fn, n, warmup=2):
    """Per-call CUDA-event times (ms) of fn(i), i = 0..n-1, after `warmup` calls."""
    import torch

    for i in range(warmup):
        fn(i)
    torch.cuda.synchronize()
    times = []
    for i in range(n):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        fn(i)
        e.record()
        torch.cuda.synchronize()
        times.append(s.elapsed_time(e))
    return sorted(times)


def run_wide_train(args, dev):
    """Wide grid 320x320x160 x 32 (bbox [-1,1]^2 x [-0.5,0.5], 24 ellipsoids ~25%),
    150 cameras on an ellipse (a=3, b=2, z=0.8) at 1920x1080, batch 8192 rays
    that hit occupied voxels; training fwd+bwd per form."""
    import torch

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
    for form in ("fp32", "bf16", "bf16s"):
        eager = _time_steps(lambda i: train_step(field, *batches[i % 8], form=form), 2, 8)
        step = TrainStepGraph(field, *batches[0], form=form, l_s=L_S)
        ms = _time_steps(lambda i: step(*batches[i % 8]), 3, 16)
        del step
        out[form] = {"ms_per_step": ms, "Mrays_per_s": B / (ms * 1e-3) / 1e6, "eager_ms_per_step": eager}
    for form in ("bf16", "bf16s"):
        out[f"{form}_speedup_vs_fp32"] = out[form]["Mrays_per_s"] / out["fp32"]["Mrays_per_s"]
    return out


def run_rt64_render(args, dev):
    """256^3 x 64-channel scene with a DIVeR64 decoder: full 800x800 frames from
    the 200 spiral cameras (radius 4, elevation -30..30 deg) for the 16-bit
    forms, every 4th camera (50) for the FP32 and split forms; p50 / p99."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    sc = scenes.grid_scene(256, 64, "diver64", device=dev)
    field = DIVeRField.from_scene(sc, dev)
    cams = scenes.spiral_cameras(200, 4.0)
    out = {"cameras": 200}
    with torch.no_grad():
        for form in ("fp32", "bf16", "fp16", "bf16s"):
            pick = list(range(0, 200, 1 if form in ("bf16", "fp16") else 4))[:max(1, args.rt64_frames)]
            rays = lambda i: scenes.camera_rays(cams[pick[i % len(pick)]], 800, 800, 960.0, dev)
            # each frame's rays are generated before its events
            times = []
            for i in range(len(pick) + 1):
                o, d = rays(i)
                torch.cuda.synchronize()
                s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s.record()
                field(o, d, form=form)
                e.record()
                torch.cuda.synchronize()
                if i > 0:
                    times.append(s.elapsed_time(e))
            times.sort()
            p50 = statistics.median(times)
            out[form] = {"frames": len(times), "p50_ms": p50, "p99_ms": pct(times, 0.99),
                         "Mrays_per_s": 640000 / (p50 * 1e-3) / 1e6}
    out["bf16_speedup_vs_fp32"] = out["bf16"]["Mrays_per_s"] / out["fp32"]["Mrays_per_s"]
    return out


def run_realtime(args, dev):
    """Real-time path (eval_rt.py): the 256^3 x 32 scene converted to the serialized
    form (sparse feature table of occupied voxels' corners), octree first hit, then
    rounds of 8-hit march + fused decoder with early termination, 800x800, frames
    from the 100 sphere cameras: p50 / p99."""
    from diver_gb300 import scenes
    from diver_gb300.realtime import RealtimeModel, convert

    sc = scenes.grid_scene(256, 32, "diver32", device=dev)
    sd = {"voxels": sc.features}
    sd.update(sc.decoder.state_dict())
    ser = convert(sd, sc.mask.float())
    model = RealtimeModel.from_serialized(ser, 256, sc.xyzmin, sc.voxel_size, dev)
    cams = scenes.sphere_cameras(100, 4.0, 3)
    frames = []
    for k in range(100):
        _, d = scenes.camera_rays(cams[k], 800, 800, 960.0, dev)
        frames.append((cams[k][:, 3], d))
    rounds = []

    def frame_loop(i):
        _, r = model.render_frame(*frames[i % 100], mode="loop")
        rounds.append(r)

    loop = _frame_times(frame_loop, 10, 1)
    fused = _frame_times(lambda i: model.render_frame(*frames[i % 100], mode="fused"), 100, 3)
    tc = _frame_times(lambda i: model.render_frame(*frames[i % 100], mode="tc"), 100, 3)
    p50 = statistics.median(tc)
    return {"frame_ms": p50, "p50_ms": p50, "p99_ms": pct(tc, 0.99), "frames": len(tc),
            "Mrays_per_s": 640000 / (p50 * 1e-3) / 1e6,
            "form": "aabb_intersect + rounds of ray_march and the tcgen05 decoder (split BF16 operands, FP32-grade)",
            "fused_fp32": {"p50_ms": statistics.median(fused), "p99_ms": pct(fused, 0.99), "frames": len(fused),
                           "form": "one launch per frame, FP32 decoder"},
            "host_loop": {"frame_ms": statistics.median(loop), "frames": len(loop), "rounds": rounds[-1],
                          "form": "aabb_intersect + rounds of ray_march / mlp_eval (the reference's loop, FP32 decoder)"},
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


# Serving: bytes a resident scene holds (FP32 grid, the 16-bit copy the
# tensor-core render reads, the occupancy bytes, decoder and weight images) and
# the working memory of the batches in flight (segment lists and per-segment
# decoder outputs: about 180 segments of 48 B per ray on these scenes, kept
# with a factor of 2 for the allocator's slack).
SEG_BYTES_PER_RAY = 2 * 180 * 48


def scene_bytes(n, ch):
    return (n + 1) ** 3 * ch * (4 + 2) + n ** 3 + (1 << 20)


def run_serving(args, dev):
    """Two 256^3x32 DIVeR32 and two 256^3x64 DIVeR64 scenes (different seeds) under a
    60 GB HBM budget that charges every resident scene's grids and the working
    memory of the rays in flight; requests: scene id, a random camera on a
    radius-4 sphere and a resolution from {200^2, 400^2, 800^2, 1280x720,
    1920x1080}, Poisson arrivals.  Two runs: the configuration's 200 req/s
    (offered load against the measured capacity; above it the latencies measure
    the queue) and a rate the box sustains (60 % of the measured capacity:
    steady-state latencies).  BF16 tensor-core decoder."""
    import torch

    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField
    from diver_gb300.serving import GpuRenderer, Request, Residency, latency_summary, serve

    specs = [("d32a", 32, "diver32", 0), ("d32b", 32, "diver32", 1), ("d64a", 64, "diver64", 2),
             ("d64b", 64, "diver64", 3)]
    max_rays, chunk = 1 << 21, 1 << 19
    res = Residency(60 << 30, reserved_bytes=max_rays * SEG_BYTES_PER_RAY)
    for name, ch, kind, k in specs:
        res.register(name, scene_bytes(256, ch), lambda ch=ch, kind=kind, k=k: DIVeRField.from_scene(
            scenes.grid_scene(256, ch, kind, device=dev, seed_offset=100 * k), dev))
    for name, *_ in specs:  # load everything (and the 16-bit grid copies) before the clock starts
        res.acquire(name)
        with torch.no_grad():
            res.scenes[name].resident.grid16("bf16")
        res.release(name)
    sizes = [(200, 200), (400, 400), (800, 800), (720, 1280), (1080, 1920)]
    mean_rays = sum(h * w for h, w in sizes) / len(sizes)

    def stream(n, rate, seed):
        g = torch.Generator().manual_seed(seed)
        t, reqs = 0.0, []
        for i in range(n):
            t += float(torch.empty(1).exponential_(rate, generator=g))
            name = specs[int(torch.randint(0, 4, (1,), generator=g))][0]
            H, W = sizes[int(torch.randint(0, 5, (1,), generator=g))]
            v = torch.randn(3, generator=g)
            c2w = scenes.look_at(v / v.norm() * 4.0)
            reqs.append(Request(i, name, c2w, H, W, 1.2 * W, arrival=t))
        return reqs

    renderer = GpuRenderer("bf16")
    # capacity: the same kind of requests all available at once (no arrivals to wait for)
    cap_reqs = stream(60, 200.0, 5)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    serve(cap_reqs, res, renderer, realtime=False, max_rays_in_flight=max_rays, chunk_rays=chunk)
    torch.cuda.synchronize()
    cap_s = time.perf_counter() - t0
    capacity = sum(r.rays for r in cap_reqs) / cap_s / 1e6
    out = {"scenes": len(specs), "hbm_budget_gb": 60, "form": "bf16", "resident_gb": res.used / 1e9,
           "reserved_working_gb": res.reserved / 1e9, "capacity_Mrays_per_s": capacity,
           "mean_rays_per_request": mean_rays}
    for tag, n, rate, seed in (("config_200_per_s", args.requests, 200.0, 4),
                               ("sustainable", max(50, args.requests * 3 // 5), 0.6 * capacity * 1e6 / mean_rays, 6)):
        reqs = stream(n, rate, seed)
        torch.cuda.synchronize()
        done = serve(reqs, res, renderer, realtime=True, max_rays_in_flight=max_rays, chunk_rays=chunk)
        torch.cuda.synchronize()
        s = latency_summary(done)
        s.update({"arrival_rate_per_s": rate, "offered_Mrays_per_s": rate * mean_rays / 1e6,
                  "offered_over_capacity": rate * mean_rays / 1e6 / capacity})
        out[tag] = s
    return out


# --- profiling drivers ------------------------------------------------------------

def run_profile(args):
    """`--profile train`: the training scene family on an n^3 grid (--grid),
    batches of 4096 rays, one step of --form captured in a CUDA graph; the
    --profiled replays sit between cudaProfilerStart/Stop, the --timed replays
    after them are printed.  `--profile render`: frames of the n^3 x C scene
    (--grid, --channels) at --size^2 per decoder form (--forms), per-stage
    CUDA-event times printed."""
    import torch

    import diver_gb300.renderer as R
    from diver_gb300 import scenes
    from diver_gb300.graphs import TrainStepGraph
    from diver_gb300.renderer import DIVeRField

    dev = torch.device("cuda")
    if args.profile == "train":
        sc = scenes.grid_scene(args.grid, 32, "diver32", device=dev)
        field = DIVeRField.from_scene(sc, dev)
        batches = scenes.training_batches(sc, 6, BATCH, dev)
        step = TrainStepGraph(field, *batches[0], form=args.form)
        counts = [field.segments(*batches[1 + i % 5][:2]).total for i in range(args.profiled)]
        print(f"segments of the profiled steps: {counts} (total {sum(counts)})", flush=True)
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStart()
        for i in range(args.profiled):
            step(*batches[1 + i % 5])
        torch.cuda.synchronize()
        torch.cuda.cudart().cudaProfilerStop()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for i in range(args.timed):
            step(*batches[i % 6])
        e1.record()
        torch.cuda.synchronize()
        print(f"{args.form} captured step: {e0.elapsed_time(e1) / args.timed:.3f} ms (batch {BATCH}, "
              f"grid {args.grid}^3)", flush=True)
        return
    kind = "diver32" if args.channels == 32 else "diver64"
    sc = scenes.grid_scene(args.grid, args.channels, kind, device=dev)
    field = DIVeRField.from_scene(sc, dev)
    cam = scenes.sphere_cameras(100, 4.0, 3)[0]
    o, d = scenes.camera_rays(cam, args.size, args.size, 1.2 * args.size, dev)

    def ev():
        e = torch.cuda.Event(enable_timing=True)
        e.record()
        return e

    with torch.no_grad():
        for _ in range(args.repeat):
            for form in args.forms.split(","):
                torch.cuda.synchronize()
                R.KERNEL_EVENTS = {}
                e0 = ev()
                seg = field.segments(o, d)
                e1 = ev()
                R.render_segments(field.voxels, field.params, seg, d, kind, True, field.tc_weights(form),
                                  field.grid16(form))
                e2 = ev()
                torch.cuda.synchronize()
                k = {n: round(sum(s.elapsed_time(e) for s, e in v), 3) for n, v in R.KERNEL_EVENTS.items()}
                R.KERNEL_EVENTS = None
                print(f"{form} segments={seg.total} traverse_ms={e0.elapsed_time(e1):.3f} "
                      f"decode_composite_ms={e1.elapsed_time(e2):.3f} {k}", flush=True)


# --- reference arm: CPU oracle port and the reference's GPU path ----------------

def oracle_counter(scene):
    """count_fn for the batch selection that runs the C restatement of the
    masked walk on the host (no use of this repository's CUDA library)."""
    import torch

    from oracle import native as orc

    mask_np = scene.mask.cpu().numpy()

    def count(o, d):
        _, num, _ = orc.masked_walk(o.cpu().numpy(), d.cpu().numpy(), scene.xyzmin, scene.voxel_num,
                                    scene.voxel_size, mask_np, 1.0, max_n=0)
        return torch.from_numpy(num).to(d.device)

    return count


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


def reference_gpu(scene, batches, dev):
    """The reference's GPU path on the same GPU: its own traversal kernels
    (masked_intersect_kernel, built from the reference sources into cubins)
    with the padded [B, 3N, 6] output and the reference's slicing to the
    longest ray, then its torch integrate / decoder / render / loss (the pinned
    torch restatement) on CUDA tensors, autograd backward: one training step of
    a 4096-ray batch, and 800x800 frames (forward only, in chunks of 65,536
    rays).  The reference launches synchronise the device after each kernel,
    as its extension does."""
    import torch

    from oracle import torch_ref
    from oracle.ref_kernels import RefKernels

    rk = RefKernels()
    n = scene.voxel_num
    mask = scene.mask.contiguous()
    layers = [(w.detach().to(dev).clone(), b.detach().to(dev).clone()) for w, b in scene.decoder.layers]

    def segments(o, d):
        inter, num, tns = rk.masked(o, d, scene.xyzmin, scene.xyzmax, n, scene.voxel_size, mask, 1.0)
        K = int(num.max().item()) if num.numel() else 0
        hit = tns[:, :K] >= 0
        seg = inter[:, :K][hit]
        ray = torch.arange(num.numel(), device=dev).repeat_interleave(num.long())
        return seg, ray, num

    def step(i):
        o, d, tgt = batches[i % len(batches)]
        seg, ray, num = segments(o, d)
        V = scene.features.detach().requires_grad_(True)
        L = [(w.requires_grad_(True), b.requires_grad_(True)) for w, b in layers]
        rgb, sigma, _ = torch_ref.forward(V, L, 3, seg, ray, num, d)
        torch_ref.loss(rgb, tgt, sigma).backward()

    ms = _time_steps(step, 2, 5)
    out = {"train_step": {"ms_per_step": ms, "Mrays_per_s": BATCH / (ms * 1e-3) / 1e6, "steps": 5,
                          "form": "reference traversal kernels + torch FP32 path with autograd, on the GPU"}}
    frames = []
    with torch.no_grad():
        for k in range(3):
            o, d = frame_rays(scene, k, dev)
            torch.cuda.synchronize()
            t = time.perf_counter()
            for a in range(0, o.shape[0], 65536):
                oo, dd = o[a:a + 65536].contiguous(), d[a:a + 65536].contiguous()
                seg, ray, num = segments(oo, dd)
                torch_ref.forward(scene.features, layers, 3, seg, ray, num, dd)
            torch.cuda.synchronize()
            if k > 0:
                frames.append((time.perf_counter() - t) * 1e3)
    frames.sort()
    out["render_800"] = {"frame_ms": statistics.median(frames), "frames": len(frames),
                         "Mrays_per_s": 640000 / (statistics.median(frames) * 1e-3) / 1e6,
                         "form": "reference traversal kernels + torch FP32 forward, chunks of 65,536 rays"}
    return out


def run_reference(args, rank, world):
    import torch

    if rank != 0:
        return None
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else torch.device("cpu")
    scene = train_scene(dev)
    # the same batches as our arm (same seeds; the occupied-ray selection by the C oracle walk)
    batches = make_batches(scene, args.warmup + args.steps, dev, count_fn=oracle_counter(scene))
    feat = scene.features.detach().cpu()
    mask_np = scene.mask.cpu().numpy()
    layers = [(w.detach().cpu().clone(), b.detach().cpu().clone()) for w, b in scene.decoder.layers]
    cores = os.cpu_count() or 1
    torch.set_num_threads(cores)
    host = [tuple(x.cpu().numpy() for x in b) for b in batches]
    for i in range(args.warmup):
        cpu_sample_step(feat, mask_np, scene, layers, *host[i])
    t = time.perf_counter()
    for i in range(args.steps):
        cpu_sample_step(feat, mask_np, scene, layers, *host[args.warmup + i])
    sec = time.perf_counter() - t
    value = BATCH * args.steps / sec / 1e6
    line = {
        "metric": METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sec * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "impl": "reference",
        "data": "synthetic: same scene and batches as the GPU arm",
        "config": train_config(1),
        "form": "reference algorithm on the host cores: C restatement of the reference traversal kernels + torch "
                "CPU integrate/decoder/render/loss/autograd (the reference's utils/integrator.py and "
                "model/diver.py:159-207 restated), full 4096-ray batches",
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": cores, "kind": "port",
                         "sample": f"the whole workload: {args.steps} timed steps of 4096-ray batches, fwd+bwd"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if dev.type == "cuda" and not args.no_reference_gpu:
        try:
            line["reference_gpu"] = reference_gpu(scene, batches[args.warmup:], dev)
        except FileNotFoundError as e:
            line["reference_gpu"] = {"unavailable": f"reference kernels not built: {e}"}
    return line


def main():
    args = parse()
    if args.profile:
        run_profile(args)
        return
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
