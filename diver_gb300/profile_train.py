"""Training-step driver for profiling: the 256^3 x 32 DIVeR32 scene, batches
of 4096 rays that hit occupied voxels, one step captured in a CUDA graph
(diver_gb300.graphs.TrainStepGraph) and replayed.  The replays between
cudaProfilerStart/Stop are the ones a profiler started with
--profile-from-start off records; the timed replays after them are printed.

    python -m diver_gb300.profile_train --form bf16 --profiled 3 --timed 20 [--grid 128]

--grid selects a smaller n^3 x 32 grid of the same scene family (for profiler
captures that replay kernels many times).
"""
from __future__ import annotations

import argparse


def main():
    import torch

    from diver_gb300 import scenes
    from diver_gb300.graphs import TrainStepGraph
    from diver_gb300.renderer import DIVeRField

    p = argparse.ArgumentParser()
    p.add_argument("--form", default="bf16")
    p.add_argument("--batch", type=int, default=4096)
    p.add_argument("--profiled", type=int, default=3)
    p.add_argument("--timed", type=int, default=20)
    p.add_argument("--grid", type=int, default=256)
    args = p.parse_args()
    dev = torch.device("cuda")
    sc = scenes.grid_scene(args.grid, 32, "diver32", device=dev)
    field = DIVeRField.from_scene(sc, dev)
    batches = scenes.training_batches(sc, 6, args.batch, dev)
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
    print(f"{args.form} captured step: {e0.elapsed_time(e1) / args.timed:.3f} ms (batch {args.batch}, "
          f"grid {args.grid}^3)", flush=True)


if __name__ == "__main__":
    main()
