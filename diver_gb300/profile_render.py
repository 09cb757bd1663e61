"""Small render driver for profiling: renders frames of the 256^3 x 32 DIVeR32
scene with chosen decoder forms and prints per-stage CUDA-event times.

    python -m diver_gb300.profile_render --size 200 --forms fp32,bf16 --repeat 2
"""
from __future__ import annotations

import argparse


def main():
    import torch

    import diver_gb300.renderer as R
    from diver_gb300 import scenes
    from diver_gb300.renderer import DIVeRField

    p = argparse.ArgumentParser()
    p.add_argument("--size", type=int, default=800)
    p.add_argument("--forms", default="fp32,bf16")
    p.add_argument("--repeat", type=int, default=2)
    p.add_argument("--channels", type=int, default=32)
    args = p.parse_args()
    dev = torch.device("cuda")
    kind = "diver32" if args.channels == 32 else "diver64"
    sc = scenes.grid_scene(256, args.channels, kind, device=dev)
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


if __name__ == "__main__":
    main()
