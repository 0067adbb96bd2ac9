"""Renders frames of one of the synthetic workloads from the command line --
the analogue of the reference's main loop drawing a scene (src/micropolis/
main.cpp, Scene::draw) without a window:

    python -m micropolis_gb300.render --workload mixed4096_1920x1080 \\
        [--path batched|plain] [--frames N] [--warmup W] [--overlap] \\
        [--backward] [--ppm out.ppm] [--option name=value ...] \\
        [--scene name=value ...]

--scene passes arguments to the workload's generator (for instance
n_views=8 for views64_512x512, n=256 for mixed4096_1920x1080): smaller
instances of a workload for profiling captures.

The timed frames run inside the NVTX range "frames" (a profiler's launch list
can be filtered to them); each frame's device time (CUDA events on the
renderer's stream) and micropolygons/s are printed.  --backward also runs
the adjoint pass of an L2 image loss after each frame (the workload's
displacement amplitude and a target rendered from perturbed control points),
inside the same range.
"""
from __future__ import annotations

import argparse
import json
import statistics


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m micropolis_gb300.render")
    ap.add_argument("--workload", default="mixed4096_1920x1080")
    ap.add_argument("--path", default="batched", choices=["batched", "plain"])
    ap.add_argument("--frames", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--overlap", action="store_true", help="batched path: bound-and-split and raster in one launch")
    ap.add_argument("--backward", action="store_true", help="the adjoint pass after every frame")
    ap.add_argument("--ppm", help="write the last frame's displayed image here")
    ap.add_argument("--option", action="append", default=[], help="reyes option override, name=value")
    ap.add_argument("--scene", action="append", default=[], help="workload generator argument, name=value")
    args = ap.parse_args(argv)

    import torch
    from . import scenes
    from .renderer import render_scene, renderer_for

    gen = {}
    for kv in args.scene:
        k, _, v = kv.partition("=")
        gen[k] = float(v) if "." in v else int(v)
    sc = scenes.WORKLOADS[args.workload](**gen)
    over = {}
    for kv in args.option:
        k, _, v = kv.partition("=")
        over[k] = float(v) if "." in v else int(v)
    if args.overlap:
        over["overlap"] = 1
    stream = torch.cuda.Stream()
    if args.backward:
        from . import adjoint
        import numpy as np
        sc.options.update({k: v for k, v in over.items()})
        dr = adjoint.DiffRenderer(sc)
        dr.r.set_stream(stream.cuda_stream)
        dev = torch.device("cuda")
        cp0 = torch.tensor(sc.draws[0].mesh.cp, device=dev)
        rng = np.random.default_rng(sc.seed + 100)
        sigma = 0.05 * 16.0 / max(16.0, float(np.sqrt(sc.n_patches)))
        with torch.cuda.stream(stream):
            cpt = cp0 + torch.tensor(rng.normal(0, sigma, size=cp0.shape).astype(np.float32), device=dev)
            target = dr.render(cpt, 1.2).clone()
        r = dr.r

        def frame():
            with torch.cuda.stream(stream):
                img = dr.render(cp0, 1.0)
                dr.backward(2 * (img - target), tuple(cp0.shape), dev)
    else:
        r = renderer_for(sc, args.path, **over)
        r.set_stream(stream.cuda_stream)

        def frame():
            render_scene(r, sc)

    for _ in range(args.warmup):
        frame()
    torch.cuda.synchronize()
    ms = []
    torch.cuda.nvtx.range_push("frames")
    for _ in range(args.frames):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        frame()
        b.record(stream)
        torch.cuda.synchronize()
        ms.append(a.elapsed_time(b))
    torch.cuda.nvtx.range_pop()
    st = r.stats()
    m = statistics.median(ms)
    print(json.dumps({"workload": args.workload, "path": args.path, "overlap": args.overlap,
                      "backward": args.backward, "ms_per_frame": m, "micropolygons": st["micropolygons"],
                      "micropolygons_per_s": st["micropolygons"] / (m / 1e3), "subpatches": st["subpatches"],
                      "fragments": st["fragments"], "passes": st["passes"], "kernels": st["kernels"]}))
    if args.ppm:
        r.save_ppm(args.ppm)
    r.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
