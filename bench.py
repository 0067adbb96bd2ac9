#!/usr/bin/env python3
"""Benchmark of the REYES core on one GB300 (replicas on N GPUs).

Workload (one step = one frame): mixed4096_1920x1080 -- 4096 patches (2048
bicubic Bezier + 2048 Gregory), centres U[-10,10]^3, lognormal sides, random
orientation, 1920x1080, bound_n_split_limit 8 px, reyes_patch_size 8, rendered
by the batched path (one persistent launch per stage, CUDA-graph replay).

Metric: micropolygons/s = reyes_patch_size^2 x emitted sub-patches per frame
(src/base/Statistics.cpp:175) / frame time.  `value` is device time (CUDA
events on the renderer's stream around each frame, L2 flushed between
frames outside the events); `e2e` is the same metric through the C ABI with
the control points uploaded from pinned host memory and the framebuffer
(colour + depth) read back to pinned host memory inside the timed step.

--impl reference times the reference's CPU path: its CPU bound-and-split and
its dice/shade/sample kernels as restated by the oracle (no OpenCL runtime
exists on this machine), on all host cores, over a bounded sample.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "mixed4096_1920x1080"
METRIC = "micropolygons/s (batched path, 4096-patch mixed Bezier/Gregory scene, 1920x1080)"
L2_FLUSH_BYTES = 256 << 20

# DRAM bytes (read + write) and warp instructions per launch of each stage's
# kernel on this workload, from one ncu capture each (dram__bytes_read.sum +
# dram__bytes_write.sum, smsp__inst_executed.sum; the summaries under
# profiles/), with a hash of the sources the kernel was built from at the
# capture.  A figure whose hash no longer matches the sources describes an
# older kernel and is left out of the bench line.  ncu replays with cold
# caches, so the traffic is an upper bound for a launch inside a frame.
CSRC = os.path.join(ROOT, "micropolis_gb300", "csrc")
KERNEL_SOURCES = {
    "dice_raster": ["mp_raster.cu", "mp_device.cuh", "mp_bns_loop.cuh", "mp_internal.h"],
    "bound_split": ["mp_bns.cu", "mp_device.cuh", "mp_bns_loop.cuh", "mp_internal.h"],
    "resolve_or_shade": ["mp_raster.cu", "mp_device.cuh", "mp_bns_loop.cuh", "mp_internal.h"],
    "canonical_sort_or_sample": ["mp_sort.cu", "mp_bns_loop.cuh", "mp_internal.h"],
}
NCU_FIGURES = {
    # ncu --set full of one frame (profiles/raster_fused_mixed4096_1920x1080.md and the
    # summaries beside it), sources as of the capture
    "dice_raster": {"source": "29884bf2bd105b71", "traffic": 101_184_768 + 66_111_744, "inst": 1_036_109_842},
    "bound_split": {"source": "83928645e25485d2", "traffic": 2_856_960 + 213_277_696, "inst": 171_051_632},
    "resolve_or_shade": {"source": "29884bf2bd105b71", "traffic": 61_478_400 + 6_120_448, "inst": 10_215_932},
    "canonical_sort_or_sample": {"source": "1b09df18b3732cc4", "traffic": 30_085_376 + 6_288_128,
                                 "inst": 33_245_208},
}


def source_hash(stage: str) -> str:
    """SHA-256 (first 16 hex digits) of the sources a stage's kernel is built from."""
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES.get(stage, []):
        with open(os.path.join(CSRC, f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


def ncu_figure(stage: str, key: str):
    """The captured figure `key` ("traffic" or "inst") of a stage's kernel,
    or None when there is none for the current sources."""
    fig = NCU_FIGURES.get(stage)
    if not fig or fig.get("source") != source_hash(stage):
        return None
    return fig.get(key)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-extras", action="store_true", help="skip plain/adjoint/cpu legs")
    ap.add_argument("--all-configs", action="store_true",
                    help="one line per workload (batched, plain, CPU oracle, backward/forward) instead of the bench line")
    ap.add_argument("--workload", action="append", help="with --all-configs: only these workloads")
    ap.add_argument("--no-tune", action="store_true",
                    help="render with the default knob values instead of the autotuner's choice (profiling runs)")
    return ap.parse_args()


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index: int):
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"mpcore_clocks_{os.getpid()}.csv")
        self.index = index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        # nvidia-smi's start-up (driver queries) delays CUDA calls made while it
        # runs: wait for its first sample before the timed region starts
        t0 = time.perf_counter()
        while self.proc and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
            if os.path.exists(self.path) and os.path.getsize(self.path) > 0:
                break
            time.sleep(0.01)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            self.proc.wait()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 7:
                rows.append(parts)
        os.remove(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(x: float, device=None) -> float:
    """The largest value of x over the ranks of the process group (x itself
    when there is no group): the whole job is as slow as its slowest rank."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(units_per_rank: float, seconds_max: float, world: int) -> float:
    """Whole-job throughput of `world` independent replicas (weak scaling):
    the units all ranks processed over the slowest rank's time."""
    return units_per_rank * world / seconds_max


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# --------------------------------------------------------------------------
# CPU baseline (the oracle's restatement of the reference CPU path)

CPU_CHUNKS = 128        # a frame's patches in this many strided chunks, dealt to the cores as they free up
_SCENES = {}


def _cpu_chunk(args):
    """Render one chunk of a frame (every `stride`-th patch of each draw from
    `first`) on one core: bound-and-split, dice, shade and sample.  Returns
    (micropolygons, seconds)."""
    name, first, stride = args
    sys.path.insert(0, ROOT)
    from micropolis_gb300 import scenes
    from oracle import oracle
    if name not in _SCENES:
        _SCENES[name] = scenes.WORKLOADS[name]()
    full = _SCENES[name]
    sc = scenes.Scene(full.name, full.width, full.height,
                      [scenes.Draw(scenes.Mesh(d.mesh.type, d.mesh.cp[first::stride]), d.mv, d.color, d.view)
                       for d in full.draws], fovy=full.fovy, near=full.near, options=full.options)
    t = time.perf_counter()
    _, _, st = oracle.render(sc)
    return st["micropolygons"], time.perf_counter() - t


def cpu_frame(name: str, pool, chunks: int = CPU_CHUNKS):
    """One frame of workload `name` on the CPU: its patches in `chunks`
    strided chunks (chunk c = every chunks-th patch of each draw from patch
    c), dealt to the pool's processes as they free up, so that the
    heavy-tailed cost per patch does not leave cores idle.  Returns
    (micropolygons/s = the frame's micropolygons / wall time, micropolygons,
    wall s)."""
    t = time.perf_counter()
    res = list(pool.imap_unordered(_cpu_chunk, [(name, c, chunks) for c in range(chunks)]))
    wall = time.perf_counter() - t
    mpoly = sum(r[0] for r in res)
    return mpoly / wall, mpoly, wall


def cpu_model() -> str:
    """The host CPU's model name (lscpu; /proc/cpuinfo as a fallback)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform
    return platform.machine()


def cpu_baseline_line(name: str, pool, cores: int, frames: int, warmup: int = 1):
    """The CPU baseline of one workload: `warmup` untimed frames, then the
    best of `frames` timed ones (cpu_frame), with how it was measured."""
    for _ in range(warmup):
        cpu_frame(name, pool)
    runs = [cpu_frame(name, pool) for _ in range(frames)]
    best = max(runs, key=lambda r: r[0])
    return {"value": best[0], "unit": "micropolygons/s", "cores": cores, "kind": "port", "cpu_model": cpu_model(),
            "sample": f"one whole frame of {name} per sample: bound&split+dice+shade+sample of its patches in "
                      f"{CPU_CHUNKS} strided chunks dealt to {cores} processes as they free up; best of {frames} "
                      f"after {warmup} warm-up ({best[1]} micropolygons in {best[2]:.2f} s)",
            "frames_s": [round(r[2], 3) for r in runs]}


def plain_grid_bytes(PS: int, subpatches: int, ms: float) -> dict:
    """Grid traffic of the plain per-pass path, which keeps the reference's
    grids in device memory (src/Reyes/RendererCL.cpp:32-48): per sub-patch
    (PS+1)^2 vertices of float4 position + int2 pixel + float depth, PS^2
    float4 quad colours and (PS/8)^2 int4 block bounds, each written once and
    read once."""
    per = (PS + 1) ** 2 * 28 + PS * PS * 16 + (PS // 8) ** 2 * 16
    total = 2 * per * subpatches
    return {"grid_bytes_per_subpatch": per, "grid_bytes_per_frame": total,
            "grid_gbs": total / (ms / 1e3) / 1e9 if ms > 0 else None}


def cpu_pool(procs: int):
    """Worker processes for the CPU legs, started with spawn (never forked
    from a process that has touched the GPU)."""
    import multiprocessing as mp
    return mp.get_context("spawn").Pool(procs)


# --------------------------------------------------------------------------

def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    cores = os.cpu_count() or 1
    # one step = one whole frame, rendered by all cores (cpu_frame)
    vals = []
    with cpu_pool(cores) as pool:
        pool.map(_cpu_chunk, [(WORKLOAD, 0, 4096)] * cores)   # import, build and make the scene in every worker
        for i in range(args.warmup + args.steps):
            v, mpoly, wall = cpu_frame(WORKLOAD, pool)
            if i >= args.warmup:
                vals.append((v, mpoly, wall))
    value = sum(v[1] for v in vals) / sum(v[2] for v in vals)
    sample = (f"one whole frame per step: bound&split+dice+shade+sample of its 4096 patches in {CPU_CHUNKS} "
              f"strided chunks dealt to {cores} processes as they free up")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "micropolygons/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(v[2] for v in vals),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, no dataset)",
            "config": {"workload": WORKLOAD, "sample": sample},
            "cpu_baseline": {"value": value, "unit": "micropolygons/s", "cores": cores, "kind": "port",
                             "cpu_model": cpu_model(), "sample": sample},
            "e2e": {"value": value, "unit": "micropolygons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def all_configs(args):
    """One JSON line per workload of micropolis_gb300.scenes.WORKLOADS: the
    batched path (autotuned knobs), the plain per-pass path, the oracle on all
    host cores (one frame shared over the cores), and for the displaced
    heightfields the backward / forward ratio."""
    import torch
    from micropolis_gb300 import adjoint, autotune, scenes
    from micropolis_gb300.renderer import render_scene, renderer_for
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    peak_gbs, peak_kind = measured_peaks()
    cores = os.cpu_count() or 1
    pool = cpu_pool(cores)
    pool.map(_cpu_chunk, [("heightfield_1024x768", 0, 64)] * cores)
    atom_peak = None
    for name, make in scenes.WORKLOADS.items():
        if args.workload and name not in args.workload:
            continue
        sc = make()
        tuned = autotune.tune(sc, frames=3, warmup=1, use_cache=False)
        line = {"workload": name, "patches": sc.n_patches, "width": sc.width, "height": sc.height,
                "views": 1 + max(d.view for d in sc.draws), "tuned": tuned.best}
        for path, over in (("batched", tuned.best), ("plain", {})):
            r = renderer_for(sc, path, **over)
            r.set_stream(stream.cuda_stream)
            render_scene(r, sc)
            if atom_peak is None:
                kp = ((1920 + 31) // 32 * 32) * ((1080 + 31) // 32 * 32)
                atom_peak = r.atomic_bench(kp, 1 << 27, 1)
            ms = []
            for _ in range(5 if path == "batched" else 3):
                with torch.cuda.stream(stream):
                    flush.fill_(1.0)
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                render_scene(r, sc)
                b.record(stream)
                torch.cuda.synchronize()
                ms.append(a.elapsed_time(b))
            st = r.stats()
            m = statistics.median(ms)
            cp_alg = sum(d.mesh.n_patches * d.mesh.cp.shape[1] * 12 for d in sc.draws)
            views = line["views"]
            frame_bytes = cp_alg + st["subpatches"] * 20 + views * sc.width * sc.height * (8 + 8 + 16)
            if path == "plain":
                line["plain_grids"] = plain_grid_bytes(int(sc.options.get("reyes_patch_size", 8)),
                                                       st["subpatches"], m)
            line[path] = {"ms_per_frame": m, "micropolygons": st["micropolygons"],
                          "value": st["micropolygons"] / (m / 1e3), "subpatches": st["subpatches"],
                          "fragments": st["fragments"], "passes": st["passes"], "kernels": st["kernels"],
                          "frac_hbm": frame_bytes / (m / 1e3) / 1e9 / peak_gbs,
                          "frac_atomic": st["fragments"] / (m / 1e3) / atom_peak}
            r.close()
        line["batched_over_plain"] = line["batched"]["value"] / line["plain"]["value"]
        line["cpu_baseline"] = cpu_baseline_line(name, pool, cores, frames=3 if sc.n_patches > 10000 else 5)
        if sc.options.get("displacement"):
            line["adjoint"] = adjoint.bench_bwd_fwd(stream, workload=name, steps=5)
        line["peaks"] = {"hbm_gbs": peak_gbs, "hbm_kind": peak_kind, "atomic_per_s": atom_peak}
        print(json.dumps(line), flush=True)
    pool.close()
    return 0


def views64_leg(stream):
    """64 independent 512x512 scenes (100..10000 patches each) in one batched
    frame with the tuned knobs, against the plain per-pass path drawing the
    same 64 layers."""
    import torch
    from micropolis_gb300 import autotune, scenes
    from micropolis_gb300.renderer import render_scene, renderer_for
    sc = scenes.views64_512x512()
    # the tuner also chooses the dice grid (8x8 or 16x16), scored by micropolygons/s
    best = autotune.tune(sc, frames=3, warmup=1, use_cache=False, tune_patch_size=True)
    rates = {}
    for t in best.trials:
        ps = t.options.get("reyes_patch_size", 8)
        rates[ps] = max(rates.get(ps, 0.0), t.micropolygons / (t.ms / 1e3))
    out = {"patches": sc.n_patches, "views": 64, "tuned": best.best,
           "best_rate_by_dice_grid": {f"{k}x{k}": v for k, v in sorted(rates.items())}}
    ps = {"reyes_patch_size": best.best.get("reyes_patch_size", 8)}
    for path, over in (("batched", best.best), ("plain", ps)):
        r = renderer_for(sc, path, **over)
        r.set_stream(stream.cuda_stream)
        render_scene(r, sc)
        ms = []
        for _ in range(5):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            render_scene(r, sc)
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        st = r.stats()
        m = statistics.median(ms)
        out[path] = {"ms_per_frame": m, "value": st["micropolygons"] / (m / 1e3), "micropolygons": st["micropolygons"],
                     "passes": st["passes"]}
        r.close()
    out["batched_over_plain"] = out["batched"]["value"] / out["plain"]["value"]
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    from micropolis_gb300 import build as mpbuild
    mpbuild.build()
    if args.all_configs:
        return all_configs(args) if rank == 0 else 0
    from micropolis_gb300 import scenes
    from micropolis_gb300.renderer import Projection, renderer_for

    from micropolis_gb300 import autotune
    sc = scenes.WORKLOADS[WORKLOAD]()
    stream = torch.cuda.Stream(dev)
    # the autotuner times every knob setting on this frame and picks the fastest
    if args.no_tune:
        tuned = autotune.Result("", dict(autotune.candidates(8)[0]))
    else:
        tuned = autotune.tune(sc, frames=5, warmup=2, use_cache=False)
    r = renderer_for(sc, "batched", **tuned.best)
    r.set_stream(stream.cuda_stream)
    proj = Projection(sc.fovy, sc.near, (sc.width, sc.height))
    handles = [1000 + k for k in range(len(sc.draws))]
    for h, d in zip(handles, sc.draws):
        r.load_patches(h, d.mesh.cp, d.mesh.type)

    def frame():
        r.prepare()
        for h, d in zip(handles, sc.draws):
            r.draw_patches(h, d.mv, proj, d.color)
        r.finish()

    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    # warm-up steps are the timed steps (the flush kernel included: its first
    # launch loads its module, a one-off host cost of up to a few hundred ms)
    for k in range(args.warmup):
        with torch.cuda.stream(stream):
            flush.fill_(float(k))
        frame()
    st0 = r.stats()
    mpoly = st0["micropolygons"]

    # ---- timed region: K frames, device time per frame
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    graph_ms = []
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed")     # the region a profiler's launch list is filtered to
        t_wall = time.perf_counter()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(float(k))           # L2 flush, outside the frame's events
            evs[k][0].record(stream)
            frame()
            evs[k][1].record(stream)
            graph_ms.append(r.stats()["gpu_ms"])
        torch.cuda.synchronize()
        t_wall = time.perf_counter() - t_wall
        torch.cuda.nvtx.range_pop()
    frame_ms = [a.elapsed_time(b) for a, b in evs]
    t_dev = max_over_ranks(sum(frame_ms) / 1e3, dev)
    if world > 1:
        torch.distributed.barrier()
    value = replica_rate(mpoly * args.steps, t_dev, world)
    stats = r.stats()
    _, depth_now = r.read_framebuffer()
    covered = int(np.count_nonzero(depth_now != 0x7FFFFFFF))

    # ---- e2e: host buffers through the C ABI (pinned), copies inside each step.
    # Each step uploads the control points, renders, and starts the read-back
    # of its colour and depth, which overlaps the next step's frame (two host
    # buffers); the timed region ends when the last step's result is in host
    # memory.
    W, H = sc.width, sc.height
    host_cp = [torch.from_numpy(np.ascontiguousarray(d.mesh.cp, np.float32)).pin_memory().numpy()
               for d in sc.draws]
    col_host = [torch.empty((W * H, 4), dtype=torch.float32).pin_memory().numpy() for _ in range(2)]
    dep_host = [torch.empty((W * H,), dtype=torch.int32).pin_memory().numpy() for _ in range(2)]
    h2d = sum(int(c.nbytes) for c in host_cp)          # xyz, widened to (x, y, z, 1) on the device
    d2h = W * H * 16 + W * H * 4

    def e2e_step(k):
        for h, c, d in zip(handles, host_cp, sc.draws):
            r.load_patches(h, c, d.mesh.type)
        r.prepare()
        for h, d in zip(handles, sc.draws):
            r.draw_patches(h, d.mv, proj, d.color)
        r.finish()
        # the read-back of step k - 1 (buffer (k - 1) % 2) may still be in flight: it
        # is waited for by this request, which reuses the staging layer
        r.read_framebuffer_async(0, col_host[k % 2].ctypes.data, dep_host[k % 2].ctypes.data)

    for k in range(2):
        e2e_step(k)
    r.wait_read_framebuffer()
    torch.cuda.synchronize()
    t_e2e = time.perf_counter()
    for k in range(args.steps):
        e2e_step(k)
    r.wait_read_framebuffer()
    t_e2e = time.perf_counter() - t_e2e
    e2e_value = replica_rate(mpoly * args.steps, max_over_ranks(t_e2e, dev), world)
    # the last step's read-back equals the device framebuffer
    col_chk, dep_chk = r.read_framebuffer()
    e2e_checked = bool(np.array_equal(dep_chk, dep_host[(args.steps - 1) % 2]) and
                       np.array_equal(col_chk.view(np.uint32), col_host[(args.steps - 1) % 2].view(np.uint32)))

    # ---- stage timing pass (same frame, stages as separate launches)
    r.set_stage_timing(True)
    stage = {k: [] for k in r.STAGES}
    for _ in range(5):
        with torch.cuda.stream(stream):
            flush.fill_(1.0)
        frame()
        for k, v in r.stats()["stage_ms"].items():
            stage[k].append(v)
    r.set_stage_timing(False)
    stage_ms = {k: statistics.median(v) for k, v in stage.items() if max(v) > 0}
    dominant = max(stage_ms, key=stage_ms.get)

    # atomic roofline: fragments resolved by 64-bit atomicMin in the dice+raster
    # stage against the device's measured atomicMin rate on a buffer of the
    # key buffer's size (uniform random slots and 8x8-tile locality)
    key_slots = ((W + 31) // 32 * 32) * ((H + 31) // 32 * 32)
    atom_peak = {"random": r.atomic_bench(key_slots, 1 << 27, 0), "tiled": r.atomic_bench(key_slots, 1 << 27, 1)}

    peak_gbs, peak_kind = measured_peaks()
    n_cp_bytes = sum(d.mesh.n_patches * d.mesh.cp.shape[1] * 16 for d in sc.draws)
    S = stats["subpatches"]
    frags = stats["fragments"]
    # algorithmic bytes of the dice+raster kernel: sub-patch records (24 B),
    # control points once (16 B per point), one 8-byte atomic per fragment
    # Algorithmic work (bytes that must cross HBM once, and depth|id atomics):
    # control points 12 B per point (xyz) read once, 20 B per sub-patch record
    # written by bound-and-split and read by dice+raster, 8 B per pixel for the
    # key clear, 8 B key + 16 B colour + 4 B depth per pixel for the resolve.
    cp_alg = sum(d.mesh.n_patches * d.mesh.cp.shape[1] * 12 for d in sc.draws)
    alg = {"dice_raster": cp_alg + S * 20,
           "bound_split": cp_alg + S * 20 + stats["bounds"] * (28 + 80),
           "resolve_or_shade": W * H * (8 + 16 + 4),
           "clear": W * H * 8,
           "raster_big": 0}
    dom_bytes = alg.get(dominant, 0)
    dom_s = stage_ms[dominant] / 1e3
    achieved = dom_bytes / dom_s / 1e9 if dom_s > 0 else 0.0
    raster_s = stage_ms.get("dice_raster", 0.0) / 1e3
    atom_rate = frags / raster_s if raster_s > 0 else 0.0
    frame_s = t_dev / args.steps
    frame_bytes = cp_alg + S * 20 + W * H * (8 + 8 + 16)
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                "frac": achieved / peak_gbs, "traffic": ncu_figure(dominant, "traffic"),
                "traffic_source": source_hash(dominant), "peak_kind": peak_kind,
                "stage_ms": stage_ms, "alg_bytes": dom_bytes,
                "atomic": {"kernel": "dice_raster", "achieved": atom_rate, "peak": atom_peak["tiled"],
                           "peak_random": atom_peak["random"], "unit": "atomicMin/s",
                           "frac": atom_rate / atom_peak["tiled"] if atom_peak["tiled"] else None},
                "frame": {"alg_bytes": frame_bytes, "atomics": frags, "ms": 1e3 * frame_s,
                          "frac_hbm": frame_bytes / frame_s / 1e9 / peak_gbs,
                          "frac_atomic": frags / frame_s / atom_peak["tiled"] if atom_peak["tiled"] else None},
                "note": "dice+raster is issue-bound (FP32/ALU instruction issue), not HBM- or atomic-bound"}
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    clk = clk.summary()
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz") or 0
    inst = ncu_figure(dominant, "inst")
    if inst and mhz and dom_s > 0:
        peak_issue = sms * 4 * mhz * 1e6
        roofline["issue"] = {"kernel": dominant, "achieved": inst / dom_s, "peak": peak_issue,
                             "unit": "warp instructions/s", "frac": inst / dom_s / peak_issue,
                             "sms": sms, "sm_mhz": mhz}

    extras = {}
    if not args.no_extras and rank == 0:
        # plain per-pass path on the same frame
        rp = renderer_for(sc, "plain")
        rp.set_stream(stream.cuda_stream)
        for h, d in zip(handles, sc.draws):
            rp.load_patches(h, d.mesh.cp, d.mesh.type)

        def pframe():
            rp.prepare()
            for h, d in zip(handles, sc.draws):
                rp.draw_patches(h, d.mv, proj, d.color)
            rp.finish()

        for _ in range(2):
            pframe()
        pms = []
        for _ in range(max(3, args.steps // 4)):
            with torch.cuda.stream(stream):
                flush.fill_(2.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pframe()
            b.record(stream)
            torch.cuda.synchronize()
            pms.append(a.elapsed_time(b))
        pst = rp.stats()
        plain_ms = statistics.mean(pms)
        extras["plain"] = {"ms_per_frame": plain_ms, "value": pst["micropolygons"] / (plain_ms / 1e3),
                           "passes": pst["passes"], "micropolygons": pst["micropolygons"],
                           **plain_grid_bytes(8, pst["subpatches"], plain_ms)}
        extras["batched_over_plain"] = value / extras["plain"]["value"]
        rp.close()
        # backward / forward on the displaced heightfields: 16x16 patches at
        # 512x512 and 512x512 patches at 3840x2160
        from micropolis_gb300 import adjoint
        for key, wl, n in (("adjoint", "heightfield16_512x512", 10), ("adjoint_4k", "heightfield512_3840x2160", 5)):
            try:
                extras[key] = adjoint.bench_bwd_fwd(stream, steps=n, workload=wl)
            except Exception as e:  # noqa: BLE001
                extras[key] = {"error": str(e)[:200]}
        extras["views64"] = views64_leg(stream)
        # CPU baseline: whole frames on the host cores, the same definition as --impl reference
        cores = os.cpu_count() or 1
        with cpu_pool(cores) as pool:
            extras["cpu_baseline"] = cpu_baseline_line(WORKLOAD, pool, cores, frames=5)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "micropolygons/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded generator, no dataset)",
                "config": {"workload": WORKLOAD, "patches": sc.n_patches, "width": W, "height": H,
                           "bound_n_split_limit": 8, "reyes_patch_size": 8, "path": "batched (CUDA graph)",
                           "parallelism": f"replicas x{world}", "l2": "flushed (256 MiB write) between frames",
                           "micropolygons_per_frame": mpoly, "subpatches": S, "fragments": frags,
                           "fragments_per_pixel": frags / (W * H),
                           "depth_complexity_covered": frags / max(covered, 1), "bounds": stats["bounds"],
                           "graph_ms_median": statistics.median(graph_ms),
                           "tuned": tuned.best,
                           # host wall clock of the device-timed loop, which also issues each
                           # frame's L2 flush, two events and a stats read (e2e is the API's wall time)
                           "timed_loop_wall_ms_per_frame": 1e3 * t_wall / args.steps},
                "e2e": {"value": e2e_value, "unit": "micropolygons/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * t_e2e / args.steps,
                        "readback": "asynchronous (mp_read_framebuffer_async), overlapping the next step's frame",
                        "result_checked": e2e_checked},
                "gpu_launches": stats["kernels"] * args.steps,
                "roofline": roofline,
                "clocks": clk}
        if "cpu_baseline" in extras:
            line["cpu_baseline"] = extras.pop("cpu_baseline")
        line.update(extras)
        print(json.dumps(line))
    r.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
