"""Autotuner for the batched path.

It picks, per workload shape, the values of the knobs that change speed but
not the rendered sub-patch set:

- ``dice_group``: sub-patches one fused block claims from the emitted
  sub-patch queue, dices, shades and rasterizes at a time (the queue chunk of
  the dice/raster stage; 8, 11, 16 or 22 for 8x8 dicing, 2, 3, 4 or 6 for
  16x16; 11 and 3 run 128-thread blocks, the others 256);
- ``raster_tile``: the tile edge, in pixels, of the depth|id key buffer that
  the 64-bit atomicMin resolves visibility in (8, 16 or 32);
- ``overlap``: bound-and-split and rasterization in one launch, with the
  rasterizing blocks consuming sub-patches as they are emitted, or separate
  launches with the canonical sub-patch order between them.  The overlapped
  form numbers micropolygons in emission order, so its depth-tie winners
  depend on scheduling; it is a candidate only with ``allow_overlap``;
- optionally ``reyes_patch_size`` (the dice grid, 8 or 16).  The dice grid
  sets how many micropolygons each sub-patch makes, so the image changes with
  it; it is tuned only when asked for, and the score is then micropolygons
  per second instead of frame time.

Choices are cached in a JSON file keyed by the workload's shape (window,
views, patch counts by type, split limit, dice grid, displacement) and the
device, the way the reference caches its configuration under a hash of the
options (src/micropolis/main.cpp:495-567).  The cache file is
``$MICROPOLIS_GB300_AUTOTUNE_CACHE`` or ``~/.cache/micropolis_gb300/autotune.json``.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
from dataclasses import dataclass, field
from typing import Callable, Dict, Iterable, List, Optional

GROUPS = {8: (8, 11, 16, 22), 16: (2, 3, 4, 6)}
DEFAULT_GROUP = {8: 11, 16: 6}   # the library's default dice_group per dice grid
TILES = (8, 16, 32)
OVERLAP = (False, True)       # the values tried with allow_overlap
CACHE_VERSION = 1


def cache_path() -> str:
    p = os.environ.get("MICROPOLIS_GB300_AUTOTUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "micropolis_gb300", "autotune.json")


def _bucket(n: int) -> int:
    """Patch counts enter the key rounded to a power of two, so scenes that
    differ by a few patches share a choice."""
    return 0 if n <= 0 else 1 << (int(n) - 1).bit_length()


def signature(scene, options: Optional[dict] = None, device: str = "") -> str:
    """Key of a workload: what the kernels' balance depends on, not the values
    of the control points."""
    o = dict(scene.options)
    o.update(options or {})
    counts: Dict[str, int] = {}
    for d in scene.draws:
        k = "bezier" if int(d.mesh.type) == 0 else "gregory"
        counts[k] = counts.get(k, 0) + len(d.mesh.cp)
    views = 1 + max((int(d.view) for d in scene.draws), default=0)
    key = {
        "v": CACHE_VERSION,
        "window": [int(scene.width), int(scene.height)],
        "views": views,
        "draws": _bucket(len(scene.draws)),
        "patches": {k: _bucket(v) for k, v in sorted(counts.items())},
        "limit": float(o.get("bound_n_split_limit", 8.0)),
        "patch_size": int(o.get("reyes_patch_size", 8)),
        "displacement": bool(o.get("displacement", False)),
        "device": device,
    }
    return hashlib.sha1(json.dumps(key, sort_keys=True).encode()).hexdigest()[:16]


def candidates(patch_size: int = 8, tune_patch_size: bool = False,
               groups: Optional[Iterable[int]] = None, tiles: Iterable[int] = TILES,
               overlap: Iterable[bool] = OVERLAP) -> List[dict]:
    """The search space, in a fixed order (defaults first)."""
    sizes = (8, 16) if tune_patch_size else (patch_size,)
    out = []
    for ps in sizes:
        gs = tuple(groups) if groups is not None else GROUPS[ps]
        gs = tuple(sorted(gs, key=lambda g: g != DEFAULT_GROUP[ps]))   # the default group first
        for g, t, ov in itertools.product(gs, tiles, overlap):
            c = {"dice_group": int(g), "raster_tile": int(t), "overlap": bool(ov)}
            if tune_patch_size:
                c["reyes_patch_size"] = ps
            out.append(c)
    return out


@dataclass
class Trial:
    options: dict
    ms: float
    micropolygons: int

    @property
    def mpps(self) -> float:
        return self.micropolygons / (self.ms * 1e-3) if self.ms > 0 else 0.0


@dataclass
class Result:
    key: str
    best: dict
    trials: List[Trial] = field(default_factory=list)
    cached: bool = False


MARGIN = 0.01


def choose(trials: List[Trial], by_rate: bool, margin: float = MARGIN) -> Trial:
    """Lowest frame time, or highest micropolygon rate when the dice grid is
    among the knobs.  Among the trials within `margin` (relative) of the best
    score, the earliest candidate wins: the search space lists the defaults
    and the simpler settings first, and the choice does not flip between runs
    on differences below the timing noise."""
    if not trials:
        raise ValueError("no trials")
    score = [(t.mpps if by_rate else -t.ms) for t in trials]
    top = max(score)
    tol = abs(top) * margin
    for t, v in zip(trials, score):
        if v >= top - tol:
            return t
    return trials[0]


def load_cache(path: Optional[str] = None) -> dict:
    path = path or cache_path()
    try:
        with open(path) as f:
            data = json.load(f)
        return data if isinstance(data, dict) and data.get("version") == CACHE_VERSION else {"version": CACHE_VERSION}
    except (OSError, ValueError):
        return {"version": CACHE_VERSION}


def save_cache(data: dict, path: Optional[str] = None) -> None:
    path = path or cache_path()
    d = os.path.dirname(path)
    if d:
        os.makedirs(d, exist_ok=True)
    tmp = path + ".tmp%d" % os.getpid()
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def measure_batched(scene, options: dict, frames: int, warmup: int) -> Trial:
    """Frame time of the batched path with these options: the median of
    `frames` frames, each timed with CUDA events around the frame's graph."""
    from .renderer import render_scene, renderer_for
    r = renderer_for(scene, "batched", **options)
    try:
        for _ in range(warmup):
            render_scene(r, scene)
        ms = []
        for _ in range(frames):
            render_scene(r, scene)
            ms.append(r.stats()["gpu_ms"])
        mp = r.stats()["micropolygons"]
    finally:
        r.close()
    ms.sort()
    return Trial(dict(options), ms[len(ms) // 2], int(mp))


def device_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            p = torch.cuda.get_device_properties(torch.cuda.current_device())
            return "%s/%d" % (p.name, p.multi_processor_count)
    except Exception:
        pass
    return ""


def tune(scene, frames: int = 5, warmup: int = 2, tune_patch_size: bool = False, allow_overlap: bool = False,
         cache: Optional[str] = None,
         use_cache: bool = True, space: Optional[List[dict]] = None,
         measure: Optional[Callable[[object, dict, int, int], Trial]] = None, device: Optional[str] = None) -> Result:
    """Times every candidate on `scene` and returns (and caches) the fastest."""
    ps = int(scene.options.get("reyes_patch_size", 8))
    dev = device_name() if device is None else device
    key = signature(scene, None, dev) + ("+ps" if tune_patch_size else "") + ("+overlap" if allow_overlap else "")
    data = load_cache(cache) if use_cache else {"version": CACHE_VERSION}
    if use_cache and key in data:
        e = data[key]
        return Result(key, dict(e["best"]), [Trial(dict(t["options"]), t["ms"], t["micropolygons"])
                                            for t in e.get("trials", [])], cached=True)
    measure = measure or measure_batched
    space = space if space is not None else candidates(ps, tune_patch_size,
                                                       overlap=OVERLAP if allow_overlap else (False,))
    trials = [measure(scene, c, frames, warmup) for c in space]
    best = choose(trials, by_rate=tune_patch_size)
    if use_cache:
        data = load_cache(cache)
        data[key] = {"best": best.options,
                     "trials": [{"options": t.options, "ms": t.ms, "micropolygons": t.micropolygons} for t in trials],
                     "window": [scene.width, scene.height]}
        save_cache(data, cache)
    return Result(key, dict(best.options), trials)


def tuned_renderer(scene, **kw):
    """A batched renderer with the tuned options for this scene's shape."""
    from .renderer import renderer_for
    res = tune(scene, **kw)
    return renderer_for(scene, "batched", **res.best)
