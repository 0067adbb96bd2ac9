"""ctypes binding of the CPU oracle: TEST INFRASTRUCTURE ONLY.

Imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg,
as the checker or the timed CPU baseline; never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_PIN_PATH = os.path.join(HERE, "_ref", "libref_pin.so")

f32p = ctypes.POINTER(ctypes.c_float)
i32p = ctypes.POINTER(ctypes.c_int32)
i64p = ctypes.POINTER(ctypes.c_int64)
f64p = ctypes.POINTER(ctypes.c_double)


class OrDraw(ctypes.Structure):
    _fields_ = [("cp", f32p), ("n_patches", ctypes.c_int32), ("type", ctypes.c_int32),
                ("mv", ctypes.c_float * 16), ("color", ctypes.c_float * 4)]


class OrParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32),
                ("fovy_deg", ctypes.c_float), ("near_plane", ctypes.c_float),
                ("bound_n_split_limit", ctypes.c_float), ("cull_ribbon", ctypes.c_float),
                ("max_split_depth", ctypes.c_int32), ("reyes_patches_per_pass", ctypes.c_int32),
                ("reyes_patch_size", ctypes.c_int32), ("subpixel_bits", ctypes.c_int32),
                ("backface_culling", ctypes.c_int32), ("displacement", ctypes.c_int32),
                ("displacement_amplitude", ctypes.c_float), ("clear_color", ctypes.c_float * 4),
                ("bound_criterion", ctypes.c_int32)]


def build() -> None:
    subprocess.check_call(["sh", os.path.join(HERE, "build.sh")], stdout=subprocess.DEVNULL)


def build_ref() -> None:
    subprocess.check_call(["sh", os.path.join(HERE, "build_ref.sh")], stdout=subprocess.DEVNULL)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        L.or_bound_n_split.restype = ctypes.c_int64
        L.or_bound_n_split.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), i32p, f32p,
                                       ctypes.c_int64, i64p]
        L.or_render.restype = ctypes.c_int
        L.or_render.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32, f32p,
                                i32p, i64p]
        L.or_render_win.restype = ctypes.c_int
        L.or_render_win.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32, f32p,
                                    i32p, i64p, i64p]
        L.or_canonical_subpatches.restype = ctypes.c_int64
        L.or_canonical_subpatches.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32,
                                              i32p, i32p, f32p, ctypes.POINTER(ctypes.c_uint64), ctypes.c_int64]
        L.or_render_subpatches_at.restype = ctypes.c_int
        L.or_render_subpatches_at.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32,
                                              ctypes.c_int64, ctypes.c_int64, i32p, i32p, f32p, f32p, i32p, i64p,
                                              i64p]
        L.or_render_subpatches.restype = ctypes.c_int
        L.or_render_subpatches.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32,
                                           ctypes.c_int64, i32p, i32p, f32p, f32p, i32p, i64p, i64p]
        L.or_dice.restype = None
        L.or_dice.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32, f32p, f32p,
                              i32p, f32p]
        L.or_shade_quads.restype = None
        L.or_shade_quads.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32, f32p, f32p]
        L.or_dice_fp64.restype = None
        L.or_dice_fp64.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int32, f32p,
                                   f64p]
        L.or_loss_fp64.restype = ctypes.c_double
        L.or_loss_fp64.argtypes = [ctypes.POINTER(OrParams), ctypes.POINTER(OrDraw), ctypes.c_int64, i32p,
                                   f32p, i64p, f32p, f64p, ctypes.c_double, f64p, f64p]
        L.or_sinf.restype = ctypes.c_float
        L.or_sinf.argtypes = [ctypes.c_float]
        L.or_cosf.restype = ctypes.c_float
        L.or_cosf.argtypes = [ctypes.c_float]
        L.or_inclusive_scan.restype = None
        L.or_inclusive_scan.argtypes = [i32p, i32p, ctypes.c_int64]
        _lib = L
    return _lib


def _ptr(a, t):
    return a.ctypes.data_as(t)


def make_params(scene, **over) -> OrParams:
    o = dict(bound_n_split_limit=8.0, cull_ribbon=32.0, max_split_depth=23, reyes_patches_per_pass=100000,
             reyes_patch_size=8, subpixel_bits=6, backface_culling=1, displacement=0,
             displacement_amplitude=1.0, clear_color=(0.1, 0.1, 0.7, 0.0), bound_criterion=0)
    o.update({k: v for k, v in scene.options.items() if k in o})
    o.update(over)
    p = OrParams()
    p.width, p.height = scene.width, scene.height
    p.fovy_deg, p.near_plane = scene.fovy, scene.near
    for k in ("bound_n_split_limit", "cull_ribbon", "displacement_amplitude"):
        setattr(p, k, float(o[k]))
    for k in ("max_split_depth", "reyes_patches_per_pass", "reyes_patch_size", "subpixel_bits",
              "backface_culling", "displacement", "bound_criterion"):
        setattr(p, k, int(o[k]))
    for i in range(4):
        p.clear_color[i] = o["clear_color"][i]
    return p


class _Draws:
    """Keeps the numpy buffers alive while the oracle reads them."""

    def __init__(self, draws):
        self.keep = []
        self.arr = (OrDraw * max(1, len(draws)))()
        for k, d in enumerate(draws):
            cp = np.ascontiguousarray(d.mesh.cp, np.float32).reshape(-1)
            self.keep.append(cp)
            self.arr[k].cp = _ptr(cp, f32p)
            self.arr[k].n_patches = d.mesh.n_patches
            self.arr[k].type = d.mesh.type
            for i in range(16):
                self.arr[k].mv[i] = float(d.mv[i])
            for i in range(4):
                self.arr[k].color[i] = float(d.color[i])
        self.n = len(draws)


def bound_n_split(scene, draw_index=0, params=None, cap=None):
    """Reference-order sub-patches of one draw: (pid int32[S], range float32[S,4], n_bounds)."""
    p = params or make_params(scene)
    ds = _Draws([scene.draws[draw_index]])
    n_b = ctypes.c_int64(0)
    n = lib().or_bound_n_split(ctypes.byref(p), ds.arr, None, None, 0, ctypes.byref(n_b))
    cap = n if cap is None else cap
    pid = np.zeros(max(cap, 1), np.int32)
    rng = np.zeros((max(cap, 1), 4), np.float32)
    lib().or_bound_n_split(ctypes.byref(p), ds.arr, _ptr(pid, i32p), _ptr(rng, f32p), cap, ctypes.byref(n_b))
    return pid[:n], rng[:n], int(n_b.value)


def render(scene, params=None, draws=None, want_win=False):
    """Full frame with micropolygons numbered in the canonical order:
    (tiled colour float32[W*H,4], tiled depth int32[W*H], stats dict), and
    with want_win the winning micropolygon number of every tiled pixel
    (int64, -1 where none) before the stats."""
    p = params or make_params(scene)
    draws = scene.draws if draws is None else draws
    ds = _Draws(draws)
    npx = scene.width * scene.height
    color = np.zeros((npx, 4), np.float32)
    depth = np.zeros(npx, np.int32)
    win = np.zeros(npx, np.int64) if want_win else None
    st = np.zeros(4, np.int64)
    rc = lib().or_render_win(ctypes.byref(p), ds.arr, ds.n, _ptr(color, f32p), _ptr(depth, i32p),
                             _ptr(win, i64p) if want_win else None, _ptr(st, i64p))
    if rc:
        raise ValueError(f"oracle render failed: {rc}")
    stats = dict(subpatches=int(st[0]), micropolygons=int(st[1]), fragments=int(st[2]), bounds=int(st[3]))
    return (color, depth, win, stats) if want_win else (color, depth, stats)


def canonical_subpatches(scene, params=None):
    """Every draw's sub-patches in the canonical order (ascending root, then
    split path): (draw int32[S], pid int32[S], range float32[S,4], key uint64[S])."""
    p = params or make_params(scene)
    ds = _Draws(scene.draws)
    n = lib().or_canonical_subpatches(ctypes.byref(p), ds.arr, ds.n, None, None, None, None, 0)
    m = max(n, 1)
    draw = np.zeros(m, np.int32)
    pid = np.zeros(m, np.int32)
    rng = np.zeros((m, 4), np.float32)
    key = np.zeros(m, np.uint64)
    lib().or_canonical_subpatches(ctypes.byref(p), ds.arr, ds.n, _ptr(draw, i32p), _ptr(pid, i32p), _ptr(rng, f32p),
                                  key.ctypes.data_as(ctypes.POINTER(ctypes.c_uint64)), n)
    return draw[:n], pid[:n], rng[:n], key[:n]


def _render_slice(args):
    """One process's share of render_parallel: the canonical sub-patches
    [first, first + len) of the frame, numbered from first."""
    scene, params_over, first, sdraw, spid, srange = args
    p = make_params(scene, **params_over)
    ds = _Draws(scene.draws)
    npx = scene.width * scene.height
    color = np.zeros((npx, 4), np.float32)
    depth = np.zeros(npx, np.int32)
    win = np.zeros(npx, np.int64)
    st = np.zeros(4, np.int64)
    sd = np.ascontiguousarray(sdraw, np.int32)
    sp = np.ascontiguousarray(spid, np.int32)
    sr = np.ascontiguousarray(srange, np.float32).reshape(-1)
    rc = lib().or_render_subpatches_at(ctypes.byref(p), ds.arr, ds.n, len(sp), int(first), _ptr(sd, i32p),
                                       _ptr(sp, i32p), _ptr(sr, f32p), _ptr(color, f32p), _ptr(depth, i32p),
                                       _ptr(win, i64p), _ptr(st, i64p))
    if rc:
        raise ValueError(f"oracle render failed: {rc}")
    return color, depth, win, int(st[2])


def render_parallel(scene, pool, params_over=None, slices=None):
    """The frame of render(scene, want_win=True), computed by `pool`
    (multiprocessing, spawn context) over slices of the canonical list and
    merged by the smallest (depth, micropolygon number) per pixel -- the rule
    one sequential pass keeps, so the merge is exact."""
    params_over = params_over or {}
    p = make_params(scene, **params_over)
    draw, pid, rng, _ = canonical_subpatches(scene, p)
    n = len(pid)
    k = max(1, min(slices or getattr(pool, "_processes", 1) * 4, n))
    bounds = [n * i // k for i in range(k + 1)]
    jobs = [(scene, params_over, bounds[i], draw[bounds[i]:bounds[i + 1]], pid[bounds[i]:bounds[i + 1]],
             rng[bounds[i]:bounds[i + 1]]) for i in range(k)]
    parts = pool.map(_render_slice, jobs)
    color, depth, win, frags = parts[0][0].copy(), parts[0][1].copy(), parts[0][2].copy(), parts[0][3]
    for c, d, w, f in parts[1:]:
        # pixels of a later slice replace only at smaller depth, or equal depth and smaller number
        take = (d < depth) | ((d == depth) & (w >= 0) & ((win < 0) | (w < win)))
        color[take] = c[take]
        depth[take] = d[take]
        win[take] = w[take]
        frags += f
    stats = dict(subpatches=n, micropolygons=n * p.reyes_patch_size ** 2, fragments=frags)
    return color, depth, win, stats


def render_subpatches(scene, sub_draw, sub_pid, sub_range, params=None, want_win=False):
    p = params or make_params(scene)
    ds = _Draws(scene.draws)
    npx = scene.width * scene.height
    color = np.zeros((npx, 4), np.float32)
    depth = np.zeros(npx, np.int32)
    win = np.zeros(npx, np.int64) if want_win else None
    st = np.zeros(4, np.int64)
    sd = np.ascontiguousarray(sub_draw, np.int32)
    sp = np.ascontiguousarray(sub_pid, np.int32)
    sr = np.ascontiguousarray(sub_range, np.float32).reshape(-1)
    rc = lib().or_render_subpatches(ctypes.byref(p), ds.arr, ds.n, len(sp), _ptr(sd, i32p), _ptr(sp, i32p),
                                    _ptr(sr, f32p), _ptr(color, f32p), _ptr(depth, i32p),
                                    _ptr(win, i64p) if want_win else None, _ptr(st, i64p))
    if rc:
        raise ValueError(f"oracle render failed: {rc}")
    stats = dict(subpatches=int(st[0]), micropolygons=int(st[1]), fragments=int(st[2]))
    return (color, depth, win, stats) if want_win else (color, depth, stats)


def dice(scene, draw_index, pid, rng, params=None):
    p = params or make_params(scene)
    ds = _Draws([scene.draws[draw_index]])
    G = p.reyes_patch_size + 1
    pos = np.zeros((G * G, 4), np.float32)
    pxl = np.zeros((G * G, 2), np.int32)
    dep = np.zeros(G * G, np.float32)
    r = np.ascontiguousarray(rng, np.float32)
    lib().or_dice(ctypes.byref(p), ds.arr, int(pid), _ptr(r, f32p), _ptr(pos, f32p), _ptr(pxl, i32p),
                  _ptr(dep, f32p))
    return pos, pxl, dep


def shade_quads(scene, draw_index, pid, rng, params=None):
    """Colour of every quad of one sub-patch (kernels/reyes.cl:172-191),
    float32[PS*PS, 4] in colour-grid order nu + nv * PS."""
    p = params or make_params(scene)
    ds = _Draws([scene.draws[draw_index]])
    col = np.zeros((p.reyes_patch_size ** 2, 4), np.float32)
    r = np.ascontiguousarray(rng, np.float32)
    lib().or_shade_quads(ctypes.byref(p), ds.arr, int(pid), _ptr(r, f32p), _ptr(col, f32p))
    return col


def dice_fp64(scene, draw_index, pid, rng, params=None):
    p = params or make_params(scene)
    ds = _Draws([scene.draws[draw_index]])
    G = p.reyes_patch_size + 1
    out = np.zeros((G * G, 3), np.float64)
    r = np.ascontiguousarray(rng, np.float32)
    lib().or_dice_fp64(ctypes.byref(p), ds.arr, int(pid), _ptr(r, f32p), _ptr(out, f64p))
    return out


def loss_fp64(scene, sub_pid, sub_range, win, target, cp, amp, params=None, grad=True):
    """FP64 loss with fixed visibility and its analytic gradient (draw 0)."""
    p = params or make_params(scene)
    ds = _Draws([scene.draws[0]])
    sp = np.ascontiguousarray(sub_pid, np.int32)
    sr = np.ascontiguousarray(sub_range, np.float32).reshape(-1)
    w = np.ascontiguousarray(win, np.int64)
    t = np.ascontiguousarray(target, np.float32).reshape(-1)
    c = np.ascontiguousarray(cp, np.float64).reshape(-1)
    g = np.zeros_like(c) if grad else None
    ga = ctypes.c_double(0)
    loss = lib().or_loss_fp64(ctypes.byref(p), ds.arr, len(sp), _ptr(sp, i32p), _ptr(sr, f32p), _ptr(w, i64p),
                              _ptr(t, f32p), _ptr(c, f64p), float(amp), _ptr(g, f64p) if grad else None,
                              ctypes.byref(ga) if grad else None)
    return (loss, g.reshape(np.shape(cp)), ga.value) if grad else loss


def sinf(x: float) -> float:
    return lib().or_sinf(x)


def inclusive_scan(a):
    a = np.ascontiguousarray(a, np.int32)
    out = np.zeros_like(a)
    lib().or_inclusive_scan(_ptr(a, i32p), _ptr(out, i32p), len(a))
    return out


# --- reference pin (only where the reference tree was compiled) -------------

def reference_dir():
    """The reference tree the pin was built from (MP_REFERENCE_DIR, else the
    directory build_ref.sh recorded), or None where it is not present."""
    d = os.environ.get("MP_REFERENCE_DIR")
    if not d:
        rec = os.path.join(HERE, "_ref", "reference_dir.txt")
        if os.path.exists(rec):
            d = open(rec).read().strip()
    return d if d and os.path.isdir(d) else None


_ref = None


def ref_pin():
    """The reference's own src/base math, compiled by build_ref.sh, or None."""
    global _ref
    if _ref is None:
        if not os.path.exists(REF_PIN_PATH):
            return None
        L = ctypes.CDLL(REF_PIN_PATH)
        L.refpin_eval_patch.argtypes = [f32p, ctypes.c_float, ctypes.c_float, f32p]
        L.refpin_eval_gregory.argtypes = [f32p, ctypes.c_float, ctypes.c_float, f32p]
        L.refpin_projection_bound.restype = ctypes.c_int
        L.refpin_projection_bound.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                                              ctypes.c_float, f32p, f32p]
        L.refpin_bound_n_split.restype = ctypes.c_long
        L.refpin_bound_n_split.argtypes = [f32p, ctypes.c_int, ctypes.c_int, f32p, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                           ctypes.c_int, i32p, f32p, ctypes.c_long]
        _ref = L
    return _ref


def ref_bound_n_split(scene, draw_index=0, params=None):
    L = ref_pin()
    if L is None:
        return None
    p = params or make_params(scene)
    d = scene.draws[draw_index]
    cp = np.ascontiguousarray(d.mesh.cp, np.float32).reshape(-1)
    mv = np.ascontiguousarray(d.mv, np.float32)
    args = (_ptr(cp, f32p), d.mesh.n_patches, d.mesh.type, _ptr(mv, f32p), p.fovy_deg, p.near_plane, p.width,
            p.height, p.cull_ribbon, p.bound_n_split_limit, p.max_split_depth)
    n = L.refpin_bound_n_split(*args, None, None, 0)
    pid = np.zeros(max(n, 1), np.int32)
    rng = np.zeros((max(n, 1), 4), np.float32)
    L.refpin_bound_n_split(*args, _ptr(pid, i32p), _ptr(rng, f32p), n)
    return pid[:n], rng[:n]


def ref_dice_shade(scene, draw_index, pid, rng, params=None, threads=None):
    """The reference's dice and shade kernels (compiled as C++ by
    oracle/build_ref.sh) over sub-patches (pid[S], range[S,4]) of one draw:
    (pos float32[S,G*G,4], pxl int32[S,G*G,2], depth float32[S,G*G],
    colour float32[S,PS*PS,4] with NaN where shade left a quad unwritten,
    block bounds int32[S,B,4]), or None where the reference tree was not
    compiled."""
    L = ref_pin()
    if L is None or not hasattr(L, "refk_dice_shade"):
        return None
    p = params or make_params(scene)
    d = scene.draws[draw_index]
    PS = p.reyes_patch_size
    G, B, S = PS + 1, (PS // 8) ** 2, len(pid)
    cp = np.ascontiguousarray(d.mesh.cp, np.float32).reshape(-1)
    mv = np.ascontiguousarray(d.mv, np.float32)
    dc = np.asarray(d.color, np.float32)
    pids = np.ascontiguousarray(pid, np.int32)
    rg = np.ascontiguousarray(rng, np.float32)
    pos = np.zeros((S, G * G, 4), np.float32)
    pxl = np.zeros((S, G * G, 2), np.int32)
    dep = np.zeros((S, G * G), np.float32)
    col = np.full((S, PS * PS, 4), np.nan, np.float32)
    blk = np.zeros((S, B, 4), np.int32)
    f = L.refk_dice_shade
    f.restype = None
    f.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                  ctypes.c_int, ctypes.c_int, f32p, ctypes.c_int, ctypes.c_int, f32p, f32p, ctypes.c_int, i32p,
                  f32p, f32p, i32p, f32p, f32p, i32p, ctypes.c_int]
    f(p.width, p.height, p.fovy_deg, p.near_plane, PS, p.subpixel_bits, p.backface_culling, p.displacement,
      _ptr(cp, f32p), d.mesh.n_patches, d.mesh.type, _ptr(mv, f32p), _ptr(dc, f32p), S, _ptr(pids, i32p),
      _ptr(rg, f32p), _ptr(pos, f32p), _ptr(pxl, i32p), _ptr(dep, f32p), _ptr(col, f32p), _ptr(blk, i32p),
      int(threads or os.cpu_count() or 1))
    return pos, pxl, dep, col, blk


def ref_bound_n_split_gpu(scene, draw_index=0, params=None):
    """The reference's GPU bound criterion (kernels/bound_n_split.h compiled
    as C++ by oracle/build_ref.sh) over one draw: (pid int32[S], range
    float32[S,4]) as a set in LIFO order, or None where the reference tree
    was not compiled."""
    L = ref_pin()
    if L is None or not hasattr(L, "refk_bound_n_split_gpu"):
        return None
    p = params or make_params(scene)
    d = scene.draws[draw_index]
    cp = np.ascontiguousarray(d.mesh.cp, np.float32).reshape(-1)
    mv = np.ascontiguousarray(d.mv, np.float32)
    f = L.refk_bound_n_split_gpu
    f.restype = ctypes.c_long
    f.argtypes = [f32p, ctypes.c_int, ctypes.c_int, f32p, ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                  ctypes.c_float, ctypes.c_float, ctypes.c_int, i32p, f32p, ctypes.c_long]
    args = (_ptr(cp, f32p), d.mesh.n_patches, d.mesh.type, _ptr(mv, f32p), p.fovy_deg, p.near_plane, p.width,
            p.height, p.cull_ribbon, p.bound_n_split_limit, p.max_split_depth)
    n = f(*args, None, None, 0)
    if n < 0:
        raise ValueError("reference bound-and-split ran past its range budget")
    pid = np.zeros(max(n, 1), np.int32)
    rng = np.zeros((max(n, 1), 4), np.float32)
    f(*args, _ptr(pid, i32p), _ptr(rng, f32p), n)
    return pid[:n], rng[:n]


def display_image(color_tiled, width, height, tile=8):
    """The image the reference's tex_draw shader shows (shaders/tex_draw.frag):
    pixel (x, y) of the framebuffer is texel (gx + ceil(W/tile) * gy) * tile^2
    + lx + tile * ly; RGB gets pow(c, 0.454545); the 8-bit window stores
    round(clamp(c, 0, 1) * 255).  gl_FragCoord.y counts from the bottom, so
    the returned (height, width, 3) uint8 array has the top row first."""
    c = np.asarray(color_tiled, np.float32).reshape(-1, 4)
    gx = (width + tile - 1) // tile
    y, x = np.mgrid[0:height, 0:width]
    idx = ((x // tile) + gx * (y // tile)) * tile * tile + (x % tile) + tile * (y % tile)
    rgb = c[idx.reshape(-1), :3].reshape(height, width, 3)
    g = np.clip(np.power(rgb, np.float32(0.454545)), 0.0, 1.0).astype(np.float32)
    out = np.rint(g * np.float32(255.0)).astype(np.uint8)
    return out[::-1].copy()


_TRACE_LINE = None


def parse_trace(text):
    """Lines of the reference's trace format (src/CL/Device.cpp:275-289), read
    with the pattern of the reference's tools/parse_trace.py: a list of
    (name, queue, queued, submit, start, end, id, deps)."""
    import re
    global _TRACE_LINE
    if _TRACE_LINE is None:
        _TRACE_LINE = re.compile(r'([^@:]*)(@[^@:]*):(\d+):(\d+):(\d+):(\d+):(\d+):([0-9|]*)')
    out = []
    for line in text.splitlines():
        m = _TRACE_LINE.match(line)
        if not m:
            raise ValueError(f"trace line format mismatch: {line!r}")
        out.append((m.group(1), m.group(2)[1:], int(m.group(3)), int(m.group(4)), int(m.group(5)), int(m.group(6)),
                    int(m.group(7)), [int(s) for s in m.group(8).split('|') if s]))
    return out


def parse_stats(text):
    """`key = value;` lines of Statistics::dump_stats (src/base/Statistics.cpp:196-217)."""
    out = {}
    for part in text.split(";"):
        part = part.strip()
        if not part:
            continue
        k, _, v = part.partition("=")
        v = v.strip()
        out[k.strip()] = [int(t) for t in v.split()] if k.strip() == "bound_n_split_balance" else int(v)
    return out


def ref_render(scene, params=None, threads=None):
    """The reference's own kernels (kernels/*.cl compiled as C++ by
    oracle/build_ref.sh) after its CPU bound-and-split: (tiled colour
    float32[W*H,4], tiled depth int32[W*H], sub-patch count), or None where
    the reference tree was not compiled."""
    L = ref_pin()
    if L is None or not hasattr(L, "refk_render"):
        return None
    p = params or make_params(scene)
    n = len(scene.draws)
    cps = [np.ascontiguousarray(d.mesh.cp, np.float32).reshape(-1) for d in scene.draws]
    cp_ptrs = (f32p * max(1, n))(*[_ptr(c, f32p) for c in cps])
    npatch = np.array([d.mesh.n_patches for d in scene.draws], np.int32)
    types = np.array([d.mesh.type for d in scene.draws], np.int32)
    mvs = np.ascontiguousarray(np.stack([np.asarray(d.mv, np.float32) for d in scene.draws]).reshape(-1))
    cols = np.ascontiguousarray(np.stack([np.asarray(d.color, np.float32) for d in scene.draws]).reshape(-1))
    clear = np.asarray(list(p.clear_color), np.float32)
    npx = scene.width * scene.height
    color = np.zeros((npx, 4), np.float32)
    depth = np.zeros(npx, np.int32)
    L.refk_render.restype = ctypes.c_long
    L.refk_render.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                              ctypes.c_float, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, f32p, ctypes.c_int, ctypes.POINTER(f32p), i32p, i32p, f32p, f32p, f32p,
                              i32p, ctypes.c_int]
    s = L.refk_render(scene.width, scene.height, p.fovy_deg, p.near_plane, p.cull_ribbon, p.bound_n_split_limit,
                      p.max_split_depth, p.reyes_patches_per_pass, p.reyes_patch_size, p.subpixel_bits,
                      p.backface_culling, p.displacement, _ptr(clear, f32p), n, cp_ptrs, _ptr(npatch, i32p),
                      _ptr(types, i32p), _ptr(mvs, f32p), _ptr(cols, f32p), _ptr(color, f32p), _ptr(depth, i32p),
                      int(threads or os.cpu_count() or 1))
    if s < 0:
        raise ValueError("reference render failed")
    return color, depth, int(s)
