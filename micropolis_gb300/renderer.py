"""Host-side mirror of the reference's renderer interface.

`Renderer` has the reference's Reyes::Renderer methods (src/Reyes/Renderer.h:29-45):
prepare(), are_patches_loaded(handle), load_patches(handle, patch_data, type),
draw_patches(handle, modelview, projection, color), finish(), dump_trace(),
with the same argument meaning.  Errors raise MpError (the reference throws
CL::Exception).  Everything runs in libmpcore.so through the C ABI.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from ._lib import MpError, MpOptions, MpProjection, MpStats, lib
from .options import ReyesOptions


class Projection:
    """Reyes::Projection(fovy, near, viewport) (src/base/Projection.h:144)."""

    def __init__(self, fovy: float, near: float, viewport):
        self.fovy = float(fovy)
        self.near = float(near)
        self.viewport = (int(viewport[0]), int(viewport[1]))

    def c(self) -> MpProjection:
        p = MpProjection()
        p.fovy_deg = self.fovy
        p.near_plane = self.near
        p.viewport[0], p.viewport[1] = self.viewport
        return p


def _f32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _i32p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


class Renderer:
    def __init__(self, options: Optional[ReyesOptions] = None, **overrides):
        opts = options or ReyesOptions()
        if overrides:
            opts = ReyesOptions(**{**opts.__dict__}).update(**overrides)
        self.options = opts
        o = MpOptions()
        lib().mp_options_default(ctypes.byref(o))
        o.window_size[0], o.window_size[1] = opts.window_size
        o.reyes_patch_size = opts.reyes_patch_size
        o.bound_n_split_limit = opts.bound_n_split_limit
        o.reyes_patches_per_pass = opts.reyes_patches_per_pass
        o.cull_ribbon = opts.cull_ribbon
        o.max_split_depth = opts.max_split_depth
        o.bound_sample_rate = opts.bound_sample_rate
        o.subpixel_bits = opts.subpixel_bits
        o.framebuffer_tile_size = opts.framebuffer_tile_size
        o.backface_culling = int(bool(opts.backface_culling))
        o.displacement = int(bool(opts.displacement))
        o.displacement_amplitude = opts.displacement_amplitude
        for i in range(4):
            o.clear_color[i] = opts.clear_color[i]
        o.batch_views = opts.batch_views
        o.path = _lib.MP_PATH_PLAIN if opts.path == "plain" else _lib.MP_PATH_BATCHED
        o.queue_capacity = opts.queue_capacity
        o.subpatch_capacity = opts.subpatch_capacity
        if opts.spin_limit:
            o.spin_limit = opts.spin_limit
        o.overlap = int(bool(opts.overlap))
        o.bns_blocks = int(opts.bns_blocks)
        o.raster_tile = int(opts.raster_tile)
        o.dice_group = int(opts.dice_group)
        o.bound_criterion = int(opts.bound_criterion)
        self._ctx = ctypes.c_void_p()
        st = lib().mp_create(ctypes.byref(o), ctypes.byref(self._ctx))
        if st != 0:
            raise MpError(st, "mp_create failed")
        self.width, self.height = opts.window_size
        self.views = opts.batch_views

    # -- error plumbing --------------------------------------------------------
    def _ck(self, st: int) -> None:
        if st != 0:
            raise MpError(st, lib().mp_last_error(self._ctx).decode())

    def close(self) -> None:
        if self._ctx:
            lib().mp_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int) -> None:
        self._ck(lib().mp_set_stream(self._ctx, ctypes.c_void_p(stream_handle or None)))

    # -- Reyes::Renderer --------------------------------------------------------
    def prepare(self) -> None:
        self._ck(lib().mp_prepare(self._ctx))

    def finish(self) -> None:
        self._ck(lib().mp_finish(self._ctx))

    def are_patches_loaded(self, handle: int) -> bool:
        v = ctypes.c_int32()
        self._ck(lib().mp_are_patches_loaded(self._ctx, handle, ctypes.byref(v)))
        return bool(v.value)

    def load_patches(self, handle: int, patch_data, patch_type: int) -> None:
        a = np.ascontiguousarray(patch_data, np.float32).reshape(-1, 3)
        self._ck(lib().mp_load_patches(self._ctx, handle, _f32p(a), a.shape[0], patch_type))

    def load_patches_device(self, handle: int, dev_ptr: int, n_points: int, patch_type: int) -> None:
        self._ck(lib().mp_load_patches_device(self._ctx, handle, ctypes.c_void_p(dev_ptr), n_points, patch_type))

    def update_patches_device(self, handle: int, dev_ptr: int) -> None:
        self._ck(lib().mp_update_patches_device(self._ctx, handle, ctypes.c_void_p(dev_ptr)))

    def delete_patches(self, handle: int) -> None:
        self._ck(lib().mp_delete_patches(self._ctx, handle))

    def draw_patches(self, handle: int, modelview, projection: Projection, color=(1, 1, 1, 1), view: int = 0) -> None:
        mv = np.ascontiguousarray(modelview, np.float32).reshape(16)
        col = np.ascontiguousarray(color, np.float32).reshape(4)
        p = projection.c()
        self._ck(lib().mp_draw_patches_view(self._ctx, handle, _f32p(mv), ctypes.byref(p), _f32p(col), view))

    def draw_views(self, items) -> None:
        """Many draws in one call: items of (handle, modelview, projection, colour, view)."""
        arr = (_lib.MpView * max(1, len(items)))()
        for k, (h, mv, proj, col, view) in enumerate(items):
            arr[k].handle = h
            arr[k].modelview[:] = [float(x) for x in np.asarray(mv, np.float32).reshape(16)]
            arr[k].proj = proj.c()
            arr[k].color[:] = [float(x) for x in np.asarray(col, np.float32).reshape(4)]
            arr[k].view = int(view)
        self._ck(lib().mp_draw_views(self._ctx, len(items), arr))

    def _text(self, fn) -> str:
        size = 4096
        while True:
            buf = ctypes.create_string_buffer(size)
            st = fn(self._ctx, buf, len(buf))
            if st != _lib.MP_ERR_OVERFLOW:
                self._ck(st)
                return buf.value.decode()
            size *= 4

    def dump_trace(self) -> str:
        """The last frame's commands in the reference's trace line format."""
        return self._text(lib().mp_dump_trace)

    def dump_stats(self) -> str:
        """The last frame's statistics in the format of Statistics::dump_stats."""
        return self._text(lib().mp_dump_stats)

    def write_trace(self, path: str) -> None:
        with open(path, "w") as f:
            f.write(self.dump_trace())

    def write_stats(self, path: str) -> None:
        with open(path, "w") as f:
            f.write(self.dump_stats())

    # -- headless framebuffer and inspection -------------------------------------
    def framebuffer_ptrs(self):
        c, d = ctypes.c_void_p(), ctypes.c_void_p()
        self._ck(lib().mp_framebuffer(self._ctx, ctypes.byref(c), ctypes.byref(d), None, None, None))
        return c.value, d.value

    def read_framebuffer(self, view: int = 0, linear: bool = False):
        n = self.width * self.height
        color = np.zeros((n, 4), np.float32)
        depth = np.zeros(n, np.int32)
        self._ck(lib().mp_read_framebuffer(self._ctx, view, _f32p(color), _i32p(depth), int(linear)))
        return color, depth

    def read_image(self, view: int = 0) -> np.ndarray:
        """The displayed image (gamma 1/2.2, 8-bit), (height, width, 3) RGB, top row first."""
        rgb = np.zeros((self.height, self.width, 3), np.uint8)
        self._ck(lib().mp_read_image(self._ctx, view, rgb.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return rgb

    def save_ppm(self, path: str, view: int = 0) -> None:
        """Binary PPM (P6) of the displayed image."""
        write_ppm(path, self.read_image(view))

    def save_pfm(self, path: str, view: int = 0) -> None:
        """Linear colour as a PFM (little-endian float RGB, bottom row first)."""
        color, _ = self.read_framebuffer(view, linear=True)
        write_pfm(path, color.reshape(self.height, self.width, 4)[:, :, :3])

    def copy_framebuffer_device(self, view: int, color_ptr: int, depth_ptr: int = 0) -> None:
        self._ck(lib().mp_copy_framebuffer_device(self._ctx, view, ctypes.c_void_p(color_ptr or None),
                                                  ctypes.c_void_p(depth_ptr or None)))

    def visibility(self, view: int = 0) -> np.ndarray:
        ids = np.zeros(self.width * self.height, np.int64)
        self._ck(lib().mp_read_visibility(self._ctx, view, ids.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        return ids

    def subpatches(self):
        cnt = ctypes.c_int64()
        self._ck(lib().mp_subpatches(self._ctx, ctypes.byref(cnt), None, None, None, 0))
        n = cnt.value
        draw = np.zeros(max(n, 1), np.int32)
        pid = np.zeros(max(n, 1), np.int32)
        rng = np.zeros((max(n, 1), 4), np.float32)
        self._ck(lib().mp_subpatches(self._ctx, ctypes.byref(cnt), _i32p(draw), _i32p(pid), _f32p(rng), n))
        return draw[:n], pid[:n], rng[:n]

    # mp_stats.stage_ms slots: the batched path fills clear, bound_split,
    # canonical_sort_or_sample (its sort), dice_raster, raster_big and
    # resolve_or_shade; the plain path bound_split, dice_raster (dice),
    # resolve_or_shade (shade), canonical_sort_or_sample (sample),
    # raster_big, pass_resolve and host_sync
    STAGES = ("clear", "bound_split", "dice_raster", "raster_big", "resolve_or_shade", "canonical_sort_or_sample",
              "pass_resolve", "host_sync")

    def stats(self) -> dict:
        s = MpStats()
        self._ck(lib().mp_stats_get(self._ctx, ctypes.byref(s)))
        out = {k: getattr(s, k) for k, _ in MpStats._fields_ if k != "stage_ms"}
        out["stage_ms"] = dict(zip(self.STAGES, list(s.stage_ms)))
        return out

    def set_stage_timing(self, on: bool) -> None:
        self._ck(lib().mp_set_stage_timing(self._ctx, int(bool(on))))

    def dice_subpatches(self, draw: int, pid, rng):
        pid = np.ascontiguousarray(pid, np.int32)
        rng = np.ascontiguousarray(rng, np.float32).reshape(-1, 4)
        n = len(pid)
        G = self.options.reyes_patch_size + 1
        pos = np.zeros((n, G * G, 4), np.float32)
        pxl = np.zeros((n, G * G, 2), np.int32)
        dep = np.zeros((n, G * G), np.float32)
        self._ck(lib().mp_dice_subpatches(self._ctx, draw, n, _i32p(pid), _f32p(rng), _f32p(pos), _i32p(pxl),
                                          _f32p(dep)))
        return pos, pxl, dep

    def read_framebuffer_async(self, view: int, color_ptr: int, depth_ptr: int) -> None:
        """Starts the read-back of layer `view` into host buffers (tiled
        float4 colour, int32 depth; page-locked for an asynchronous copy) and
        returns at once; wait_read_framebuffer() completes it."""
        self._ck(lib().mp_read_framebuffer_async(self._ctx, view, ctypes.c_void_p(color_ptr or None),
                                                 ctypes.c_void_p(depth_ptr or None)))

    def wait_read_framebuffer(self) -> None:
        self._ck(lib().mp_wait_read_framebuffer(self._ctx))

    def set_displacement_amplitude(self, amp: float) -> None:
        self._ck(lib().mp_set_displacement_amplitude(self._ctx, float(amp)))

    def set_displacement_amplitude_device(self, dev_ptr: int) -> None:
        """The amplitude multiplier from one float32 in device memory (stream-ordered copy)."""
        self._ck(lib().mp_set_displacement_amplitude_device(self._ctx, ctypes.c_void_p(dev_ptr)))

    def set_grad_buffer(self, draw: int, dev_ptr: int) -> None:
        self._ck(lib().mp_set_grad_buffer(self._ctx, draw, ctypes.c_void_p(dev_ptr)))

    def backward(self, view: int, grad_color_ptr: int, grad_amp_ptr: int) -> None:
        self._ck(lib().mp_backward(self._ctx, view, ctypes.c_void_p(grad_color_ptr), ctypes.c_void_p(grad_amp_ptr)))

    def inclusive_scan(self, values) -> np.ndarray:
        a = np.ascontiguousarray(values, np.int32)
        out = np.zeros_like(a)
        self._ck(lib().mp_inclusive_scan(self._ctx, _i32p(a), _i32p(out), len(a)))
        return out

    def atomic_bench(self, n_slots: int, n_ops: int, pattern: int) -> float:
        r = ctypes.c_double()
        self._ck(lib().mp_atomic_bench(self._ctx, n_slots, n_ops, pattern, ctypes.byref(r)))
        return r.value


def write_ppm(path: str, rgb: np.ndarray) -> None:
    """(height, width, 3) uint8 RGB, top row first, as binary PPM."""
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(b"P6\n%d %d\n255\n" % (w, h))
        f.write(np.ascontiguousarray(rgb, np.uint8).tobytes())


def read_ppm(path: str) -> np.ndarray:
    with open(path, "rb") as f:
        data = f.read()
    parts = data.split(maxsplit=4)
    if parts[0] != b"P6" or int(parts[3]) != 255:
        raise ValueError("not an 8-bit binary PPM")
    w, h = int(parts[1]), int(parts[2])
    return np.frombuffer(parts[4][:w * h * 3], np.uint8).reshape(h, w, 3)


def write_pfm(path: str, rgb_rows_up: np.ndarray) -> None:
    """(height, width, 3) float RGB whose row 0 is the bottom row (the
    framebuffer's y axis), as PFM, which stores rows bottom first."""
    h, w, _ = rgb_rows_up.shape
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(rgb_rows_up, "<f4").tobytes())


def render_scene(renderer: Renderer, scene, handles=None) -> None:
    """Scene::draw (src/micropolis/Scene.cpp:179-197): prepare, load on first
    use, draw every object, finish."""
    renderer.prepare()
    for k, d in enumerate(scene.draws):
        h = handles[k] if handles else id(d.mesh)
        if not renderer.are_patches_loaded(h):
            renderer.load_patches(h, d.mesh.cp, d.mesh.type)
        renderer.draw_patches(h, d.mv, Projection(scene.fovy, scene.near, (scene.width, scene.height)), d.color,
                              view=d.view)
    renderer.finish()


def renderer_for(scene, path: str = "batched", **over) -> Renderer:
    opts = ReyesOptions(window_size=(scene.width, scene.height), path=path)
    known = {k: v for k, v in scene.options.items() if hasattr(opts, k)}
    opts.update(**known)
    if over:
        opts.update(**over)
    return Renderer(opts)
