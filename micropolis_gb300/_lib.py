"""ctypes binding of libmpcore.so (include/mp_core.h).

The library is built in tree by micropolis_gb300/build.py.  Loading fails
loudly when it is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmpcore.so")

MP_OK, MP_ERR_INVALID_ARG, MP_ERR_OUT_OF_MEMORY, MP_ERR_OVERFLOW, MP_ERR_TIMEOUT, MP_ERR_CUDA, \
    MP_ERR_NOT_LOADED, MP_ERR_STATE = range(8)
STATUS_NAMES = {0: "MP_OK", 1: "MP_ERR_INVALID_ARG", 2: "MP_ERR_OUT_OF_MEMORY", 3: "MP_ERR_OVERFLOW",
                4: "MP_ERR_TIMEOUT", 5: "MP_ERR_CUDA", 6: "MP_ERR_NOT_LOADED", 7: "MP_ERR_STATE"}
MP_BEZIER, MP_GREGORY = 0, 1
MP_PATH_PLAIN, MP_PATH_BATCHED = 0, 1


class MpOptions(ctypes.Structure):
    _fields_ = [("window_size", ctypes.c_int32 * 2), ("reyes_patch_size", ctypes.c_int32),
                ("bound_n_split_limit", ctypes.c_float), ("reyes_patches_per_pass", ctypes.c_int32),
                ("cull_ribbon", ctypes.c_float), ("max_split_depth", ctypes.c_int32),
                ("bound_sample_rate", ctypes.c_int32), ("subpixel_bits", ctypes.c_int32),
                ("framebuffer_tile_size", ctypes.c_int32), ("backface_culling", ctypes.c_int32),
                ("displacement", ctypes.c_int32), ("displacement_amplitude", ctypes.c_float),
                ("clear_color", ctypes.c_float * 4), ("batch_views", ctypes.c_int32), ("path", ctypes.c_int32),
                ("queue_capacity", ctypes.c_int64), ("subpatch_capacity", ctypes.c_int64),
                ("spin_limit", ctypes.c_int64), ("overlap", ctypes.c_int32), ("bns_blocks", ctypes.c_int32),
                ("raster_tile", ctypes.c_int32), ("dice_group", ctypes.c_int32),
                ("bound_criterion", ctypes.c_int32)]


class MpProjection(ctypes.Structure):
    _fields_ = [("fovy_deg", ctypes.c_float), ("near_plane", ctypes.c_float), ("viewport", ctypes.c_int32 * 2)]


class MpView(ctypes.Structure):
    _fields_ = [("handle", ctypes.c_uint64), ("modelview", ctypes.c_float * 16), ("proj", MpProjection),
                ("color", ctypes.c_float * 4), ("view", ctypes.c_int32)]


class MpStats(ctypes.Structure):
    _fields_ = [("subpatches", ctypes.c_int64), ("micropolygons", ctypes.c_int64), ("bounds", ctypes.c_int64),
                ("passes", ctypes.c_int64), ("fragments", ctypes.c_int64), ("big_quads", ctypes.c_int64),
                ("gpu_ms", ctypes.c_double), ("stage_ms", ctypes.c_double * 8), ("kernels", ctypes.c_int64)]


c_void_p = ctypes.c_void_p
i32, i64, u64, f32 = ctypes.c_int32, ctypes.c_int64, ctypes.c_uint64, ctypes.c_float
P = ctypes.POINTER

# every symbol declared in include/mp_core.h: (name, restype, argtypes)
SIGNATURES = [
    ("mp_options_default", None, [P(MpOptions)]),
    ("mp_create", ctypes.c_int, [P(MpOptions), P(c_void_p)]),
    ("mp_destroy", None, [c_void_p]),
    ("mp_last_error", ctypes.c_char_p, [c_void_p]),
    ("mp_set_stream", ctypes.c_int, [c_void_p, c_void_p]),
    ("mp_are_patches_loaded", ctypes.c_int, [c_void_p, u64, P(i32)]),
    ("mp_load_patches", ctypes.c_int, [c_void_p, u64, P(f32), ctypes.c_size_t, ctypes.c_int]),
    ("mp_load_patches_device", ctypes.c_int, [c_void_p, u64, c_void_p, ctypes.c_size_t, ctypes.c_int]),
    ("mp_delete_patches", ctypes.c_int, [c_void_p, u64]),
    ("mp_prepare", ctypes.c_int, [c_void_p]),
    ("mp_draw_patches", ctypes.c_int, [c_void_p, u64, P(f32), P(MpProjection), P(f32)]),
    ("mp_draw_patches_view", ctypes.c_int, [c_void_p, u64, P(f32), P(MpProjection), P(f32), i32]),
    ("mp_draw_views", ctypes.c_int, [c_void_p, i32, P(MpView)]),
    ("mp_finish", ctypes.c_int, [c_void_p]),
    ("mp_set_stage_timing", ctypes.c_int, [c_void_p, i32]),
    ("mp_dump_trace", ctypes.c_int, [c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    ("mp_framebuffer", ctypes.c_int, [c_void_p, P(c_void_p), P(c_void_p), P(i32), P(i32), P(i32)]),
    ("mp_read_framebuffer", ctypes.c_int, [c_void_p, i32, P(f32), P(i32), i32]),
    ("mp_copy_framebuffer_device", ctypes.c_int, [c_void_p, i32, c_void_p, c_void_p]),
    ("mp_read_visibility", ctypes.c_int, [c_void_p, i32, P(i64)]),
    ("mp_subpatches", ctypes.c_int, [c_void_p, P(i64), P(i32), P(i32), P(f32), i64]),
    ("mp_stats_get", ctypes.c_int, [c_void_p, P(MpStats)]),
    ("mp_dice_subpatches", ctypes.c_int, [c_void_p, i32, i64, P(i32), P(f32), P(f32), P(i32), P(f32)]),
    ("mp_set_grad_buffer", ctypes.c_int, [c_void_p, i32, c_void_p]),
    ("mp_backward", ctypes.c_int, [c_void_p, i32, c_void_p, c_void_p]),
    ("mp_set_displacement_amplitude", ctypes.c_int, [c_void_p, f32]),
    ("mp_set_displacement_amplitude_device", ctypes.c_int, [c_void_p, c_void_p]),
    ("mp_read_framebuffer_async", ctypes.c_int, [c_void_p, i32, c_void_p, c_void_p]),
    ("mp_wait_read_framebuffer", ctypes.c_int, [c_void_p]),
    ("mp_update_patches_device", ctypes.c_int, [c_void_p, u64, c_void_p]),
    ("mp_inclusive_scan", ctypes.c_int, [c_void_p, P(i32), P(i32), i64]),
    ("mp_inclusive_scan_noalloc", ctypes.c_int, [c_void_p, c_void_p, i64, c_void_p]),
    ("mp_atomic_bench", ctypes.c_int, [c_void_p, i64, i64, i32, P(ctypes.c_double)]),
    ("mp_read_image", ctypes.c_int, [c_void_p, i32, P(ctypes.c_uint8)]),
    ("mp_dump_stats", ctypes.c_int, [c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    ("mp_scene_load", ctypes.c_int, [ctypes.c_char_p, P(c_void_p)]),
    ("mp_scene_parse", ctypes.c_int, [ctypes.c_char_p, ctypes.c_size_t, P(c_void_p)]),
    ("mp_scene_free", None, [c_void_p]),
    ("mp_scene_counts", ctypes.c_int, [c_void_p, P(i32), P(i32), P(i32), P(i32)]),
    ("mp_scene_mesh", ctypes.c_int, [c_void_p, i32, P(ctypes.c_char_p), P(i32), P(P(f32)), P(i64)]),
    ("mp_scene_object", ctypes.c_int, [c_void_p, i32, P(ctypes.c_char_p), P(i32), P(f32), P(f32)]),
    ("mp_scene_camera", ctypes.c_int, [c_void_p, i32, P(ctypes.c_char_p), P(f32), P(f32), P(f32), P(f32)]),
    ("mp_scene_modelview", ctypes.c_int, [c_void_p, i32, i32, P(f32)]),
    ("mp_scene_draw", ctypes.c_int, [c_void_p, c_void_p, i32]),
]

_lib = None


def lib():
    """The loaded libmpcore.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run micropolis_gb300.build.build() "
                               "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class MpError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status
