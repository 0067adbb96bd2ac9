"""Shared comparison helpers for the parity tests."""
import numpy as np


def subpatch_set(pid, rng, draw=None):
    """Sub-patch records as a set of (draw, pid, range bit patterns)."""
    bits = np.ascontiguousarray(rng, np.float32).view(np.uint32).reshape(-1, 4)
    d = np.zeros(len(pid), np.int64) if draw is None else np.asarray(draw)
    return set(zip(d.tolist(), np.asarray(pid).tolist(), map(tuple, bits.tolist())))


def framebuffer_diff(color_a, depth_a, color_b, depth_b, rel=1e-5):
    """(#pixels whose depth or colour differ beyond rel, #pixels not bit-equal)."""
    ca, cb = np.asarray(color_a), np.asarray(color_b)
    tol = rel * np.maximum(np.abs(ca), np.abs(cb))
    cbad = np.any(np.abs(ca - cb) > tol, axis=1)
    dbad = np.asarray(depth_a) != np.asarray(depth_b)
    exact = np.any(ca != cb, axis=1) | dbad
    return int(np.count_nonzero(cbad | dbad)), int(np.count_nonzero(exact))
