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


GOLDEN_DIR = __import__("os").path.join(__import__("os").path.dirname(__import__("os").path.abspath(__file__)),
                                        "golden")
GOLDEN_CASES = ("heightfield_1024x768", "mixed96_bezier_512", "mixed96_gregory_512", "mixed96_gregory_depth3_512",
                "heightfield_eye_plane_512x384")


def golden_case(name):
    """(scene, options, pid, range) of a golden fixture written by
    tests/golden/make_golden.py from the reference's own bound-and-split."""
    import os
    from micropolis_gb300 import scenes
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    opts = dict(bound_n_split_limit=float(z["limit"]), cull_ribbon=float(z["cull_ribbon"]),
                max_split_depth=int(z["max_split_depth"]))
    draw = scenes.Draw(scenes.Mesh(int(z["type"]), z["cp"].copy()), z["mv"].copy(), (0.9, 0.7, 0.3, 1.0))
    sc = scenes.Scene(name, int(z["width"]), int(z["height"]), [draw], fovy=float(z["fovy"]), near=float(z["near"]),
                      options=dict(opts))
    return sc, opts, z["pid"], z["range"]


GOLDEN_FRAMES = ("frame_mixed96_bezier_512_d0_ps8", "frame_mixed96_bezier_512_d1_ps8",
                 "frame_mixed96_gregory_512_d0_ps8", "frame_mixed96_gregory_depth3_512_d1_ps8",
                 "frame_mixed96_bezier_512_d0_ps16")


def golden_frame(name):
    """(scene, options, colour float32[N,4], depth int32[N]) of a golden
    framebuffer written by tests/golden/make_golden_frames.py from the
    reference's own kernels; the options include the displacement and dice
    grid it was rendered with."""
    import os
    z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
    sc, opts, _, _ = golden_case(str(z["case"]))
    opts = dict(opts, displacement=int(z["displacement"]), reyes_patch_size=int(z["patch_size"]))
    sc.options.update(opts)
    n = int(z["pixels"])
    color = np.empty((n, 4), np.float32)
    color[:] = np.asarray(z["clear"], np.float32)
    depth = np.full(n, 0x7fffffff, np.int32)
    color[z["index"]] = z["color"]
    depth[z["index"]] = z["depth"]
    return sc, opts, color, depth


def frame_agrees(color, depth, gcolor, gdepth, rel=1e-5, budget=1e-4):
    """Coverage identical, and depth and colour within rel except in at most
    budget of the frame's pixels (ties); returns the number of such pixels."""
    assert np.array_equal(depth != 0x7fffffff, gdepth != 0x7fffffff)
    bad, _ = framebuffer_diff(color, depth, gcolor, gdepth, rel)
    assert bad <= budget * depth.size, (bad, depth.size)
    return bad


GOLDEN_GPU_CRITERION = ("mixed96_bezier_512", "mixed96_gregory_512", "heightfield_eye_plane_512x384")


def golden_gpucrit(name):
    """(pid, range) of the reference's GPU bound criterion on the inputs of
    golden case `name` (tests/golden/make_golden.py): a set, in no order."""
    import os
    z = np.load(os.path.join(GOLDEN_DIR, "gpucrit_" + name + ".npz"))
    return z["pid"], z["range"]


def same_colour(a, b):
    """Per-pixel bit equality of two float colour arrays (any two NaNs agree)."""
    a, b = np.asarray(a, np.float32), np.asarray(b, np.float32)
    same = (a.view(np.uint32) == b.view(np.uint32)) | (np.isnan(a) & np.isnan(b))
    return np.all(same, axis=-1)


def assert_identical_to_oracle(r, scene, params=None, oracle_frame=None):
    """A batched frame against the oracle's frame of the same scene: the
    sub-patch list equal to the oracle's canonical list in order and bit for
    bit, colour and depth bit-identical at every pixel, and the same winning
    micropolygon number at every pixel (ties included: both number
    micropolygons in the canonical order and keep the smallest at equal
    depth).  oracle_frame: (colour, depth, winners, stats) when already
    rendered (oracle.render_parallel).  Returns the oracle's stats."""
    from oracle import oracle
    p = params or oracle.make_params(scene)
    odraw, opid, orng, _ = oracle.canonical_subpatches(scene, p)
    draw, pid, rng = r.subpatches()
    assert len(pid) == len(opid), (len(pid), len(opid))
    assert np.array_equal(draw, odraw) and np.array_equal(pid, opid)
    assert np.array_equal(np.ascontiguousarray(rng, np.float32).view(np.uint32),
                          np.ascontiguousarray(orng, np.float32).view(np.uint32))
    if oracle_frame is None:
        oracle_frame = oracle.render(scene, params=p, want_win=True)
    ocol, odep, owin, ost = oracle_frame
    col, dep = r.read_framebuffer()
    assert np.array_equal(dep, odep), int(np.count_nonzero(dep != odep))
    same = same_colour(col, ocol)
    assert same.all(), int(np.count_nonzero(~same))
    vis = r.visibility()
    assert np.array_equal(vis, owin), int(np.count_nonzero(vis != owin))
    st = r.stats()
    assert st["micropolygons"] == ost["micropolygons"] and st["fragments"] == ost["fragments"]
    return ost
