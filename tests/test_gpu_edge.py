"""Edge cases of the GPU path against the oracle, through the C ABI: empty and
fully culled scenes, NaN control points, the depth cap, patches crossing the
eye plane, capacity overflow and regrowth, bounded waits, 16x16 dicing,
backface culling off, and many independent views in one batched frame."""
import numpy as np
import pytest

from helpers import framebuffer_diff, subpatch_set

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
COVERAGE_BUDGET = 1e-4


def _render(scene, path="batched", **over):
    from micropolis_gb300.renderer import render_scene, renderer_for
    r = renderer_for(scene, path, **over)
    render_scene(r, scene)
    return r


def _oracle(scene, **over):
    from oracle import oracle
    p = oracle.make_params(scene, **over)
    s = set()
    for k in range(len(scene.draws)):
        pid, rng, _ = oracle.bound_n_split(scene, k, params=p)
        s |= subpatch_set(pid, rng, np.full(len(pid), k))
    col, dep, st = oracle.render(scene, params=p)
    return s, col, dep, st


def _check(scene, path="batched", **over):
    r = _render(scene, path, **over)
    want, ocol, odep, ost = _oracle(scene, **over)
    d, p, g = r.subpatches()
    assert subpatch_set(p, g, d) == want
    col, dep = r.read_framebuffer()
    bad, _ = framebuffer_diff(col, dep, ocol, odep, REL_TOL)
    assert bad <= COVERAGE_BUDGET * dep.size, bad
    assert r.stats()["fragments"] == ost["fragments"]
    r.close()
    return len(want)


def _small_scene(**kw):
    from micropolis_gb300 import scenes
    return scenes.mixed4096_1920x1080(n=kw.pop("n", 128), width=kw.pop("width", 512), height=kw.pop("height", 512),
                                      **kw)


def test_empty_mesh(built, cuda):
    from micropolis_gb300 import scenes
    sc = _small_scene()
    sc.draws[0].mesh = scenes.Mesh(scenes.BEZIER, np.zeros((0, 16, 3), np.float32))
    for path in ("batched", "plain"):
        _check(sc, path)


def test_everything_culled(built, cuda):
    from micropolis_gb300 import scenes
    sc = _small_scene()
    for d in sc.draws:   # look away from the scene
        d.mv = scenes.look_at((0, 0, 40), (0, 0, 80), (0, 1, 0))
    for path in ("batched", "plain"):
        r = _render(sc, path)
        assert r.stats()["subpatches"] == 0
        col, dep = r.read_framebuffer()
        assert np.all(dep == 0x7FFFFFFF)
        r.close()


def test_nan_control_points(built, cuda):
    sc = _small_scene()
    cp = sc.draws[0].mesh.cp
    cp[3, 5, 1] = np.nan      # one interior point of one Bezier patch
    cp[7, :, :] = np.nan      # a whole patch
    sc.draws[1].mesh.cp[2, 13, 0] = np.nan
    for path in ("batched", "plain"):
        _check(sc, path)


@pytest.mark.parametrize("depth", [0, 3])
def test_depth_cap(built, cuda, depth):
    sc = _small_scene()
    _check(sc, "batched", max_split_depth=depth)


def test_eye_plane_crossing(built, cuda):
    """A heightfield seen from just above its surface: patches straddle z = 0
    in eye space and hit the depth cap near the eye."""
    from micropolis_gb300 import scenes
    sc = scenes.heightfield_1024x768()
    sc.width, sc.height = 512, 384
    sc.draws[0].mv = scenes.look_at((0.0, -0.3, 0.05), (0.0, 1.0, 0.0), (0, 0, 1))
    n = _check(sc, "batched", max_split_depth=12)
    assert n > 0


def test_overflow_regrowth(built, cuda):
    """Tiny first capacities: the frame regrows its buffers and matches."""
    sc = _small_scene(n=256)
    _check(sc, "batched", queue_capacity=256, subpatch_capacity=16)


@pytest.mark.parametrize("overlap", [0, 1])
def test_bounded_wait_reports_timeout(built, cuda, overlap):
    """With a spin limit of one iteration the waits run out: the grid holds
    far more tickets than the scene has ranges, so warps whose tickets are
    never filled check twice, 32 ns apart, long before bound-and-split ends
    (the overlapped kernel's raster blocks likewise wait for slots).  The
    frame reports MP_ERR_TIMEOUT instead of hanging and rasterizes nothing of
    its incomplete list; a fresh context renders the scene correctly."""
    from micropolis_gb300 import _lib
    sc = _small_scene(n=512)
    with pytest.raises(_lib.MpError) as e:
        _render(sc, "batched", spin_limit=1, overlap=overlap)
    assert e.value.status == _lib.MP_ERR_TIMEOUT
    _check(sc, "batched")


def test_dice16(built, cuda):
    sc = _small_scene()
    _check(sc, "batched", reyes_patch_size=16)
    _check(sc, "plain", reyes_patch_size=16)


def test_backface_culling_off(built, cuda):
    sc = _small_scene()
    _check(sc, "batched", backface_culling=False)


def test_many_views_batched_equals_per_view_plain(built, cuda):
    """Independent scenes in one batched frame (one layer each) equal the same
    scenes rendered one by one with the plain path."""
    from micropolis_gb300 import scenes
    sc = scenes.views64_512x512(n_views=8, size=256)
    for d in sc.draws:  # keep the test quick: at most 400 patches per view
        d.mesh = scenes.Mesh(d.mesh.type, d.mesh.cp[:400])
    rb = _render(sc, "batched")
    db, pb, gb = rb.subpatches()
    for v, d in enumerate(sc.draws):
        one = scenes.Scene(sc.name, sc.width, sc.height, [scenes.Draw(d.mesh, d.mv, d.color, 0)],
                           options={k: x for k, x in sc.options.items() if k != "batch_views"})
        rp = _render(one, "plain")
        _, pp, gp = rp.subpatches()
        sel = db == v
        assert subpatch_set(pb[sel], gb[sel]) == subpatch_set(pp, gp)
        cb, zb = rb.read_framebuffer(view=v)
        cp_, zp = rp.read_framebuffer()
        bad, _ = framebuffer_diff(cb, zb, cp_, zp, REL_TOL)
        assert bad <= COVERAGE_BUDGET * zb.size
        rp.close()
    rb.close()


def test_no_draws(built, cuda):
    """prepare + finish with nothing drawn leaves the cleared frame."""
    from micropolis_gb300 import scenes
    from micropolis_gb300.renderer import renderer_for
    sc = _small_scene()
    for path in ("batched", "plain"):
        r = renderer_for(sc, path)
        r.prepare()
        r.finish()
        assert r.stats()["subpatches"] == 0 and r.stats()["fragments"] == 0
        col, dep = r.read_framebuffer()
        assert np.all(dep == 0x7FFFFFFF)
        r.close()


def test_more_draws_than_staged(built, cuda):
    """100 draws (beyond the 64 draw records staged in shared memory), each a
    few patches of its own mesh, in both paths."""
    from micropolis_gb300 import scenes
    base = _small_scene(n=200)
    draws = []
    for k in range(100):
        d = base.draws[k % 2]
        draws.append(scenes.Draw(scenes.Mesh(d.mesh.type, d.mesh.cp[2 * (k // 2):2 * (k // 2) + 2].copy()), d.mv,
                                 d.color))
    sc = scenes.Scene("many", base.width, base.height, draws, options=dict(base.options))
    for path in ("batched", "plain"):
        _check(sc, path)


def test_largest_frame(built, cuda):
    """A 4096-pixel-wide frame (the fast raster's coordinate bound at 6 subpixel bits)."""
    sc = _small_scene(n=64, width=4096, height=2304)
    _check(sc, "batched")


def test_regrowth_over_many_frames(built, cuda):
    """Frames whose buffers regrow between renders (first frame from small
    capacities, then a larger scene in the same context) keep matching the
    oracle: the captured frame graph is rebuilt after every reallocation."""
    from micropolis_gb300.renderer import render_scene, renderer_for
    small = _small_scene(n=64)
    big = _small_scene(n=512)
    r = renderer_for(small, "batched", queue_capacity=64, subpatch_capacity=16)
    for sc in (small, big, small, big):
        render_scene(r, sc)
        want, ocol, odep, ost = _oracle(sc)
        d, p, g = r.subpatches()
        assert subpatch_set(p, g, d) == want
        assert r.stats()["fragments"] == ost["fragments"]
    r.close()


def test_draw_views_equals_per_draw_calls(built, cuda):
    """mp_draw_views (a batch of draws in one call) renders the frame that the
    same draws issued one by one render."""
    from micropolis_gb300 import scenes
    from micropolis_gb300.renderer import Projection, renderer_for
    sc = scenes.views64_512x512(n_views=4, size=256)
    for d in sc.draws:
        d.mesh = scenes.Mesh(d.mesh.type, d.mesh.cp[:200])
    proj = Projection(sc.fovy, sc.near, (sc.width, sc.height))
    frames = []
    for batch in (False, True):
        r = renderer_for(sc, "batched")
        for k, d in enumerate(sc.draws):
            r.load_patches(10 + k, d.mesh.cp, d.mesh.type)
        r.prepare()
        if batch:
            r.draw_views([(10 + k, d.mv, proj, d.color, d.view) for k, d in enumerate(sc.draws)])
        else:
            for k, d in enumerate(sc.draws):
                r.draw_patches(10 + k, d.mv, proj, d.color, view=d.view)
        r.finish()
        d_, p_, g_ = r.subpatches()
        frames.append((subpatch_set(p_, g_, d_), [r.read_framebuffer(view=v)[1] for v in range(4)]))
        r.close()
    assert frames[0][0] == frames[1][0]
    for a, b in zip(frames[0][1], frames[1][1]):
        assert np.array_equal(a, b)


def test_pinned_and_pageable_uploads_agree(built, cuda):
    """mp_load_patches copies a page-locked source directly and a pageable one
    through its staging buffer; both widen on the device to the same control
    points, so the frames agree: depth exactly, colour except where two
    micropolygons tie in depth (the emission order, and so which of them
    wins, varies from run to run)."""
    from micropolis_gb300 import scenes
    from micropolis_gb300.renderer import Projection, renderer_for
    torch = cuda
    sc = scenes.mixed4096_1920x1080(n=256, width=640, height=360)
    frames = []
    for pinned in (False, True):
        r = renderer_for(sc, "batched")
        proj = Projection(sc.fovy, sc.near, (sc.width, sc.height))
        for k, d in enumerate(sc.draws):
            cp = np.ascontiguousarray(d.mesh.cp, np.float32)
            if pinned:
                cp = torch.from_numpy(cp).pin_memory().numpy()
            r.load_patches(100 + k, cp, d.mesh.type)
        r.prepare()
        for k, d in enumerate(sc.draws):
            r.draw_patches(100 + k, d.mv, proj, d.color)
        r.finish()
        frames.append(r.read_framebuffer())
        r.close()
    assert np.array_equal(frames[0][1], frames[1][1])
    bad, _ = framebuffer_diff(frames[0][0], frames[0][1], frames[1][0], frames[1][1], REL_TOL)
    assert bad <= COVERAGE_BUDGET * frames[0][1].size
