"""Full-size workloads: the headline mixed scene's whole frame, four of the
64 views at their full patch counts and a crop of the 4K displaced
heightfield, each bit-identical to the oracle (colour, depth, winning
micropolygon); and properties the whole frames keep: bit-exact sub-patch
sets against the oracle's bound-and-split, batched path equal to the plain
per-pass path, determinism, micropolygon counts, and dyadic ranges inside
[0,1]^2."""
import os

import numpy as np
import pytest

from helpers import assert_identical_to_oracle, framebuffer_diff, same_colour, subpatch_set


@pytest.fixture(scope="module")
def pool():
    """Oracle worker processes (spawned: never forked from a process that
    has touched the GPU)."""
    import multiprocessing as mp
    p = mp.get_context("spawn").Pool(min(16, os.cpu_count() or 1))
    yield p
    p.close()
    p.join()


def _sorted_records(pid, rng, draw=None):
    """Sub-patch records as one sorted structured array (bit patterns)."""
    n = len(pid)
    rec = np.zeros(n, dtype=[("d", "<i4"), ("p", "<i4"), ("r", "<u4", 4)])
    rec["d"] = 0 if draw is None else draw
    rec["p"] = pid
    rec["r"] = np.ascontiguousarray(rng, np.float32).view(np.uint32).reshape(n, 4)
    return np.sort(rec.view(np.dtype((np.void, rec.dtype.itemsize))))

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
COVERAGE_BUDGET = 1e-4


def _render(scene, path, **over):
    from micropolis_gb300.renderer import render_scene, renderer_for
    r = renderer_for(scene, path, **over)
    render_scene(r, scene)
    return r


def _dyadic_ok(rng):
    w = rng[:, 2] - rng[:, 0]
    h = rng[:, 3] - rng[:, 1]
    mw, _ = np.frexp(w)
    mh, _ = np.frexp(h)
    aligned = np.all(np.mod(rng[:, 0], w) == 0) and np.all(np.mod(rng[:, 1], h) == 0)
    return bool(np.all(mw == 0.5) and np.all(mh == 0.5) and aligned and np.all(rng >= 0) and np.all(rng <= 1))


def test_mixed4096_full_size(built, cuda):
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.mixed4096_1920x1080()
    rb = _render(sc, "batched")
    rp = _render(sc, "plain")
    db, pb, gb = rb.subpatches()
    dp, pp, gp = rp.subpatches()
    got = subpatch_set(pb, gb, db)
    assert len(got) == len(pb)                      # no duplicates
    assert got == subpatch_set(pp, gp, dp)
    want = set()
    bounds = 0
    for k in range(2):
        pid, rng, nb = oracle.bound_n_split(sc, k)
        want |= subpatch_set(pid, rng, np.full(len(pid), k))
        bounds += nb
    assert got == want
    # every range bounded once, as by the oracle's bound-and-split
    assert rb.stats()["bounds"] == bounds
    assert _dyadic_ok(gb)
    assert rb.stats()["micropolygons"] == 64 * len(pb)
    assert rb.stats()["fragments"] == rp.stats()["fragments"]
    cb, zb = rb.read_framebuffer()
    cp_, zp = rp.read_framebuffer()
    bad, _ = framebuffer_diff(cb, zb, cp_, zp, REL_TOL)
    assert bad <= COVERAGE_BUDGET * zb.size
    # a second frame renders the same image, bit for bit
    from micropolis_gb300.renderer import render_scene
    render_scene(rb, sc)
    cb2, zb2 = rb.read_framebuffer()
    assert np.array_equal(zb, zb2) and same_colour(cb, cb2).all()
    rb.close()
    rp.close()


def test_mixed4096_full_size_gpu_criterion(built, cuda):
    """The headline scene under the reference's GPU bound criterion
    (bound_criterion = 1): both paths emit the oracle's set of that
    criterion, every range bounded once, and render the same frame."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.mixed4096_1920x1080()
    rb = _render(sc, "batched", bound_criterion=1)
    rp = _render(sc, "plain", bound_criterion=1)
    db, pb, gb = rb.subpatches()
    dp, pp, gp = rp.subpatches()
    got = subpatch_set(pb, gb, db)
    assert len(got) == len(pb)
    assert got == subpatch_set(pp, gp, dp)
    p = oracle.make_params(sc, bound_criterion=1)
    want = set()
    bounds = 0
    for k in range(len(sc.draws)):
        pid, rng, nb = oracle.bound_n_split(sc, k, params=p)
        want |= subpatch_set(pid, rng, np.full(len(pid), k))
        bounds += nb
    assert got == want
    assert rb.stats()["bounds"] == bounds
    assert _dyadic_ok(gb)
    cb, zb = rb.read_framebuffer()
    cp_, zp = rp.read_framebuffer()
    bad, _ = framebuffer_diff(cb, zb, cp_, zp, REL_TOL)
    assert bad <= COVERAGE_BUDGET * zb.size
    rb.close()
    rp.close()


@pytest.mark.parametrize("over", [{}, {"bound_criterion": 1}, {"reyes_patch_size": 16}],
                         ids=["default", "gpu_criterion", "dice16"])
def test_mixed4096_frame_identical_to_oracle(built, cuda, pool, over):
    """The headline frame (4,096 mixed patches, 1920x1080, limit 8, dice
    8x8), and the same scene under the reference's GPU bound criterion and
    at 16x16 dicing: canonical sub-patch list, colour, depth and visibility
    bit-identical to the oracle's frame at every pixel."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.mixed4096_1920x1080()
    r = _render(sc, "batched", **over)
    frame = oracle.render_parallel(sc, pool, params_over=over)
    assert_identical_to_oracle(r, sc, oracle.make_params(sc, **over), frame)
    r.close()


def test_views64_four_layers_identical_to_oracle(built, cuda):
    """The 64-view frame at full patch counts: four of its layers, each
    against the oracle's frame of that view's draw alone (its micropolygon
    numbers offset by the sub-patches of the earlier draws)."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.views64_512x512()
    r = _render(sc, "batched")
    draw, pid, rng = r.subpatches()
    counts = np.bincount(draw, minlength=len(sc.draws))
    first = np.concatenate([[0], np.cumsum(counts)[:-1]])
    for v in (0, 21, 42, 63):
        d = sc.draws[v]
        one = scenes.Scene(sc.name, sc.width, sc.height, [scenes.Draw(d.mesh, d.mv, d.color, 0)], fovy=sc.fovy,
                           near=sc.near, options={k: x for k, x in sc.options.items() if k != "batch_views"})
        p = oracle.make_params(one)
        odraw, opid, orng, _ = oracle.canonical_subpatches(one, p)
        sl = slice(first[v], first[v] + counts[v])
        assert np.array_equal(pid[sl], opid)
        assert np.array_equal(rng[sl].view(np.uint32), orng.view(np.uint32))
        ocol, odep, owin, _ = oracle.render(one, params=p, want_win=True)
        col, dep = r.read_framebuffer(view=v)
        assert np.array_equal(dep, odep) and same_colour(col, ocol).all(), v
        vis = r.visibility(view=v)
        want = np.where(owin >= 0, owin + first[v] * 64, -1)
        assert np.array_equal(vis, want), v
    r.close()


def _crop_patches(scene, x0, y0, x1, y1, margin_px=4):
    """Patches whose displaced surface can reach pixels [x0, x1) x [y0, y1):
    the eye-space box of the control points (a Bezier patch lies in their
    convex hull) grown by the largest displacement (0.07 x amplitude per
    coordinate, kernels/dice.cl:51-67), projected through its corners; boxes
    reaching the eye plane are kept."""
    d = scene.draws[0]
    mv = np.asarray(d.mv, np.float64).reshape(4, 4).T
    cp = d.mesh.cp.astype(np.float64)
    eye = cp @ mv[:3, :3].T + mv[:3, 3]
    amp = float(scene.options.get("displacement_amplitude", 1.0)) if scene.options.get("displacement") else 0.0
    m = 0.07 * abs(amp) * 1.01 + 1e-6
    lo, hi = eye.min(axis=1) - m, eye.max(axis=1) + m
    keep = hi[:, 2] >= -scene.near
    f = 1.0 / np.tan(np.radians(scene.fovy) / 2)
    aspect = scene.width / scene.height
    corners = np.stack([np.stack([np.where(k & 1, hi[:, 0], lo[:, 0]), np.where(k & 2, hi[:, 1], lo[:, 1]),
                                  np.where(k & 4, hi[:, 2], lo[:, 2])], -1) for k in range(8)], 1)
    w = -corners[:, :, 2]
    with np.errstate(divide="ignore", invalid="ignore"):
        px = (f / aspect) * corners[:, :, 0] / w * scene.width / 2 + scene.width / 2
        py = f * corners[:, :, 1] / w * scene.height / 2 + scene.height / 2
    hit = (px.min(1) <= x1 + margin_px) & (px.max(1) >= x0 - margin_px) & \
          (py.min(1) <= y1 + margin_px) & (py.max(1) >= y0 - margin_px)
    return np.nonzero(keep | hit)[0]


def test_heightfield512_4k_crop_identical_to_oracle(built, cuda, pool):
    """A 256x256-pixel crop of the 262,144-patch displaced heightfield at
    3840x2160 (limit 4 px): colour, depth and the winning micropolygon's
    identity (patch, range, quad) at every crop pixel equal the oracle's
    frame of the patches that can reach the crop."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.heightfield512_3840x2160()
    r = _render(sc, "batched")
    col, dep = r.read_framebuffer(linear=True)
    vis_t = r.visibility()
    draw, pid, rng = r.subpatches()
    x0, y0, x1, y1 = 1792, 952, 2048, 1208
    sel = _crop_patches(sc, x0, y0, x1, y1)
    assert 0 < len(sel) < sc.n_patches // 4
    d = sc.draws[0]
    sub = scenes.Scene(sc.name, sc.width, sc.height, [scenes.Draw(scenes.Mesh(d.mesh.type, d.mesh.cp[sel]), d.mv,
                                                                  d.color)],
                       fovy=sc.fovy, near=sc.near, options=dict(sc.options))
    p = oracle.make_params(sub)
    _, opid, orng, _ = oracle.canonical_subpatches(sub, p)
    ocol_t, odep_t, owin_t, _ = oracle.render_parallel(sub, pool)
    # tiled -> row-major for the crop
    W, H = sc.width, sc.height
    yy, xx = np.mgrid[y0:y1, x0:x1]
    tiled = ((xx // 8) + (W // 8) * (yy // 8)) * 64 + (xx % 8) + 8 * (yy % 8)
    lin = yy * W + xx
    assert np.array_equal(dep[lin], odep_t[tiled])
    assert same_colour(col[lin], ocol_t[tiled]).all()
    g = vis_t[tiled]
    o = owin_t[tiled]
    assert np.array_equal(g >= 0, o >= 0)
    covered = g >= 0
    assert covered.mean() > 0.5
    gs, gq = g[covered] // 64, g[covered] % 64
    os_, oq = o[covered] // 64, o[covered] % 64
    assert np.array_equal(gq, oq)
    assert np.array_equal(pid[gs], sel[opid[os_]])
    assert np.array_equal(rng[gs].view(np.uint32), orng[os_].view(np.uint32))
    r.close()


def test_heightfield512_4k_full_size(built, cuda):
    """262,144-patch fractal heightfield at 3840x2160, split limit 4 px,
    displacement on: batched equals plain, sub-patch set equals the oracle's."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.heightfield512_3840x2160()
    rb = _render(sc, "batched")
    st = rb.stats()
    assert st["subpatches"] > 1_000_000
    db, pb, gb = rb.subpatches()
    pid, rng, _ = oracle.bound_n_split(sc, 0)
    got, want = _sorted_records(pb, gb), _sorted_records(pid, rng)
    assert len(got) == len(want) and np.array_equal(got, want)
    assert _dyadic_ok(gb)
    rp = _render(sc, "plain")
    assert rp.stats()["subpatches"] == st["subpatches"]
    assert rp.stats()["fragments"] == st["fragments"]
    cb, zb = rb.read_framebuffer()
    cp_, zp = rp.read_framebuffer()
    bad, _ = framebuffer_diff(cb, zb, cp_, zp, REL_TOL)
    assert bad <= COVERAGE_BUDGET * zb.size
    rb.close()
    rp.close()
