"""GPU parity of the REYES core against the CPU oracle, through the C ABI.

Sub-patch sets must be bit-identical to the oracle's restatement of the
reference's CPU bound-and-split.  Framebuffers must match the oracle's
restatement of the dice/shade/sample kernels within 1e-5 relative per pixel
(colour) and exactly (int depth), with differing pixels below 1e-4 of the
frame (ties between equally deep micropolygons resolve by the smaller id here
and by the first writer in the oracle).
"""
import ctypes

import numpy as np
import pytest

from helpers import framebuffer_diff, subpatch_set

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
COVERAGE_BUDGET = 1e-4


def _render(scene, path, **over):
    from micropolis_gb300.renderer import render_scene, renderer_for
    r = renderer_for(scene, path, **over)
    render_scene(r, scene)
    return r


def _oracle_set(scene, **over):
    from oracle import oracle
    p = oracle.make_params(scene, **over)
    out = set()
    for k in range(len(scene.draws)):
        pid, rng, _ = oracle.bound_n_split(scene, k, params=p)
        out |= subpatch_set(pid, rng, np.full(len(pid), k))
    return out


def _check_frame(scene, r, **over):
    from oracle import oracle
    p = oracle.make_params(scene, **over)
    ocol, odep, ost = oracle.render(scene, params=p)
    col, dep = r.read_framebuffer()
    bad, inexact = framebuffer_diff(col, dep, ocol, odep, REL_TOL)
    assert bad <= COVERAGE_BUDGET * dep.size, f"{bad} pixels differ (budget {COVERAGE_BUDGET * dep.size:.0f})"
    st = r.stats()
    assert st["micropolygons"] == ost["micropolygons"]
    assert st["fragments"] == ost["fragments"]
    return bad, inexact


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_heightfield_subpatches_bit_exact(built, cuda, path):
    from micropolis_gb300 import scenes
    sc = scenes.heightfield_1024x768()
    r = _render(sc, path)
    draw, pid, rng = r.subpatches()
    assert subpatch_set(pid, rng, draw) == _oracle_set(sc)
    st = r.stats()
    assert st["micropolygons"] == 64 * len(pid)
    r.close()


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_heightfield_framebuffer_matches_oracle(built, cuda, path):
    from micropolis_gb300 import scenes
    sc = scenes.heightfield_1024x768()
    r = _render(sc, path)
    bad, inexact = _check_frame(sc, r)
    r.close()


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_mixed_bezier_gregory_small(built, cuda, path):
    from micropolis_gb300 import scenes
    sc = scenes.mixed4096_1920x1080(n=256, width=640, height=360)
    r = _render(sc, path)
    draw, pid, rng = r.subpatches()
    assert subpatch_set(pid, rng, draw) == _oracle_set(sc)
    _check_frame(sc, r)
    r.close()


def test_displaced_heightfield(built, cuda):
    from micropolis_gb300 import scenes
    sc = scenes.heightfield16_512x512()
    r = _render(sc, "batched")
    draw, pid, rng = r.subpatches()
    assert subpatch_set(pid, rng, draw) == _oracle_set(sc)
    _check_frame(sc, r)
    r.close()


def test_plain_equals_batched(built, cuda):
    from micropolis_gb300 import scenes
    sc = scenes.mixed4096_1920x1080(n=512, width=1024, height=576)
    a = _render(sc, "batched")
    b = _render(sc, "plain", reyes_patches_per_pass=1024)
    da, pa, ra = a.subpatches()
    db, pb, rb = b.subpatches()
    assert subpatch_set(pa, ra, da) == subpatch_set(pb, rb, db)
    ca, za = a.read_framebuffer()
    cb, zb = b.read_framebuffer()
    bad, _ = framebuffer_diff(ca, za, cb, zb, REL_TOL)
    assert bad <= COVERAGE_BUDGET * za.size
    assert b.stats()["passes"] > 1
    a.close()
    b.close()


def test_dice_positions_match_fp64(built, cuda):
    from micropolis_gb300 import scenes
    from oracle import oracle
    for sc in (scenes.heightfield_1024x768(), scenes.heightfield16_512x512()):
        r = _render(sc, "batched")
        draw, pid, rng = r.subpatches()
        sel = np.random.default_rng(0).choice(len(pid), size=min(64, len(pid)), replace=False)
        pos, pxl, dep = r.dice_subpatches(0, pid[sel], rng[sel])
        for k, s in enumerate(sel):
            ref = oracle.dice_fp64(sc, 0, pid[s], rng[s])
            err = np.abs(pos[k, :, :3] - ref).max() / max(np.abs(ref).max(), 1e-30)
            assert err < 2e-6, err
            opos, opxl, odep = oracle.dice(sc, 0, pid[s], rng[s])
            assert np.array_equal(pos[k], opos) and np.array_equal(pxl[k], opxl) and np.array_equal(dep[k], odep)
        r.close()


def test_prefix_sum_reference_selftest(built, cuda):
    """The reference's test_CL_prefix_sum (src/micropolis/main.cpp:343-400):
    srand(43), values rand()%8+1, inclusive scan and total."""
    from micropolis_gb300.renderer import Renderer
    libc = ctypes.CDLL(None)
    libc.srand(43)
    for n in (1, 127, 128, 1000, 4096, 100000, 1 << 20):
        vals = np.array([libc.rand() % 8 + 1 for _ in range(n)] if n <= 4096 else
                        np.random.default_rng(n).integers(1, 9, n), np.int32)
        r = Renderer(window_size=(64, 64))
        out = r.inclusive_scan(vals)
        assert np.array_equal(out, np.cumsum(vals, dtype=np.int64).astype(np.int32))
        r.close()


def test_gregory_form_dices_to_the_bezier_surface(built, cuda):
    """Known answer of tools/bez2mscene_greg.py:111 on the CUDA dicer: a
    Bezier patch and its 20-point Gregory form dice to the same surface
    (within a few FP32 roundings), and each form's grid is bit-exact to the
    oracle's."""
    from oracle import oracle
    from test_bez2greg_cpu import RANGES, REL_TOL, bezier_and_gregory_scene
    sc = bezier_and_gregory_scene()
    r = _render(sc, "batched")
    n = sc.draws[0].mesh.n_patches
    pid = np.repeat(np.arange(n, dtype=np.int32), len(RANGES))
    rng = np.tile(RANGES, (n, 1))
    pb, xb, db = r.dice_subpatches(0, pid, rng)
    pg, xg, dg = r.dice_subpatches(1, pid, rng)
    for k in range(len(pid)):
        scale = np.abs(pb[k, :, :3]).max()
        assert np.abs(pg[k, :, :3] - pb[k, :, :3]).max() <= REL_TOL * scale, k
        assert np.abs(xg[k] - xb[k]).max() <= 1
        for draw, pos, pxl, dep in ((0, pb, xb, db), (1, pg, xg, dg)):
            opos, opxl, odep = oracle.dice(sc, draw, pid[k], rng[k])
            assert np.array_equal(pos[k], opos) and np.array_equal(pxl[k], opxl) and np.array_equal(dep[k], odep)
    r.close()
