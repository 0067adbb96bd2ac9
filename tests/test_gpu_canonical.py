"""Canonical numbering of the batched path: bound-and-split's output is put
in ascending (root, split path) order before rasterization, so a frame's
sub-patch list, its micropolygon numbers and the winners of depth ties do not
depend on how the GPU scheduled the work.  The oracle numbers its
micropolygons in the same order, so batched frames are bit-identical to the
oracle's at every pixel, visibility included."""
import numpy as np
import pytest

from helpers import assert_identical_to_oracle

pytestmark = pytest.mark.gpu


def _render(scene, **over):
    from micropolis_gb300.renderer import render_scene, renderer_for
    r = renderer_for(scene, "batched", **over)
    render_scene(r, scene)
    return r


def _scenes():
    from micropolis_gb300 import scenes
    return {
        "heightfield_1024x768": (scenes.heightfield_1024x768(), {}),
        "mixed256_640x360": (scenes.mixed4096_1920x1080(n=256, width=640, height=360), {}),
        "heightfield16_displaced": (scenes.heightfield16_512x512(), {}),
        "mixed256_dice16": (scenes.mixed4096_1920x1080(n=256, width=640, height=360), {"reyes_patch_size": 16}),
        "mixed256_no_backface": (scenes.mixed4096_1920x1080(n=256, width=640, height=360),
                                 {"backface_culling": 0}),
        "mixed256_gpu_criterion": (scenes.mixed4096_1920x1080(n=256, width=640, height=360),
                                   {"bound_criterion": 1}),
    }


@pytest.mark.parametrize("name", list(_scenes()))
def test_batched_frame_identical_to_oracle(built, cuda, name):
    from oracle import oracle
    sc, over = _scenes()[name]
    sc.options.update(over)
    r = _render(sc)
    assert_identical_to_oracle(r, sc, oracle.make_params(sc))
    r.close()


@pytest.mark.parametrize("tile", [8, 32])
def test_every_pixel_a_tie(built, cuda, tile):
    """The same mesh drawn twice with the same modelview in two colours:
    every covered pixel is a tie between the two draws, and the first draw's
    micropolygons (smaller numbers) win all of them, as in the oracle."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    base = scenes.heightfield_1024x768()
    d0 = base.draws[0]
    d1 = scenes.Draw(d0.mesh, d0.mv.copy(), (0.2, 0.9, 0.4, 1.0))
    sc = scenes.Scene("twice", base.width, base.height, [d0, d1], fovy=base.fovy, near=base.near,
                      options=dict(base.options))
    r = _render(sc, raster_tile=tile)
    assert_identical_to_oracle(r, sc, oracle.make_params(sc))
    vis = r.visibility()
    n0 = r.stats()["subpatches"] // 2 * 64
    covered = vis >= 0
    assert covered.any() and np.all(vis[covered] < n0)
    r.close()


def test_fresh_contexts_give_identical_frames(built, cuda):
    """Two renders of the full-size mixed scene, each in a fresh context:
    identical sub-patch lists, colour, depth and visibility."""
    from micropolis_gb300 import scenes
    sc = scenes.mixed4096_1920x1080()
    out = []
    for _ in range(2):
        r = _render(sc)
        d, p, g = r.subpatches()
        col, dep = r.read_framebuffer()
        out.append((d, p, g.view(np.uint32), col.view(np.uint32), dep, r.visibility()))
        r.close()
    for a, b in zip(*out):
        assert np.array_equal(a, b)


def test_adjoint_forward_deterministic(built, cuda):
    """The differentiable renderer's forward pass twice in fresh contexts:
    identical images and visibility (the visibility the backward holds fixed)."""
    import torch
    from micropolis_gb300 import adjoint, scenes
    sc = scenes.heightfield16_512x512()
    cp = torch.tensor(sc.draws[0].mesh.cp, device="cuda")
    imgs, vis = [], []
    for _ in range(2):
        dr = adjoint.DiffRenderer(sc)
        imgs.append(dr.render(cp, torch.tensor(1.1, device="cuda")).cpu().numpy())
        torch.cuda.synchronize()
        vis.append(dr.r.visibility())
        dr.r.close()
    assert np.array_equal(imgs[0].view(np.uint32), imgs[1].view(np.uint32))
    assert np.array_equal(vis[0], vis[1])
