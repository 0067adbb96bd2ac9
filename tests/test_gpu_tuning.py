"""Every value of the tuning knobs (key tile size, sub-patches per fused
block, bound-and-split overlapped with rasterization) renders the same
sub-patch set, fragment count and image as the oracle."""
import numpy as np
import pytest

from helpers import assert_identical_to_oracle, framebuffer_diff, subpatch_set

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
COVERAGE_BUDGET = 1e-4


def _scene(ps):
    from micropolis_gb300 import scenes
    sc = scenes.mixed4096_1920x1080(n=192, width=640, height=448)
    sc.options = dict(sc.options, reyes_patch_size=ps)
    return sc


def _oracle(sc):
    from oracle import oracle
    p = oracle.make_params(sc)
    want = set()
    for k in range(len(sc.draws)):
        pid, rng, _ = oracle.bound_n_split(sc, k, params=p)
        want |= subpatch_set(pid, rng, np.full(len(pid), k))
    col, dep, st = oracle.render(sc, params=p)
    return want, col, dep, st


@pytest.mark.parametrize("ps,groups", [(8, (8, 11, 16, 22)), (16, (2, 3, 4, 6))])
def test_knobs_match_oracle(built, cuda, ps, groups):
    """Every knob setting renders the oracle's frame: bit-identical (list
    order, colour, depth, visibility) in separate launches; the same
    sub-patch set and fragments, and pixels within the tie budget, with the
    overlapped kernel, whose numbering follows the emission order."""
    from micropolis_gb300.renderer import render_scene, renderer_for
    from oracle import oracle
    sc = _scene(ps)
    want, ocol, odep, ost = _oracle(sc)
    frame = oracle.render(sc, params=oracle.make_params(sc), want_win=True)
    for tile in (8, 16, 32):
        for group in groups:
            for overlap in (False, True):
                r = renderer_for(sc, "batched", raster_tile=tile, dice_group=group, overlap=overlap)
                render_scene(r, sc)
                if not overlap:
                    assert_identical_to_oracle(r, sc, oracle.make_params(sc), frame)
                    # clear, bound-and-split, canonical sort, dice+raster, slow raster, resolve
                    assert r.stats()["kernels"] == 6
                    r.close()
                    continue
                d, p, g = r.subpatches()
                assert subpatch_set(p, g, d) == want, (tile, group, overlap)
                assert r.stats()["fragments"] == ost["fragments"], (tile, group, overlap)
                assert r.stats()["kernels"] == 4
                col, dep = r.read_framebuffer()
                bad, _ = framebuffer_diff(col, dep, ocol, odep, REL_TOL)
                assert bad <= COVERAGE_BUDGET * dep.size, (tile, group, overlap, bad)
                r.close()


def test_rejects_unknown_knob_values(built, cuda):
    from micropolis_gb300 import _lib
    from micropolis_gb300.renderer import renderer_for
    sc = _scene(8)
    for over in ({"raster_tile": 12}, {"dice_group": 5}):
        with pytest.raises(_lib.MpError) as e:
            renderer_for(sc, "batched", **over)
        assert e.value.status == _lib.MP_ERR_INVALID_ARG


def test_autotuner_on_gpu(built, cuda, tmp_path):
    """The tuner times every candidate on the device, caches the choice, and
    the tuned renderer draws the oracle's sub-patch set."""
    from micropolis_gb300 import autotune
    from micropolis_gb300.renderer import render_scene
    sc = _scene(8)
    cache = str(tmp_path / "tune.json")
    res = autotune.tune(sc, frames=2, warmup=1, cache=cache)
    assert len(res.trials) == 12 and all(t.ms > 0 for t in res.trials)
    assert not any(t.options["overlap"] for t in res.trials)
    assert len({t.micropolygons for t in res.trials}) == 1
    assert autotune.tune(sc, cache=cache).cached
    r = autotune.tuned_renderer(sc, cache=cache)
    render_scene(r, sc)
    want, _, _, _ = _oracle(sc)
    d, p, g = r.subpatches()
    assert subpatch_set(p, g, d) == want
    r.close()
