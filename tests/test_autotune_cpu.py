"""Autotuner host logic on the CPU: search space, selection, signature and the
JSON cache, with a fake timer in place of GPU frames."""
import json

import pytest

from micropolis_gb300 import autotune, scenes


def _scene(n=64, **kw):
    return scenes.mixed4096_1920x1080(n=n, width=kw.pop("width", 256), height=kw.pop("height", 256), **kw)


def test_candidates_cover_space_default_first():
    c8 = autotune.candidates(8)
    assert len(c8) == 4 * 3 * 2
    assert c8[0] == {"dice_group": 11, "raster_tile": 8, "overlap": False}
    assert {c["dice_group"] for c in c8} == {8, 11, 16, 22}
    c16 = autotune.candidates(16)
    assert {c["dice_group"] for c in c16} == {2, 3, 4, 6}
    both = autotune.candidates(8, tune_patch_size=True)
    assert len(both) == 48 and {c["reyes_patch_size"] for c in both} == {8, 16}


def test_choose_by_time_and_by_rate():
    t = [autotune.Trial({"a": 0}, 2.0, 100), autotune.Trial({"a": 1}, 1.5, 100),
         autotune.Trial({"a": 2}, 1.5, 100), autotune.Trial({"a": 3}, 3.0, 400)]
    assert autotune.choose(t, by_rate=False).options == {"a": 1}      # ties keep the earlier one
    assert autotune.choose(t, by_rate=True).options == {"a": 3}
    # within the margin the earlier candidate wins
    near = [autotune.Trial({"a": 0}, 1.005, 100), autotune.Trial({"a": 1}, 1.0, 100)]
    assert autotune.choose(near, by_rate=False).options == {"a": 0}
    assert autotune.choose(near, by_rate=False, margin=0.0).options == {"a": 1}
    with pytest.raises(ValueError):
        autotune.choose([], by_rate=False)


def test_signature_depends_on_shape_not_values():
    a = _scene(seed=1)
    b = _scene(seed=2)
    assert autotune.signature(a) == autotune.signature(b)
    assert autotune.signature(a) != autotune.signature(_scene(width=512))
    assert autotune.signature(a) != autotune.signature(_scene(n=4096))
    assert autotune.signature(a) != autotune.signature(a, {"reyes_patch_size": 16})
    assert autotune.signature(a, device="x") != autotune.signature(a, device="y")


def test_tune_picks_fastest_and_caches(tmp_path):
    cache = str(tmp_path / "c.json")
    sc = _scene()
    calls = []

    def fake(scene, opts, frames, warmup):
        calls.append(dict(opts))
        ms = 1.0 + 0.1 * opts["dice_group"] / 8 + (0.0 if opts["raster_tile"] == 16 else 0.05) \
            - (0.2 if opts["overlap"] else 0.0)
        return autotune.Trial(dict(opts), ms, 1000)

    # by default only separate launches (the canonical, deterministic numbering) are candidates
    r = autotune.tune(sc, cache=cache, measure=fake, device="dev")
    assert r.best == {"dice_group": 8, "raster_tile": 16, "overlap": False}
    assert not r.cached and len(calls) == 12 and len(r.trials) == 12
    data = json.load(open(cache))
    assert data["version"] == autotune.CACHE_VERSION and r.key in data
    r2 = autotune.tune(sc, cache=cache, measure=fake, device="dev")
    assert r2.cached and r2.best == r.best and len(calls) == 12
    # another device tunes again
    autotune.tune(sc, cache=cache, measure=fake, device="other")
    assert len(calls) == 24
    # the overlapped launch, when the caller allows it, is tuned and cached apart
    r3 = autotune.tune(sc, cache=cache, measure=fake, device="dev", allow_overlap=True)
    assert r3.best == {"dice_group": 8, "raster_tile": 16, "overlap": True} and not r3.cached
    assert len(calls) == 48 and r3.key != r.key


def test_tune_patch_size_scores_rate(tmp_path):
    sc = _scene()

    def fake(scene, opts, frames, warmup):
        ps = opts["reyes_patch_size"]
        return autotune.Trial(dict(opts), 2.0 if ps == 16 else 1.0, 4000 if ps == 16 else 1000)

    r = autotune.tune(sc, tune_patch_size=True, use_cache=False, measure=fake, device="")
    assert r.best["reyes_patch_size"] == 16


def test_bad_cache_file_is_ignored(tmp_path):
    p = tmp_path / "c.json"
    p.write_text("{not json")
    assert autotune.load_cache(str(p)) == {"version": autotune.CACHE_VERSION}
    p.write_text(json.dumps({"version": -1, "k": 1}))
    assert autotune.load_cache(str(p)) == {"version": autotune.CACHE_VERSION}
