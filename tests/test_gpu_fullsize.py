"""Full-size workloads, checked through properties that do not need the CPU
to render the frame: bit-exact sub-patch sets against the oracle's
bound-and-split, batched path equal to the plain per-pass path, determinism,
micropolygon counts, and dyadic ranges inside [0,1]^2."""
import numpy as np
import pytest

from helpers import framebuffer_diff, subpatch_set


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
    for k in range(2):
        pid, rng, _ = oracle.bound_n_split(sc, k)
        want |= subpatch_set(pid, rng, np.full(len(pid), k))
    assert got == want
    assert _dyadic_ok(gb)
    assert rb.stats()["micropolygons"] == 64 * len(pb)
    assert rb.stats()["fragments"] == rp.stats()["fragments"]
    cb, zb = rb.read_framebuffer()
    cp_, zp = rp.read_framebuffer()
    bad, _ = framebuffer_diff(cb, zb, cp_, zp, REL_TOL)
    assert bad <= COVERAGE_BUDGET * zb.size
    # a second frame renders the same image
    from micropolis_gb300.renderer import render_scene
    render_scene(rb, sc)
    cb2, zb2 = rb.read_framebuffer()
    bad, _ = framebuffer_diff(cb, zb, cb2, zb2, REL_TOL)
    assert bad <= COVERAGE_BUDGET * zb.size
    rb.close()
    rp.close()


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
