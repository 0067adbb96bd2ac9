"""The reference's GPU bound criterion (kernels/bound_n_split.h) as an option:
the batched and plain paths emit the oracle's sub-patch set for it bit for
bit and render the oracle's image, on the mixed scene and on a heightfield
seen from just above (eye-plane split rule and depth cull)."""
import numpy as np
import pytest

from helpers import framebuffer_diff, subpatch_set

pytestmark = pytest.mark.gpu

REL_TOL = 1e-5
COVERAGE_BUDGET = 1e-4


def _scenes():
    from micropolis_gb300 import scenes
    mixed = scenes.mixed4096_1920x1080(n=256, width=640, height=448)
    low = scenes.heightfield_1024x768()
    low.width, low.height = 512, 384
    low.draws[0].mv = scenes.look_at((0.0, -0.3, 0.05), (0.0, 1.0, 0.0), (0, 0, 1))
    return [mixed, low]


@pytest.mark.parametrize("which", [0, 1])
@pytest.mark.parametrize("path", ["batched", "plain"])
def test_gpu_criterion_matches_oracle(built, cuda, which, path):
    from micropolis_gb300.renderer import render_scene, renderer_for
    from oracle import oracle
    sc = _scenes()[which]
    over = dict(bound_criterion=1, max_split_depth=12)
    p = oracle.make_params(sc, **over)
    want = set()
    for k in range(len(sc.draws)):
        pid, rng, _ = oracle.bound_n_split(sc, k, params=p)
        want |= subpatch_set(pid, rng, np.full(len(pid), k))
    cpu = set()
    for k in range(len(sc.draws)):
        pid, rng, _ = oracle.bound_n_split(sc, k, params=oracle.make_params(sc, max_split_depth=12))
        cpu |= subpatch_set(pid, rng, np.full(len(pid), k))
    assert want and want != cpu
    r = renderer_for(sc, path, **over)
    render_scene(r, sc)
    d, pid, rng = r.subpatches()
    assert subpatch_set(pid, rng, d) == want
    col, dep = r.read_framebuffer()
    ocol, odep, ost = oracle.render(sc, params=p)
    bad, _ = framebuffer_diff(col, dep, ocol, odep, REL_TOL)
    assert bad <= COVERAGE_BUDGET * dep.size
    assert r.stats()["fragments"] == ost["fragments"]
    r.close()
