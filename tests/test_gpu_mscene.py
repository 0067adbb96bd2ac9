"""A scene written as a packed .mscene file and drawn through mp_scene_draw
(Reyes::Scene::draw over the C ABI) renders the oracle's sub-patch set and
image, and the same frame as drawing its objects one by one."""
import numpy as np
import pytest

from helpers import framebuffer_diff, subpatch_set

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_mscene_draw_matches_oracle(built, cuda, path, tmp_path):
    from micropolis_gb300 import mscene, scenes
    from micropolis_gb300.renderer import render_scene, renderer_for
    from oracle import oracle
    src = scenes.mixed4096_1920x1080(n=256, width=640, height=448)
    meshes, objects, cams = mscene.records_from_scene(src, mscene.camera_from_view(src.draws[0].mv))
    objects[1].transform = mscene.Transform((0.3, -0.2, 0.1), (np.cos(0.1), 0.0, 0.0, np.sin(0.1)))
    f = tmp_path / "scene.mscene"
    mscene.write_mscene(str(f), meshes, objects, cams)
    sf = mscene.SceneFile.load(str(f))
    sc = sf.to_scene(src.width, src.height)
    r = renderer_for(sc, path)
    sf.draw(r)
    d, pid, rng = r.subpatches()
    got = subpatch_set(pid, rng, d)
    want = set()
    for k in range(len(sc.draws)):
        p_, r_, _ = oracle.bound_n_split(sc, k)
        want |= subpatch_set(p_, r_, np.full(len(p_), k))
    assert got == want and len(got) > 0
    col, dep = r.read_framebuffer()
    ocol, odep, ost = oracle.render(sc)
    bad, _ = framebuffer_diff(col, dep, ocol, odep, 1e-5)
    assert bad <= 1e-4 * dep.size
    # drawing the converted scene object by object gives the same frame (up
    # to which of two micropolygons at exactly equal depth a pixel shows: the
    # batched path's emission order, and so the id tie-break, varies per run)
    r2 = renderer_for(sc, path)
    render_scene(r2, sc)
    col2, dep2 = r2.read_framebuffer()
    assert np.array_equal(dep, dep2)
    bad, _ = framebuffer_diff(col, dep, col2, dep2, 1e-5)
    assert bad <= 1e-4 * dep.size
    r.close()
    r2.close()
