"""Both CUDA paths against the golden vectors of the reference's own CPU
bound-and-split (tests/golden/): the emitted sub-patch set, bit for bit; and
against golden framebuffers of the reference's own kernels: identical
coverage, depth and colour within 1e-5 except in < 1e-4 of the pixels."""
import numpy as np
import pytest

from helpers import GOLDEN_CASES, GOLDEN_FRAMES, frame_agrees, golden_case, golden_frame, subpatch_set

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", ["batched", "plain"])
@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_cuda_matches_golden(built, cuda, name, path):
    from micropolis_gb300.renderer import render_scene, renderer_for
    sc, opts, gpid, grng = golden_case(name)
    r = renderer_for(sc, path, **opts)
    render_scene(r, sc)
    d, pid, rng = r.subpatches()
    got = subpatch_set(pid, rng, d)
    assert len(got) == len(pid) == len(gpid)
    assert got == subpatch_set(gpid, grng, np.zeros(len(gpid), np.int32))
    r.close()


@pytest.mark.parametrize("path", ["batched", "plain"])
@pytest.mark.parametrize("name", GOLDEN_FRAMES)
def test_cuda_matches_golden_frame(built, cuda, name, path):
    from micropolis_gb300.renderer import render_scene, renderer_for
    sc, opts, gcolor, gdepth = golden_frame(name)
    r = renderer_for(sc, path, **opts)
    render_scene(r, sc)
    col, dep = r.read_framebuffer()
    # every pixel, the cleared ones included (the clear colour's powf runs on
    # this host, the fixture's where it was written)
    frame_agrees(col, dep, gcolor, gdepth)
    r.close()
