"""The oracle against golden vectors of the reference's own CPU
bound-and-split (tests/golden/, written by tests/golden/make_golden.py from
the reference's src/base/Patch.cpp and Projection.cpp): the same sub-patches,
bit for bit, in the same emission order; and against golden framebuffers of
the reference's own kernels (tests/golden/make_golden_frames.py)."""
import numpy as np
import pytest

from helpers import (GOLDEN_CASES, GOLDEN_FRAMES, GOLDEN_GPU_CRITERION, frame_agrees, golden_case, golden_frame,
                     golden_gpucrit, subpatch_set)


@pytest.mark.parametrize("name", GOLDEN_CASES)
def test_oracle_matches_golden(built, name):
    from oracle import oracle
    sc, opts, gpid, grng = golden_case(name)
    pid, rng, _ = oracle.bound_n_split(sc, 0, params=oracle.make_params(sc, **opts))
    assert len(gpid) > 0
    assert np.array_equal(pid, gpid)
    assert np.array_equal(rng.view(np.uint32), grng.view(np.uint32))


@pytest.mark.parametrize("name", GOLDEN_FRAMES)
def test_oracle_matches_golden_frame(built, name):
    """The oracle's frame against the reference kernels' own framebuffer
    (tests/golden/make_golden_frames.py): identical coverage and clear
    pixels, depth and colour within 1e-5 except in < 1e-4 of the pixels."""
    from oracle import oracle
    sc, opts, gcolor, gdepth = golden_frame(name)
    col, dep, _ = oracle.render(sc, params=oracle.make_params(sc, **opts))
    empty = gdepth == 0x7fffffff
    assert np.array_equal(col[empty].view(np.uint32), gcolor[empty].view(np.uint32))
    frame_agrees(col, dep, gcolor, gdepth)


@pytest.mark.parametrize("name", GOLDEN_GPU_CRITERION)
def test_oracle_gpu_criterion_matches_golden(built, name):
    """The oracle's GPU bound criterion against the set of the reference's
    own bound() (kernels/bound_n_split.h) on the same inputs."""
    from oracle import oracle
    sc, opts, _, _ = golden_case(name)
    pid, rng, _ = oracle.bound_n_split(sc, params=oracle.make_params(sc, bound_criterion=1, **opts))
    gpid, grng = golden_gpucrit(name)
    assert len(gpid) > 0
    assert subpatch_set(pid, rng) == subpatch_set(gpid, grng)
