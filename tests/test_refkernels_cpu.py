"""The oracle's dice / shade / sample restatement against the reference's own
kernels (kernels/dice.cl, kernels/reyes.cl, kernels/framebuffer.cl), compiled
as C++ by oracle/build_ref.sh and run on the CPU with the launch geometry of
src/Reyes/RendererCL.cpp after the reference's CPU bound-and-split.

Both sides compute in FP32 with fused multiply-adds, but gcc contracts the
kernel source where it chooses and divides with IEEE `/`, while the oracle
fixes one contraction per expression and divides by a reciprocal (the
arithmetic the CUDA kernels use).  So the frames agree to rounding, not bit
for bit: pixel coverage exactly, depth keys within a few units of the 2^31
scale, colours within 1e-3 relative in all but a few pixels (quads whose
normal comes from nearly equal positions amplify the rounding).
"""
import numpy as np
import pytest

from helpers import golden_case

EMPTY = 0x7fffffff
CASES = [("heightfield_1024x768", 0), ("heightfield_1024x768", 1), ("mixed96_bezier_512", 0),
         ("mixed96_gregory_512", 0), ("mixed96_gregory_512", 1), ("mixed96_gregory_depth3_512", 1),
         ("heightfield_eye_plane_512x384", 0)]


def _ref_lib():
    from oracle import oracle
    L = oracle.ref_pin()
    if L is None or not hasattr(L, "refk_render"):
        pytest.skip("reference tree not compiled here")
    return oracle


@pytest.mark.parametrize("name,disp", CASES)
def test_oracle_frame_matches_reference_kernels(built, name, disp):
    oracle = _ref_lib()
    sc, _, _, _ = golden_case(name)
    p = oracle.make_params(sc, displacement=disp)
    rc, rd, rn = oracle.ref_render(sc, params=p)
    col, dep, st = oracle.render(sc, params=p)
    assert rn == st["subpatches"]
    cov_r, cov_o = rd != EMPTY, dep != EMPTY
    assert cov_r.sum() > 0
    assert np.array_equal(cov_r, cov_o)
    # clear colour where nothing was drawn
    assert np.array_equal(rc[~cov_r], col[~cov_o])
    dd = np.abs(rd.astype(np.int64) - dep.astype(np.int64))[cov_r]
    assert dd.max() <= 128, dd.max()
    rel = np.max(np.abs(rc - col), axis=1) / np.maximum(np.max(np.abs(rc), axis=1), 1e-30)
    rel = rel[cov_r]
    assert np.mean(rel > 1e-3) <= 5e-3, np.mean(rel > 1e-3)
    assert rel.max() <= 5e-2, rel.max()


def test_reference_kernels_see_planted_oracle_change(built):
    """The comparison catches a one-pixel shift of the dice grid: the oracle's
    subpixel precision lowered by one bit against the reference's."""
    oracle = _ref_lib()
    sc, _, _, _ = golden_case("mixed96_bezier_512")
    p = oracle.make_params(sc)
    rc, rd, _ = oracle.ref_render(sc, params=p)
    q = oracle.make_params(sc, subpixel_bits=p.subpixel_bits - 1)
    col, dep, _ = oracle.render(sc, params=q)
    assert not np.array_equal(rd != EMPTY, dep != EMPTY)


BOUND_CASES = [("heightfield_1024x768", {}), ("mixed96_bezier_512", {}), ("mixed96_gregory_512", {}),
               ("mixed96_gregory_depth3_512", {}), ("heightfield_eye_plane_512x384", {}),
               ("mixed96_bezier_512", {"bound_n_split_limit": 4.0, "cull_ribbon": 0.0}),
               ("mixed96_gregory_512", {"bound_n_split_limit": 16.0, "cull_ribbon": 8.0})]


@pytest.mark.parametrize("name,over", BOUND_CASES)
def test_gpu_criterion_matches_reference_bound(built, name, over):
    """The oracle's restatement of the reference's GPU bound criterion emits
    the same sub-patch set, bit for bit, as bound() of
    kernels/bound_n_split.h compiled as C++."""
    from helpers import subpatch_set
    oracle = _ref_lib()
    if not hasattr(oracle.ref_pin(), "refk_bound_n_split_gpu"):
        pytest.skip("reference tree not compiled here")
    sc, _, _, _ = golden_case(name)
    p = oracle.make_params(sc, bound_criterion=1, **over)
    pid, rng, _ = oracle.bound_n_split(sc, params=p)
    rpid, rrng = oracle.ref_bound_n_split_gpu(sc, params=p)
    assert len(rpid) > 0
    assert subpatch_set(pid, rng) == subpatch_set(rpid, rrng)


def test_gpu_criterion_pin_sees_planted_change(built):
    """A split limit 0.1 % lower in the oracle changes the set."""
    from helpers import subpatch_set
    oracle = _ref_lib()
    sc, _, _, _ = golden_case("heightfield_1024x768")
    p = oracle.make_params(sc, bound_criterion=1)
    rpid, rrng = oracle.ref_bound_n_split_gpu(sc, params=p)
    q = oracle.make_params(sc, bound_criterion=1, bound_n_split_limit=p.bound_n_split_limit * 0.999)
    pid, rng, _ = oracle.bound_n_split(sc, params=q)
    assert subpatch_set(pid, rng) != subpatch_set(rpid, rrng)
