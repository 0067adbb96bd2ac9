"""The oracle's dice / shade / sample restatement against the reference's own
kernels (kernels/dice.cl, kernels/reyes.cl, kernels/framebuffer.cl), compiled
as C++ by oracle/build_ref.sh and run on the CPU with the launch geometry of
src/Reyes/RendererCL.cpp after the reference's CPU bound-and-split.

The reference's -cl-fast-relaxed-math build leaves the rounding of
contractions, divisions, float-to-int conversions and native_sin open; the
compiled kernels take the oracle's choices for the last three (the shim) and
gcc's own contraction, which the oracle's R1 table follows.  So the diced
grids agree bit for bit, and the frames meet the framebuffer bar: depth
and colour within 1e-5 relative per pixel except in fewer than 1e-4 of the
frame's pixels (tie pixels, where the two sides let a different one
of two equally deep micropolygons win).
"""
import numpy as np
import pytest

from helpers import golden_case

EMPTY = 0x7fffffff
CASES = [("heightfield_1024x768", 0), ("heightfield_1024x768", 1), ("mixed96_bezier_512", 0),
         ("mixed96_gregory_512", 0), ("mixed96_gregory_512", 1), ("mixed96_gregory_depth3_512", 1),
         ("heightfield_eye_plane_512x384", 0)]
# 16x16 dicing (four 8x8 blocks per sub-patch), no backface culling, 4 subpixel bits
FRAME_CASES = [(n, d, {}) for n, d in CASES] + [
    ("mixed96_bezier_512", 0, {"reyes_patch_size": 16}),
    ("heightfield_eye_plane_512x384", 1, {"reyes_patch_size": 16}),
    ("mixed96_gregory_512", 0, {"backface_culling": 0, "reyes_patch_size": 16}),
    ("heightfield_1024x768", 0, {"subpixel_bits": 4})]


def _ref_lib():
    from oracle import oracle
    L = oracle.ref_pin()
    if L is None or not hasattr(L, "refk_render"):
        pytest.skip("reference tree not compiled here")
    return oracle


@pytest.mark.parametrize("name,disp,over", FRAME_CASES)
def test_oracle_frame_matches_reference_kernels(built, name, disp, over):
    oracle = _ref_lib()
    sc, _, _, _ = golden_case(name)
    p = oracle.make_params(sc, displacement=disp, **over)
    rc, rd, rn = oracle.ref_render(sc, params=p)
    col, dep, st = oracle.render(sc, params=p)
    assert rn == st["subpatches"]
    cov_r, cov_o = rd != EMPTY, dep != EMPTY
    assert cov_r.sum() > 0
    assert np.array_equal(cov_r, cov_o)
    rel = np.max(np.abs(rc - col), axis=1) / np.maximum(np.max(np.abs(rc), axis=1), 1e-30)
    bad = (rd != dep) | (rel > 1e-5)
    assert bad.sum() <= 1e-4 * rd.size, (int(bad.sum()), rd.size)


@pytest.mark.parametrize("name,disp", CASES)
def test_oracle_grids_match_reference_dice_shade(built, name, disp):
    """Position, pixel and depth grids bit for bit; quad colours within 1e-5
    relative (the largest seen is 2e-7: the reference's shading goes through
    the shim's vector operators, whose contraction gcc picks per call site)."""
    oracle = _ref_lib()
    if not hasattr(oracle.ref_pin(), "refk_dice_shade"):
        pytest.skip("reference tree not compiled here")
    sc, _, pid, rng = golden_case(name)
    p = oracle.make_params(sc, displacement=disp)
    sel = np.linspace(0, len(pid) - 1, min(len(pid), 160)).astype(int)
    pid, rng = pid[sel], rng[sel]
    rpos, rpxl, rdep, rcol, _ = oracle.ref_dice_shade(sc, 0, pid, rng, params=p)
    written = 0
    for k in range(len(pid)):
        pos, pxl, dep = oracle.dice(sc, 0, pid[k], rng[k], params=p)
        assert np.array_equal(rpos[k].view(np.uint32), pos.view(np.uint32)), k
        assert np.array_equal(rpxl[k], pxl), k
        assert np.array_equal(rdep[k].view(np.uint32), dep.view(np.uint32)), k
        c = oracle.shade_quads(sc, 0, pid[k], rng[k], params=p)
        w = ~np.isnan(rcol[k][:, 0])
        written += int(w.sum())
        rel = np.max(np.abs(rcol[k][w] - c[w]), axis=1) / np.maximum(np.max(np.abs(rcol[k][w]), axis=1), 1e-30)
        assert rel.size == 0 or rel.max() <= 1e-5, (k, rel.max())
    assert written > 0


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
