"""Known answer: a bicubic Bezier patch rewritten as a 20-point Gregory patch
with the index map of the reference's tools/bez2mscene_greg.py:111 (its
interior point k stands for both face points of its corner) is the same
surface.  In exact arithmetic each face blend (u*A + v*A) / (u + v) is A; in
FP32 it is A within a few rounding steps, so the diced positions agree to
about 1e-7 of the patch size, and where a blend is 0/0 (the corners, whose
blend weight is zero) the NaN is zeroed and changes nothing.

Checked for the oracle's dicer (kernels/dice.cl + kernels/utility.h
restated) over whole patches and interior sub-patch ranges, against FP64
Bernstein evaluation of the Bezier patch, and -- where the reference tree
was compiled -- for the reference's own CPU evaluators eval_patch and
eval_gregory_patch (src/base/Patch.cpp:114-128,186-210)."""
import numpy as np
import pytest

from micropolis_gb300 import scenes

# positions of the two forms may differ by a few FP32 roundings of the
# patch's coordinates (relative to its largest eye-space coordinate)
REL_TOL = 1e-6

RANGES = np.array([[0.0, 0.0, 1.0, 1.0], [0.25, 0.25, 0.5, 0.5], [0.5, 0.0, 0.75, 0.125],
                   [0.125, 0.625, 0.1875, 0.6875]], np.float32)


def bezier_and_gregory_scene(n=16):
    """One draw of n Bezier patches (heightfield over [-1,1]^2) and one draw
    of the same patches converted to Gregory form, same camera."""
    hf = scenes.heightfield_1024x768()
    d = hf.draws[0]
    bez = d.mesh.cp[:n]
    greg = bez[:, scenes.BEZIER_TO_GREGORY, :]
    draws = [scenes.Draw(scenes.Mesh(scenes.BEZIER, bez), d.mv, d.color),
             scenes.Draw(scenes.Mesh(scenes.GREGORY, np.ascontiguousarray(greg)), d.mv, d.color)]
    return scenes.Scene("bez_greg", hf.width, hf.height, draws, fovy=hf.fovy, near=hf.near,
                        options=dict(hf.options))


def test_gregory_form_dices_to_the_bezier_surface(built):
    from oracle import oracle
    sc = bezier_and_gregory_scene()
    for pid in range(sc.draws[0].mesh.n_patches):
        for rng in RANGES:
            pb, xb, db = oracle.dice(sc, 0, pid, rng)
            pg, xg, dg = oracle.dice(sc, 1, pid, rng)
            assert np.isfinite(pg).all()
            scale = np.abs(pb[:, :3]).max()
            assert np.abs(pg[:, :3] - pb[:, :3]).max() <= REL_TOL * scale, (pid, rng)
            # both within FP64 evaluation of the Bezier patch
            ref = oracle.dice_fp64(sc, 0, pid, rng)
            assert np.abs(pg[:, :3] - ref).max() <= 2e-6 * scale
            # fixed-point pixels at most one unit apart (a coordinate on a
            # rounding boundary), most of them identical
            assert np.abs(xg - xb).max() <= 1
            assert np.mean(np.all(xg == xb, axis=1)) > 0.9


def test_gregory_corner_blends_are_zeroed(built):
    """At the patch corners the face blends are 0/0; the corner vertices are
    still the Bezier corners, exactly."""
    from oracle import oracle
    sc = bezier_and_gregory_scene(n=4)
    G = 9
    corners = [0, G - 1, G * (G - 1), G * G - 1]
    for pid in range(4):
        pb, _, _ = oracle.dice(sc, 0, pid, RANGES[0])
        pg, _, _ = oracle.dice(sc, 1, pid, RANGES[0])
        assert np.array_equal(pb[corners], pg[corners])


def test_reference_cpu_evaluators_agree():
    """The reference's own eval_patch and eval_gregory_patch (compiled from
    its tree by oracle/build_ref.sh) on the two forms of random patches."""
    from oracle import oracle
    L = oracle.ref_pin()
    if L is None:
        pytest.skip("the reference tree was not compiled here (MP_REFERENCE_DIR)")
    rng = np.random.default_rng(9)
    f32p = oracle.f32p
    for _ in range(32):
        bez = rng.normal(size=(16, 3)).astype(np.float32)
        greg = np.ascontiguousarray(bez[scenes.BEZIER_TO_GREGORY])
        for u, v in rng.uniform(0.02, 0.98, size=(16, 2)).astype(np.float32):
            a = np.zeros(3, np.float32)
            b = np.zeros(3, np.float32)
            L.refpin_eval_patch(bez.ctypes.data_as(f32p), u, v, a.ctypes.data_as(f32p))
            L.refpin_eval_gregory(greg.ctypes.data_as(f32p), u, v, b.ctypes.data_as(f32p))
            assert np.abs(a - b).max() <= REL_TOL * np.abs(bez).max(), (u, v, a, b)
