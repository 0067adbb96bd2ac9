"""CPU checks of the oracle and of the C-ABI library (no GPU needed)."""
import math
import os
import re

import numpy as np
import pytest

from helpers import subpatch_set

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol(built):
    """libmpcore.so loads and exports each function declared in include/mp_core.h."""
    import ctypes
    from micropolis_gb300 import _lib
    header = open(os.path.join(ROOT, "include", "mp_core.h")).read()
    declared = set(re.findall(r"\b(mp_[a-z_]+)\s*\(", header))
    L = ctypes.CDLL(_lib.LIB_PATH)
    for name in declared:
        assert hasattr(L, name), name
    assert declared == {n for n, _, _ in _lib.SIGNATURES}


def test_oracle_matches_reference_pin_heightfield(built):
    from micropolis_gb300 import scenes
    from oracle import oracle
    if oracle.ref_pin() is None:
        pytest.skip("reference tree not compiled here")
    sc = scenes.heightfield_1024x768()
    pid, rng, _ = oracle.bound_n_split(sc)
    rpid, rrng = oracle.ref_bound_n_split(sc)
    assert np.array_equal(pid, rpid)
    assert np.array_equal(rng.view(np.uint32), rrng.view(np.uint32))


def test_oracle_matches_reference_pin_mixed(built):
    from micropolis_gb300 import scenes
    from oracle import oracle
    if oracle.ref_pin() is None:
        pytest.skip("reference tree not compiled here")
    sc = scenes.mixed4096_1920x1080(n=512, width=1024, height=576)
    for k in range(2):
        pid, rng, _ = oracle.bound_n_split(sc, k)
        rpid, rrng = oracle.ref_bound_n_split(sc, k)
        assert subpatch_set(pid, rng) == subpatch_set(rpid, rrng)
        assert np.array_equal(pid, rpid)


def test_oracle_sin_accuracy(built):
    from oracle import oracle
    xs = np.concatenate([np.linspace(-50, 50, 20001), np.random.default_rng(1).uniform(-700, 700, 5000)])
    errs = []
    for x in xs.astype(np.float32):
        ref = math.sin(float(x))
        got = oracle.sinf(float(x))
        errs.append(abs(got - ref))
    assert max(errs) < 4e-7


def test_oracle_scan():
    from oracle import oracle
    a = np.random.default_rng(3).integers(1, 9, 5000).astype(np.int32)
    assert np.array_equal(oracle.inclusive_scan(a), np.cumsum(a))


def test_dyadic_tiling_and_counts(built):
    """Emitted ranges of every patch are dyadic, pairwise disjoint and inside [0,1]^2."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.mixed4096_1920x1080(n=256, width=640, height=360)
    for k in range(2):
        pid, rng, nb = oracle.bound_n_split(sc, k)
        assert nb >= len(pid)
        w = rng[:, 2] - rng[:, 0]
        h = rng[:, 3] - rng[:, 1]
        for v in (w, h):
            m, e = np.frexp(v)
            assert np.all(m == 0.5)  # powers of two
        by = {}
        for p, r in zip(pid, rng):
            by.setdefault(int(p), []).append(r)
        for p, rs in by.items():
            rs = np.array(rs)
            assert np.all(rs[:, :2] >= 0) and np.all(rs[:, 2:] <= 1)
            assert (rs[:, 2] - rs[:, 0]).dot(rs[:, 3] - rs[:, 1]) <= 1.0
            # no two ranges overlap in area
            for i in range(len(rs)):
                ox = np.minimum(rs[i, 2], rs[i + 1:, 2]) - np.maximum(rs[i, 0], rs[i + 1:, 0])
                oy = np.minimum(rs[i, 3], rs[i + 1:, 3]) - np.maximum(rs[i, 1], rs[i + 1:, 1])
                assert not np.any((ox > 0) & (oy > 0))


def test_oracle_render_counts(built):
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.heightfield_1024x768()
    col, dep, st = oracle.render(sc)
    assert st["micropolygons"] == 64 * st["subpatches"]
    assert 0 < st["fragments"]
    assert np.count_nonzero(dep != 0x7FFFFFFF) > 0.1 * dep.size


def test_options_file_and_cli():
    from micropolis_gb300.options import load_options
    text = "// comment\nreyes_patch_size = 16\nbound_n_split_limit = 4\nclear_color = 0 0 0 1\n#hash:123\n"
    o = load_options(text, ["--max_split_depth=12", "--backface_culling=false"])
    assert o.reyes_patch_size == 16 and o.bound_n_split_limit == 4.0
    assert o.clear_color == (0.0, 0.0, 0.0, 1.0)
    assert o.max_split_depth == 12 and o.backface_culling is False


def test_gpu_criterion_oracle_properties(built):
    """The restated GPU criterion emits dyadic ranges that never overlap
    within a patch, differs from the CPU criterion, and drops ranges at
    depth >= max_split_depth - 1."""
    from micropolis_gb300 import scenes
    from oracle import oracle
    sc = scenes.mixed4096_1920x1080(n=128, width=512, height=512)
    for depth in (23, 6):
        p = oracle.make_params(sc, bound_criterion=1, max_split_depth=depth)
        pid, rng, nb = oracle.bound_n_split(sc, 0, params=p)
        assert len(pid) > 0
        w = rng[:, 2] - rng[:, 0]
        h = rng[:, 3] - rng[:, 1]
        assert np.all(np.frexp(w)[0] == 0.5) and np.all(np.frexp(h)[0] == 0.5)
        assert np.all(np.mod(rng[:, 0], w) == 0) and np.all(np.mod(rng[:, 1], h) == 0)
        # splits below the cull depth only: at most depth - 2 halvings
        assert np.all(-np.log2(w) - np.log2(h) <= depth - 2)
        for q in np.unique(pid)[:20]:
            a = rng[pid == q]
            for i in range(len(a)):
                for j in range(i + 1, len(a)):
                    ox = min(a[i, 2], a[j, 2]) - max(a[i, 0], a[j, 0])
                    oy = min(a[i, 3], a[j, 3]) - max(a[i, 1], a[j, 1])
                    assert ox <= 0 or oy <= 0
    cpu_pid, _, _ = oracle.bound_n_split(sc, 0, params=oracle.make_params(sc))
    gpu_pid, _, _ = oracle.bound_n_split(sc, 0, params=oracle.make_params(sc, bound_criterion=1))
    assert len(cpu_pid) != len(gpu_pid)
