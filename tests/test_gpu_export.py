"""Headless framebuffer export and the reference-format trace and statistics
writers, through the C ABI: the displayed image against the oracle's
restatement of the reference's tex_draw shader, trace lines parsed with the
reference tool's pattern, statistics in Statistics::dump_stats format."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# command names the reference's tools/trace_summary.py maps
TRACE_NAMES = {"sample", "dice", "shade", "bound & split", "clear framebuffer", "accumulate"}


def _scene():
    from micropolis_gb300 import scenes
    return scenes.mixed4096_1920x1080(n=256, width=640, height=448)


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_display_image_matches_oracle(built, cuda, path, tmp_path):
    from micropolis_gb300.renderer import read_ppm, render_scene, renderer_for
    from oracle import oracle
    sc = _scene()
    r = renderer_for(sc, path)
    render_scene(r, sc)
    col, _ = r.read_framebuffer()
    img = r.read_image()
    want = oracle.display_image(col, sc.width, sc.height)
    diff = np.abs(img.astype(int) - want.astype(int))
    assert diff.max() <= 1 and np.count_nonzero(diff) <= 1e-3 * diff.size
    # the background is the gamma-corrected clear colour, not black
    assert img.shape == (sc.height, sc.width, 3) and len(np.unique(img.reshape(-1, 3), axis=0)) > 100
    p = tmp_path / "f.ppm"
    r.save_ppm(str(p))
    assert np.array_equal(read_ppm(str(p)), img)
    r.save_pfm(str(tmp_path / "f.pfm"))
    r.close()


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_trace_and_stats_formats(built, cuda, path):
    from micropolis_gb300.renderer import render_scene, renderer_for
    from oracle import oracle
    sc = _scene()
    r = renderer_for(sc, path)
    r.set_stage_timing(True)
    render_scene(r, sc)
    st = r.stats()
    items = oracle.parse_trace(r.dump_trace())
    assert items and {it[0] for it in items} <= TRACE_NAMES
    assert [it[6] for it in items] == list(range(len(items)))
    assert all(it[7] == ([it[6] - 1] if it[6] else []) for it in items)
    assert all(it[5] >= it[4] >= 0 for it in items)
    total_ms = sum(it[5] - it[4] for it in items) / 1e6
    stage_ms = sum(v for k, v in st["stage_ms"].items() if k != "host_sync")
    assert abs(total_ms - stage_ms) <= 1e-3 * len(items) + 1e-3
    if path == "plain":
        assert sum(1 for it in items if it[0] == "bound & split") == st["passes"]
    s = oracle.parse_stats(r.dump_stats())
    assert s["patches_per_frame"] == st["subpatches"]
    assert s["processed_patches_per_frame"] == st["bounds"]
    assert s["pass_count"] == st["passes"]
    assert s["total_input_patches"] == sc.n_patches
    assert s["opencl_mem"] == sum(v for k, v in s.items() if k.startswith("opencl_mem@"))
    assert s["max_patches"] > 0 and s["opengl_mem"] == 0
    r.set_stage_timing(False)
    render_scene(r, sc)
    if path == "batched":
        # the frame's graph records its stage events: same lines without stage timing
        items = oracle.parse_trace(r.dump_trace())
        assert [it[0] for it in items] == ["clear framebuffer", "bound & split", "accumulate", "dice", "sample",
                                           "shade"]
        assert all(it[5] >= it[4] >= 0 for it in items)
        assert abs(sum(r.stats()["stage_ms"].values()) - sum(it[5] - it[4] for it in items) / 1e6) < 1e-3
    else:
        from micropolis_gb300 import _lib
        with pytest.raises(_lib.MpError) as e:
            r.dump_trace()
        assert e.value.status == _lib.MP_ERR_STATE
    r.close()


@pytest.mark.parametrize("path", ["batched", "plain"])
def test_trace_matches_committed_fixture(built, cuda, path):
    """The trace fixture that tests/test_trace_tools_cpu.py feeds to the
    reference's own tools still has the form this library writes: the same
    commands in the same order, ids and dependencies for the same frame."""
    import os
    import sys
    from oracle import oracle
    here = os.path.dirname(os.path.abspath(__file__))
    sys.path.insert(0, os.path.join(here, "golden"))
    import make_trace_fixtures
    trace, _ = make_trace_fixtures.frame_texts(path)
    live = oracle.parse_trace(trace)
    with open(os.path.join(here, "golden", f"trace_{path}.txt")) as f:
        fixture = oracle.parse_trace(f.read())
    assert [(it[0], it[1], it[6], it[7]) for it in live] == [(it[0], it[1], it[6], it[7]) for it in fixture]
    assert all(b[4] >= a[5] for a, b in zip(live, live[1:]))


def test_async_read_back_equals_sync(built, cuda):
    """mp_read_framebuffer_async: frames read back while the next frame
    renders equal the synchronous read-back of each frame, bit for bit, with
    two alternating host buffers and a different camera every frame."""
    torch = cuda
    from micropolis_gb300 import scenes
    from micropolis_gb300.renderer import render_scene, renderer_for
    base = _scene()
    r = renderer_for(base, "batched")
    n = base.width * base.height
    cols = [torch.empty((n, 4), dtype=torch.float32).pin_memory().numpy() for _ in range(2)]
    deps = [torch.empty((n,), dtype=torch.int32).pin_memory().numpy() for _ in range(2)]
    want = []
    for k in range(4):
        sc = scenes.mixed4096_1920x1080(n=256, width=640, height=448, distance=11.0 + k)
        render_scene(r, sc)
        c, d = r.read_framebuffer()
        want.append((c.copy(), d.copy()))
        if k >= 2:
            # the buffers of frame k - 2 are reused: its read-back must have landed
            assert np.array_equal(deps[k % 2], want[k - 2][1])
        r.read_framebuffer_async(0, cols[k % 2].ctypes.data, deps[k % 2].ctypes.data)
        if k % 2 == 1:
            r.wait_read_framebuffer()
            for j in (k - 1, k):
                assert np.array_equal(deps[j % 2], want[j][1])
                assert np.array_equal(cols[j % 2].view(np.uint32), want[j][0].view(np.uint32))
    r.close()
