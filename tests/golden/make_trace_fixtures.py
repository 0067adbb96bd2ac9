"""Writes trace_batched.txt, trace_plain.txt and stats_batched.txt: the
trace (mp_dump_trace, the reference's `name@queue:queued:submit:start:end:
id:deps` lines of src/CL/Device.cpp:275-289) and statistics (mp_dump_stats,
Statistics::dump_stats) of one frame of the 256-patch mixed scene at
640x448, rendered on the GPU with the batched path (stage events of its
graph) and the plain path (stage timing on).  tests/test_trace_tools_cpu.py
reads them with the reference's own tools/parse_trace.py and
tools/trace_summary.py.  Needs a GPU:

    python tests/golden/make_trace_fixtures.py [out_dir]
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def scene():
    from micropolis_gb300 import scenes
    return scenes.mixed4096_1920x1080(n=256, width=640, height=448)


def frame_texts(path):
    """(trace, stats) of the second frame of the scene on `path` (the first
    one sizes the buffers)."""
    from micropolis_gb300.renderer import render_scene, renderer_for
    sc = scene()
    r = renderer_for(sc, path)
    if path == "plain":
        r.set_stage_timing(True)
    render_scene(r, sc)
    render_scene(r, sc)
    out = r.dump_trace(), r.dump_stats()
    r.close()
    return out


def main(out_dir):
    os.makedirs(out_dir, exist_ok=True)
    for path in ("batched", "plain"):
        trace, stats = frame_texts(path)
        with open(os.path.join(out_dir, f"trace_{path}.txt"), "w") as f:
            f.write(trace)
        if path == "batched":
            with open(os.path.join(out_dir, "stats_batched.txt"), "w") as f:
                f.write(stats)
    print("trace fixtures written to", out_dir)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
