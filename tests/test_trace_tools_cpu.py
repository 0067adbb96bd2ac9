"""The trace and statistics this core writes, read by the reference's own
tools: tools/parse_trace.py (its line pattern and TraceItem) and the Summary
of tools/trace_summary.py, whose nmap must know every command name (a name it
does not know raises KeyError).  The inputs are one frame of each path
recorded on the GPU by tests/golden/make_trace_fixtures.py; the reference's
tools are imported from its tree where that exists (MP_REFERENCE_DIR, or the
tree oracle/build_ref.sh compiled), else those checks are skipped."""
import io
import os
import sys

import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
PATHS = ["batched", "plain"]


def _text(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return f.read()


def _reference_tools():
    from oracle import oracle
    d = oracle.reference_dir()
    tools = os.path.join(d, "tools") if d else ""
    if not tools or not os.path.exists(os.path.join(tools, "trace_summary.py")):
        pytest.skip("the reference tree is not present here")
    pytest.importorskip("tabulate")
    if tools not in sys.path:
        sys.path.insert(0, tools)
    import parse_trace
    import trace_summary
    return parse_trace, trace_summary


@pytest.mark.parametrize("path", PATHS)
def test_trace_lines_parse(path):
    """Every line matches the reference's pattern; ids count up and each
    command depends on the one before it; times are ordered."""
    from oracle import oracle
    items = oracle.parse_trace(_text(f"trace_{path}.txt"))
    assert items
    assert [it[6] for it in items] == list(range(len(items)))
    assert all(it[7] == ([it[6] - 1] if it[6] else []) for it in items)
    assert all(it[5] >= it[4] >= 0 for it in items)
    assert all(b[4] >= a[5] for a, b in zip(items, items[1:]))


@pytest.mark.parametrize("path", PATHS)
def test_reference_summary_reads_trace(path, capsys):
    parse_trace, trace_summary = _reference_tools()
    items = parse_trace.parse(io.StringIO(_text(f"trace_{path}.txt")))
    assert len(items) == len(_text(f"trace_{path}.txt").splitlines())
    s = trace_summary.Summary(items)
    # every command lands in one of the reference's categories; the frame's
    # time is the sum of its commands plus idle gaps
    assert set(s.times) <= {"sample", "dice", "shade", "subdivision", "clear", "idle"}
    assert {"subdivision", "dice", "shade"} <= set(s.times)
    assert abs(sum(s.times.values()) - s.duration) < 1e-6 * max(1.0, s.duration)
    assert s.times["idle"] >= -1e-9
    s.print_duration()
    s.print_times()
    s.print_percentages()
    assert "total frame time" in capsys.readouterr().out


def test_stats_format():
    from oracle import oracle
    s = oracle.parse_stats(_text("stats_batched.txt"))
    assert s["patches_per_frame"] > 0 and s["pass_count"] == 1
    assert s["total_input_patches"] == 256
    assert s["opencl_mem"] == sum(v for k, v in s.items() if k.startswith("opencl_mem@"))


def test_reference_reads_trace_and_stats_files(capsys):
    """The reference's command-line entry (a trace file and a statistics
    file) on the batched frame's fixtures."""
    parse_trace, trace_summary = _reference_tools()
    s = trace_summary.parse_trace_file_and_create_summary(os.path.join(GOLDEN, "trace_batched.txt"),
                                                          os.path.join(GOLDEN, "stats_batched.txt"))
    from oracle import oracle
    ours = oracle.parse_stats(_text("stats_batched.txt"))
    # what the reference's pattern reads agrees with ours, and the frame's
    # counters are among it
    assert s.statistics and all(ours[k] == v for k, v in s.statistics.items())
    assert {"patches_per_frame", "processed_patches_per_frame", "pass_count"} <= set(s.statistics)
    s.print()
    assert "patches_per_frame" in capsys.readouterr().out
