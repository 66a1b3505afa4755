"""CPU tests of bench.py's host-side helpers: argument defaults (one GPU, the
1080p frame), the --traversal option, and the DRAM traffic that each
workload's roofline reads from its committed ncu summary."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
sys.path.insert(0, str(ROOT))

import bench  # noqa: E402


def _args(argv):
    old = sys.argv
    sys.argv = ["bench.py"] + argv
    try:
        return bench.parse_args()
    finally:
        sys.argv = old


def test_defaults_are_one_gpu_on_the_frame():
    a = _args([])
    assert a.gpus == 1 and a.workload == "frame" and a.impl == "ours"
    assert (a.width, a.height) == (1920, 1080)
    assert a.warmup >= 3 and a.traversal is None
    s = _args(["--workload", "scene"])
    assert (s.width, s.height) == (1280, 720)


def test_traversal_option_is_a_config_tuple():
    a = _args(["--traversal", "256,0,24,1"])
    from rtgallery import abi

    cfg = abi.RtTraversalConfig(*(int(v) for v in a.traversal.split(",")))
    assert cfg.as_tuple() == (256, 0, 24, abi.RT_TRAVERSAL_PACKET_PRIMARY)


def test_profiled_traffic_of_each_frame_workload():
    for name in ("k_trace_full_1080p.md", "k_trace_default_scene_720p.md"):
        t = bench.profiled_traffic(name)
        assert t is not None and 1e7 < t < 1e10, (name, t)
    assert bench.profiled_traffic("no_such_profile.md") is None
