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


def test_defaults_are_one_gpu_on_the_headline_batch():
    a = _args([])
    assert a.gpus == 1 and a.workload == "batch" and a.impl == "ours"
    assert a.batch_scenes == 64 and a.serve_seconds == 120.0
    assert a.warmup >= 3 and a.traversal is None
    f = _args(["--workload", "frame"])
    assert (f.width, f.height) == (1920, 1080)
    s = _args(["--workload", "scene"])
    assert (s.width, s.height) == (1280, 720)


def test_headline_metric_is_the_baseline_metric():
    import json

    base = json.loads((ROOT / "BASELINE.json").read_text())
    assert bench.BATCH_METRIC == base["metric"]


def test_camera_ray_sample_points_into_the_view():
    import numpy as np

    from rtgallery import scenes

    sc = scenes.scene_batch_member(0)
    r = bench.camera_ray_sample(sc, 8)
    assert len(r) == ((sc.height + 7) // 8) * ((sc.width + 7) // 8)
    d = r["direction"]
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-5)
    # the centre ray looks at the scene's target (0, 0.5, 0)
    vi = np.array(sc.uniforms.view_inverse, np.float32).reshape(4, 4).T
    eye = vi[:3, 3]
    to_target = np.array([0.0, 0.5, 0.0]) - eye
    to_target /= np.linalg.norm(to_target)
    assert float((d @ to_target).max()) > 0.999


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
