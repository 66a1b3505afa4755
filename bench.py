"""Benchmark of the ray-tracing hot path on one GB300 (or N replicas).

Default workload (--workload batch; one step = 64 scenes): 64 independent
procedural scenes (unique triangles log-uniform in [10k, 2M], resolutions
from 128^2 to 1920x1080, primary + 2 blue-noise soft shadows + 1 reflection
bounce).  `value` is the quantised + batched path: BLASes with 8-bit
quantised child boxes, all 64 scenes in one batched launch sequence replayed
from a CUDA graph, launch shape and node width chosen by rt_ctx_autotune.
Beside it stands the plain FP32 path (FP32 child boxes, one rt_cmd_trace_rays
per scene, the default launch shape) and their ratio; every image of the two
paths and the hits of a camera-ray sample are compared bit for bit; the
radiance error against the FP32 and FP64 oracles is reported per image; then
the serving stream (Poisson arrivals over 32 resident scenes) gives its
p50 / p99 / p99.9 latencies.

Metric: Mrays/s = traversals (primary + shadow + reflection, each traceRay
counted once) / time, time from CUDA events on the launching stream with the
L2 flushed (a 256 MiB write) before every step, outside the events.  `e2e`
runs the same graph through the C ABI with host buffers: the uniforms come
in from pinned host memory and every image is written into pinned host
memory, inside the timed span.

Other workloads: --workload frame (the full plain feature set at 1920x1080:
256 instances, TLAS rebuild per frame, two frames in flight), scene (the
reference's default scene from GLB / PNG files, 1280x720, TLAS refit per
frame), precision (10,485,760 triangles, 4M random rays, quantised vs FP32
nodes) and serve (the request stream alone, batched and plain in full).

--impl reference runs the CPU oracle (the restatement of the reference's
shader logic; the reference itself needs a Vulkan ray-tracing driver, which
does not exist on this machine) over bounded samples of the same work.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
import __graft_entry__  # noqa: E402

__graft_entry__.load_package()
from rtgallery import abi, scenes  # noqa: E402

FRAMES = 60
WIDTH, HEIGHT = 1920, 1080
WORKLOAD = ("full plain feature set, 1920x1080, 256 instances (torus 64x32 / displaced UV sphere 128x64 / "
            "alpha-clipped 200x1 fence), 10% mirrors, per-frame SO(3)+translation transforms over 60 frames "
            "with a TLAS rebuild each frame, 4 blue-noise soft shadows (2 deg), 1 reflection bounce")
L2_FLUSH_BYTES = 256 << 20
NODE_BYTES, TRI_BYTES, RAY_BYTES, HIT_BYTES, INST_BYTES = 256, 48, 32, 16, 128
QNODE_BYTES, RAY_HIT_BYTES = 96, 32
PRECISION_RAYS = 4 << 20
E2E_CHUNK = 1 << 20  # rays per chunk of the host-buffer query
PRECISION_WORKLOAD = ("precision: displaced icosphere (level 9, every triangle bisected on its longest edge: "
                      "10,485,760 triangles, radius 10, 0.5 fbm displacement), 4,194,304 random rays per step "
                      "(origins U[-15,15]^3, directions uniform on S^2, tmin 0, tmax inf), closest hit")


def parse_args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--width", type=int, default=None, help="frame: 1920, scene: 1280")
    p.add_argument("--height", type=int, default=None, help="frame: 1080, scene: 720")
    p.add_argument("--workload", default="batch", choices=["batch", "frame", "scene", "precision", "serve"],
                   help="batch (default): 64 scenes, the quantised + batched path against the plain FP32 path, "
                        "then the serving stream's latency percentiles; frame: the full 1080p frame; scene: the "
                        "reference's default scene from GLB / PNG files at 1280x720 with a TLAS refit per frame; "
                        "precision: 10,485,760-triangle icosphere, 4M random rays, quantised vs FP32 nodes; "
                        "serve: the Poisson request stream over 32 resident scenes alone")
    p.add_argument("--traversal", default=None, metavar="B,D,W,P",
                   help="batch / frame / scene: set this RtTraversalConfig (block_size, shared_stack_depth, "
                        "leaf_wait, packet_lists) instead of running rt_ctx_autotune on the workload")
    p.add_argument("--batch-scenes", type=int, default=64, help=argparse.SUPPRESS)
    p.add_argument("--serve-seconds", type=float, default=120.0,
                   help="batch / serve: length of the request stream (0: batch skips the stream)")
    p.add_argument("--serve-plain-seconds", type=float, default=30.0,
                   help="batch: the plain per-request server replays the stream's first this many seconds")
    p.add_argument("--serve-rate", type=float, default=400.0, help=argparse.SUPPRESS)
    p.add_argument("--serve-scenes", type=int, default=32, help=argparse.SUPPRESS)
    p.add_argument("--serve-budget-gb", type=float, default=150.0, help=argparse.SUPPRESS)
    p.add_argument("--precision-level", type=int, default=9, help=argparse.SUPPRESS)
    p.add_argument("--precision-rays", type=int, default=PRECISION_RAYS, help=argparse.SUPPRESS)
    args = p.parse_args()
    dw, dh = (1280, 720) if args.workload == "scene" else (WIDTH, HEIGHT)
    args.width = args.width or dw
    args.height = args.height or dh
    return args


class FullSceneFrames:
    """The default workload: the full plain feature set (module docstring)."""

    key = "frame"
    description = WORKLOAD
    path = "plain FP32 8-wide BVH"
    depth, shadows, refit = 2, 4, False
    profile = "k_trace_full_1080p.md"
    data = "synthetic (procedural scenes from seeds)"

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self.models = scenes.full_scene_models()

    def scene(self, k: int):
        return scenes.scene_full(k % FRAMES, self.width, self.height, models=self.models)

    def instances(self, k: int) -> np.ndarray:
        return scenes.full_scene_instances(k % FRAMES)

    def uniforms(self, k: int):
        return self.scene(k).uniforms

    def loop_note(self) -> str:
        return "2 frames in flight (own instance buffer, TLAS, uniforms, image, stream)"


class DefaultSceneFrames:
    """The reference's default scene (src/scene.rs:35-204) assembled from GLB /
    PNG files that librtcore decodes (the package's stand-in files of the
    reference's kinds and sizes), rendered as the reference's loop renders
    it: the figure turns 0.05 rad per frame, the frame's instance records are
    written and its TLAS refitted in place, two frames in flight."""

    key = "scene"
    description = ("the reference's default scene from GLB / PNG files decoded by librtcore (textured plane x10, "
                   "two linked tori, a 45,448-triangle textured figure turning 0.05 rad per frame, portal plane, "
                   "alpha-masked fence, 100 small tori half of them mirrors), 3 bounce iterations, 2 blue-noise "
                   "soft shadows (radius 0.05), TLAS refitted in place every frame")
    path = "plain FP32 8-wide BVH, TLAS refit"
    depth, shadows, refit = 3, 2, True
    profile = "k_trace_default_scene_720p.md"
    data = "synthetic stand-in asset files (GLB / PNG written from seeds), decoded by librtcore"

    def __init__(self, width: int, height: int):
        from rtgallery import assets

        self.assets = assets
        self.width, self.height = width, height
        self.sc0 = assets.default_scene(assets.standin_assets(), width, height, frame=0)

    def scene(self, k: int):
        import copy

        sc = copy.copy(self.sc0)
        sc.instances = self.instances(k)
        sc.uniforms = self.uniforms(k)
        return sc

    def instances(self, k: int) -> np.ndarray:
        return self.assets.default_scene_instances(0, k % FRAMES)

    def uniforms(self, k: int):
        return self.assets.default_scene_uniforms(self.width, self.height, k % FRAMES + 1)

    def loop_note(self) -> str:
        return "2 frames in flight (own instance buffer, TLAS refitted in place, uniforms, image, stream)"


def frame_workload(args):
    cls = DefaultSceneFrames if args.workload == "scene" else FullSceneFrames
    return cls(args.width, args.height)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def reduce_over_ranks(dist, total_ms: float, rays: float, device: str = "cuda") -> tuple[float, float]:
    """Whole-job numbers of N replicas: the slowest rank's time and the sum of
    every rank's rays (no data is exchanged otherwise).  `dist` None = one rank."""
    if dist is None:
        return total_ms, rays
    import torch

    t = torch.tensor([total_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    r = torch.tensor([rays], dtype=torch.float64, device=device)
    dist.all_reduce(r, op=dist.ReduceOp.SUM)
    return float(t.item()), float(r.item())


def profiled_figures(name: str) -> dict:
    """Figures of the committed ncu summary profiles/<name>: the lines
    `dram_bytes_per_launch: N` (DRAM read + write bytes of one launch of the
    kernel, used as roofline.traffic), `dram_frac: F` (DRAM throughput as a
    fraction of peak) and `l2_pct: P` (L2 throughput, % of peak)."""
    p = ROOT / "profiles" / name
    out = {}
    if not p.exists():
        return out
    for line in p.read_text().splitlines():
        key, _, rest = line.strip().partition(":")
        if key in ("dram_bytes_per_launch", "dram_frac", "l2_pct") and rest.strip():
            try:
                out[key] = float(rest.strip().split()[0])
            except ValueError:
                pass
    return out


def profiled_traffic(name: str = "k_trace_full_1080p.md"):
    """DRAM bytes per traversal launch from the committed ncu summary of this
    workload (profiles/<name>, line `dram_bytes_per_launch: N`)."""
    return profiled_figures(name).get("dram_bytes_per_launch")


_T0 = time.perf_counter()


def note(msg: str) -> None:
    """Progress on stderr (the JSON line alone goes to stdout)."""
    print(f"[bench {time.perf_counter() - _T0:7.1f} s] {msg}", file=sys.stderr, flush=True)


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.file.flush()
        rows = []
        with open(self.file.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(wl, budget_s: float = 12.0) -> dict:
    """The oracle (FP32, all host threads) rendering bands of the workload's
    frames until about `budget_s` seconds of CPU work."""
    from oracle.oracle import OracleScene, default_threads

    threads = default_threads()
    height = wl.height
    rays = 0
    t_total = 0.0
    frames_done = 0
    band = max(8, height // 8)
    o = None
    for k in range(FRAMES * 100):   # the 60 frames again and again until the budget is spent
        sc = wl.scene(k)
        if o is None:
            o = OracleScene(sc)
        else:
            o.set_instances(sc.instances)
        y0 = (k * band) % max(1, height - band)
        t = time.perf_counter()
        _, _, st = o.render(uniforms=sc.uniforms, rows=(y0, y0 + band), threads=threads)
        t_total += time.perf_counter() - t
        rays += st["traversals"]
        frames_done += 1
        if t_total >= budget_s:
            break
    return {"value": rays / t_total / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{frames_done} frames x {band} of {height} rows ({rays} traversals, {t_total:.1f} s)"}


def bench_reference(args):
    """The reference arm: the CPU restatement of the reference's path (the
    reference's own renderer needs a Vulkan ray-tracing driver)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import OracleScene, default_threads

    threads = default_threads()
    wl = frame_workload(args)
    band = max(8, args.height // 16)
    o = None
    times, rays = [], 0
    for k in range(args.warmup + args.steps):
        sc = wl.scene(k)
        if o is None:
            o = OracleScene(sc)
        t = time.perf_counter()
        o.set_instances(sc.instances)   # TLAS rebuild, as the GPU step does
        y0 = (k * band) % max(1, args.height - band)
        _, _, st = o.render(uniforms=sc.uniforms, rows=(y0, y0 + band), threads=threads)
        dt = time.perf_counter() - t
        if k >= args.warmup:
            times.append(dt)
            rays += st["traversals"]
    total = sum(times)
    value = rays / total / 1e6
    line = {
        "impl": "reference", "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": wl.description, "sample": f"{band}-row band of each frame", "width": args.width,
                   "height": args.height},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{band} of {args.height} rows per frame, {args.steps} frames"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def bench_ours(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from rtgallery import host

    dev = host.Device()
    lib = dev.lib
    W, H = args.width, args.height
    wl = frame_workload(args)
    DEPTH, SHADOWS = wl.depth, wl.shadows
    sc0 = wl.scene(0)
    t0 = time.perf_counter()
    gs = host.GpuScene(dev, sc0)
    torch.cuda.synchronize()
    blas_build_ms = 1e3 * (time.perf_counter() - t0)
    n_inst = gs.num_instances
    frames_host = [gs.patch_instances(wl.instances(k)) for k in range(FRAMES)]
    frames_dev = [host.Device.upload(f) for f in frames_host]
    uniforms = [wl.uniforms(k) for k in range(FRAMES)]
    uni_dev = [host.Device.upload(np.frombuffer(bytes(u), np.uint8)) for u in uniforms]
    # the reference's frame loop: two frames in flight, each with its own instance buffer, TLAS,
    # uniforms, image and stream; every frame rebuilds (or refits) its TLAS from that frame's
    # instance records
    loop = host.FrameLoop(dev, gs, W, H, frames_in_flight=2)
    flushes = [torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda") for _ in range(2)]
    stream = torch.cuda.current_stream()

    def frame(k: int, **kw):
        # the L2 flush (a 256 MiB write) runs on the frame's stream before its work
        return loop.record(k, DEPTH, SHADOWS, uniforms_dev=uni_dev[k % FRAMES], refit=wl.refit,
                           before=lambda st: flushes[k & 1].fill_(k & 0xFF), **kw)

    def read_timings() -> dict:
        tt = abi.RtTraceTimings()
        dev.check(lib.rt_ctx_read_trace_timings(dev.ctx, C.byref(tt)))
        return tt.as_dict()

    loop.begin()
    for k in range(args.warmup):
        frame(k, instances=frames_dev[k % FRAMES])
    loop.end()
    torch.cuda.synchronize()

    # ---- the autotuner picks the traversal configuration on one frame of this workload (a batch of
    # one: the first slot's TLAS and frame 0's uniforms), untimed; the loop then runs with it ----
    if args.traversal:
        tuned = abi.RtTraversalConfig(*(int(v) for v in args.traversal.split(",")))
        dev.check(lib.rt_ctx_set_traversal_config(dev.ctx, C.byref(tuned)))
        tune_note = {"chosen_by": "--traversal"}
    else:
        t_tune = time.perf_counter()
        tune_item = host.batch_scene(loop.slots[0], DEPTH, SHADOWS, uniforms_address=uni_dev[0].data_ptr())
        tune_arr = (abi.RtBatchScene * 1)(tune_item)
        report = abi.RtAutotuneReport()
        dev.check(lib.rt_ctx_autotune(dev.ctx, tune_arr, 1, None, 3, host.Device.stream_handle(stream),
                                      C.byref(report)))
        best = report.configs[report.best].as_tuple()
        default_cfg = (128, 0, 20, 0)
        tune_note = {"chosen_by": f"rt_ctx_autotune on frame 0 ({report.count} configs, "
                                  f"{time.perf_counter() - t_tune:.1f} s, untimed), then 10 untimed frames "
                                  "of this loop for its pick and its launch shape with packet_lists 0 / 1 / 5",
                     "tuned_ms": report.median_ms[report.best],
                     "default_config_ms": [report.median_ms[i] for i in range(report.count)
                                           if report.configs[i].as_tuple() == default_cfg][0]}
        # the tuner times one warm frame; the loop rebuilds / refits and flushes L2 every frame, so
        # the pick is confirmed on 10 frames of the loop itself
        cands = list(dict.fromkeys([best] + [best[:3] + (pl,) for pl in
                                             (0, abi.RT_TRAVERSAL_PACKET_PRIMARY,
                                              abi.RT_TRAVERSAL_PACKET_PRIMARY | abi.RT_TRAVERSAL_PACKET_LANE_BOUNCES)]))
        loop_ms = {}
        for cfg in cands:
            dev.check(lib.rt_ctx_set_traversal_config(dev.ctx, C.byref(abi.RtTraversalConfig(*cfg))))
            for rep in range(2):  # the first pass warms the configuration's kernels
                torch.cuda.synchronize()
                ea, eb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                ea.record(stream)
                loop.begin()
                for k in range(10):
                    frame(k, instances=frames_dev[k % FRAMES])
                loop.end()
                eb.record(stream)
                torch.cuda.synchronize()
            loop_ms[cfg] = ea.elapsed_time(eb) / 10
        pick = min(loop_ms, key=loop_ms.get)
        tuned = abi.RtTraversalConfig(*pick)
        dev.check(lib.rt_ctx_set_traversal_config(dev.ctx, C.byref(tuned)))
        tune_note["loop_ms_per_frame"] = {",".join(map(str, k)): v for k, v in loop_ms.items()}
    loop.begin()
    for k in range(args.warmup):
        frame(k, instances=frames_dev[k % FRAMES])
    loop.end()
    torch.cuda.synchronize()
    dev.read_stats(reset=True)

    # ---- device-resident timing (value): one span over all frames, both streams ----
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.rt_kernel_launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e_begin, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e_begin.record(stream)
    loop.begin()
    for k in range(args.steps):
        frame(k, instances=frames_dev[k % FRAMES])
    loop.end()
    e_end.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = lib.rt_kernel_launch_count() - launches0
    clk = clocks.stop()
    total_ms = e_begin.elapsed_time(e_end)
    stats = dev.read_stats(reset=True)
    rays_local = stats["traversals"]

    # ---- per-kernel split of serial frames (CUDA events after each kernel; outside the value span) ----
    kernel_times, serial_ms = [], []
    for k in range(min(args.steps, 10)):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        flushes[0].fill_(k & 0xFF)
        torch.cuda.synchronize()
        e0.record(loop.streams[0])
        loop.record(2 * k, DEPTH, SHADOWS, instances=frames_dev[k % FRAMES], uniforms_dev=uni_dev[k % FRAMES],
                    flags=abi.RT_TRACE_FLAG_KERNEL_TIMINGS, refit=wl.refit)
        e1.record(loop.streams[0])
        torch.cuda.synchronize()
        serial_ms.append(e0.elapsed_time(e1))
        kernel_times.append(read_timings())
    trace_ms = [kt["total_ms"] for kt in kernel_times]
    traversal_ms = [kt["trace_ms"] for kt in kernel_times]
    traversal_launches = kernel_times[0]["trace_launches"]
    dev.read_stats(reset=True)
    total_ms, rays_all = reduce_over_ranks(dist, total_ms, float(rays_local))
    value = rays_all / (total_ms / 1e3) / 1e6

    # ---- end-to-end through the C ABI with host buffers (e2e): each frame's instance records come
    # from pinned host memory and its RGBA8 image goes back to pinned host memory, on its stream ----
    pinned_frames = [torch.from_numpy(f.view(np.uint8).reshape(-1).copy()).pin_memory() for f in frames_host]
    images_host = [torch.empty((H, W, 4), dtype=torch.uint8).pin_memory() for _ in range(2)]
    dev.read_stats(reset=True)
    torch.cuda.synchronize()
    e_begin.record(stream)
    loop.begin()
    for k in range(args.steps):
        frame(k, instances_host=pinned_frames[k % FRAMES], image_host=images_host[k & 1], image_direct=True)
    loop.end()
    e_end.record(stream)
    torch.cuda.synchronize()
    e2e_stats = dev.read_stats(reset=True)
    e2e_ms = e_begin.elapsed_time(e_end)
    e2e_value = e2e_stats["traversals"] / (e2e_ms / 1e3) / 1e6 * (world if world > 1 else 1)

    # ---- roofline of the dominant kernel (trace) ----
    # algorithmic bytes per launch from an untimed statistics run of frame 0
    dev.read_stats(reset=True)
    loop.record(0, DEPTH, SHADOWS, instances=frames_dev[0], uniforms_dev=uni_dev[0],
                flags=abi.RT_TRACE_FLAG_COLLECT_STATS, refit=wl.refit)
    torch.cuda.synchronize()
    s = dev.read_stats(reset=True)
    # the traversal kernel (k_trace) is the dominant kernel; per frame it runs
    # once per bounce (closest hit) and once for the shadow rays
    bytes_per_frame = (s["traversals"] * (RAY_BYTES + HIT_BYTES) + s["nodes_visited"] * NODE_BYTES +
                       s["triangles_tested"] * TRI_BYTES + s["instances_visited"] * INST_BYTES)
    bytes_per_launch = bytes_per_frame / traversal_launches
    avg_launch_s = sum(traversal_ms) / len(traversal_ms) / traversal_launches / 1e3
    peak, peak_kind = measured_peaks()
    achieved = bytes_per_launch / avg_launch_s / 1e9
    traffic = profiled_traffic(wl.profile) if wl.profile else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(wl)

    if rank == 0:
        line = {
            "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": wl.data,
            "config": {"workload": wl.description, "width": W, "height": H, "instances": n_inst,
                       "instanced_triangles": sc0.instanced_triangles, "frames": FRAMES,
                       "max_trace_depth": DEPTH, "shadow_rays": SHADOWS,
                       "path": wl.path, "parallelism": f"replicas x{world}",
                       "frame_loop": wl.loop_note(),
                       "l2": "flushed before every frame on its stream (256 MiB write, inside the timed span)",
                       "traversals_per_step": rays_local / args.steps, "blas_build_ms": blas_build_ms,
                       "serial_ms_per_frame": sum(serial_ms) / len(serial_ms),
                       "trace_pipeline_ms_per_step": sum(trace_ms) / len(trace_ms),
                       "traversal_ms_per_step": sum(traversal_ms) / len(traversal_ms),
                       "shade_ms_per_step": sum(kt["shade_ms"] for kt in kernel_times) / len(kernel_times),
                       "tlas_build_and_flush_ms_per_step": (sum(serial_ms) - sum(trace_ms)) / len(serial_ms),
                       "traversal_config": {"block_size": tuned.block_size,
                                            "shared_stack_depth": tuned.shared_stack_depth,
                                            "leaf_wait": tuned.leaf_wait, "packet_lists": tuned.packet_lists,
                                            **tune_note},
                       "work_counts": "nodes / triangles per ray from a statistics frame of the per-lane "
                                      "traversal (what each ray needs)"},
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": n_inst * 64,
                    "d2h_bytes_per_step": W * H * 4},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_trace (traversal; closest-hit per bounce + shadow)",
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "launches_per_step": traversal_launches,
                         "algorithmic_bytes_per_launch": bytes_per_launch,
                         "bytes_per_ray": bytes_per_frame / max(1, s["traversals"]),
                         "nodes_per_ray": s["nodes_visited"] / max(1, s["traversals"]),
                         "triangles_per_ray": s["triangles_tested"] / max(1, s["traversals"])},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
        }
        print(json.dumps(line))
    dev.close()
    if dist:
        dist.destroy_process_group()


PRECISION_RAY_SEED = 2024


def precision_inputs(args):
    model = scenes.precision_mesh(level=args.precision_level)
    sc = scenes.single_mesh_scene(model)
    rays = scenes.random_rays(args.precision_rays, PRECISION_RAY_SEED, 30.0)
    return sc, rays


def precision_cpu(sc, rays, budget_s: float = 12.0) -> dict:
    """The oracle tracing chunks of the step's rays (FP32, all host threads)
    until about `budget_s` seconds of CPU work; the BVH build is untimed."""
    from oracle.oracle import OracleScene, default_threads

    threads = default_threads()
    o = OracleScene(sc)
    chunk = 1 << 18
    done, t_total = 0, 0.0
    while t_total < budget_s and done < len(rays):
        part = rays[done:done + chunk]
        t = time.perf_counter()
        o.trace(part, with_models=False, threads=threads)
        t_total += time.perf_counter() - t
        done += len(part)
    return {"value": done / t_total / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"first {done} of the step's {len(rays)} rays ({t_total:.1f} s; binary SAH host BVH, "
                      f"build untimed)"}


def bench_precision_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import OracleScene, default_threads

    threads = default_threads()
    sc, rays = precision_inputs(args)
    o = OracleScene(sc)
    chunk = max(1, len(rays) // 16)
    times, traced = [], 0
    for k in range(args.warmup + args.steps):
        i0 = (k * chunk) % len(rays)
        part = rays[i0:i0 + chunk]
        t = time.perf_counter()
        o.trace(part, with_models=False, threads=threads)
        dt = time.perf_counter() - t
        if k >= args.warmup:
            times.append(dt)
            traced += len(part)
    total = sum(times)
    value = traced / total / 1e6
    print(json.dumps({
        "impl": "reference", "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": PRECISION_WORKLOAD, "sample": f"{chunk} of the {len(rays)} rays per step"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"{chunk} rays per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def bench_precision(args):
    """Quantised (8-bit child boxes) against FP32 nodes over the same mesh and
    rays: one step = one rt_cmd_trace_ray_buffer launch over all rays."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from rtgallery import host

    dev = host.Device()
    lib = dev.lib
    sc, rays = precision_inputs(args)
    n = len(rays)
    stream = torch.cuda.current_stream()
    sh = host.Device.stream_handle(stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    rays_dev = host.Device.upload(rays)
    hits_dev = torch.empty(n * RAY_HIT_BYTES, dtype=torch.uint8, device="cuda")
    arms = {}
    for name, flags in (("fp32", abi.RT_BUILD_PREFER_FAST_TRACE),
                        ("quantized", abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_QUANTIZED_NODES)):
        torch.cuda.synchronize()
        b0, b1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        b0.record(stream)
        gs = host.GpuScene(dev, sc, blas_flags=flags, stream=stream)
        b1.record(stream)
        torch.cuda.synchronize()
        info = gs.models[0].blas.info(dev)
        # the build's device work alone: the same BLAS rebuilt into its own
        # memory (inputs resident, scratch allocated, L2 flushed before each)
        rebuild_ms = []
        for i in range(3):
            flush.fill_(i & 0xFF)
            r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            r0.record(stream)
            gs.models[0].blas.rebuild_blas(dev, gs.scratch, gs.models[0].geometries, stream)
            r1.record(stream)
            torch.cuda.synchronize()
            rebuild_ms.append(r0.elapsed_time(r1))
        arms[name] = {"scene": gs, "build_ms": b0.elapsed_time(b1), "rebuild_ms": sorted(rebuild_ms)[1],
                      "blas_bytes": int(info.total_size), "node_bytes": int(info.node_bytes),
                      "nodes": int(info.node_count)}

    def launch(gs, ray_ptr, hit_ptr, ray_flags=0):
        push = abi.RtPushConstantBufferAddresses()
        dev.check(lib.rt_cmd_trace_ray_buffer(dev.ctx, gs.tlas.device_address(), C.byref(push), None, ray_flags,
                                              0xFF, 0, ray_ptr, n, hit_ptr, sh))

    def timed(gs, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for i in range(steps):
            flush.fill_(i & 0xFF)
            ev[i][0].record(stream)
            launch(gs, rays_dev.data_ptr(), hits_dev.data_ptr())
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in ev]

    for arm in arms.values():
        timed(arm["scene"], args.warmup)
    # both arms' hits must agree bit for bit before anything is reported
    launch(arms["fp32"]["scene"], rays_dev.data_ptr(), hits_dev.data_ptr())
    h_fp32 = hits_dev.clone()
    launch(arms["quantized"]["scene"], rays_dev.data_ptr(), hits_dev.data_ptr())
    torch.cuda.synchronize()
    identical = bool(torch.equal(h_fp32, hits_dev))
    hit_rate = float((h_fp32.view(torch.int32).view(-1, 8)[:, 3] != -1).float().mean())  # instance_id
    del h_fp32

    clocks = ClockSampler(local)
    clocks.start()
    launches0 = lib.rt_kernel_launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for name in ("fp32", "quantized"):
        arms[name]["ms"] = timed(arms[name]["scene"], args.steps)
    if dist:
        dist.barrier()
    launches = lib.rt_kernel_launch_count() - launches0
    clk = clocks.stop()
    for arm in arms.values():
        total_ms, _ = reduce_over_ranks(dist, sum(arm["ms"]), 0.0)
        arm["total_ms"] = total_ms
        arm["value"] = n * world * args.steps / (total_ms / 1e3) / 1e6

    # algorithmic bytes per launch: an untimed statistics launch per arm
    for arm in arms.values():
        dev.read_stats(reset=True)
        launch(arm["scene"], rays_dev.data_ptr(), hits_dev.data_ptr(), abi.RT_RAY_FLAG_EXT_COLLECT_STATS)
        s = dev.read_stats(reset=True)
        arm["stats"] = s
        arm["bytes_per_launch"] = (n * (RAY_BYTES + RAY_HIT_BYTES) + s["nodes_visited"] * arm["node_bytes"] +
                                   s["triangles_tested"] * TRI_BYTES + s["instances_visited"] * INST_BYTES)
        arm["gbs"] = arm["bytes_per_launch"] / (arm["total_ms"] / args.steps / 1e3) / 1e9

    # end to end through the C ABI with host buffers (pinned): rt_trace_ray_buffer_host with chunk_rays 0
    # traces straight from / into the mapped host memory in one launch; with chunk_rays > 0 it stages
    # copies chunk by chunk on two streams, overlapped with the traversal (both measured)
    q = arms["quantized"]["scene"]
    rays_pinned = torch.from_numpy(rays.view(np.uint8).reshape(-1).copy()).pin_memory()
    hits_pinned = torch.empty(n * RAY_HIT_BYTES, dtype=torch.uint8).pin_memory()
    push0 = abi.RtPushConstantBufferAddresses()

    def host_query(chunk):
        dev.check(lib.rt_trace_ray_buffer_host(dev.ctx, q.tlas.device_address(), C.byref(push0), None, 0, 0xFF, 0,
                                               rays_pinned.data_ptr(), n, hits_pinned.data_ptr(), chunk, sh))

    e2e_modes = {}
    for mode, chunk in (("direct", 0), ("staged", E2E_CHUNK)):
        hits_pinned.zero_()
        host_query(chunk)
        torch.cuda.synchronize()
        e2e_ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
                  for _ in range(args.steps)]
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            e2e_ev[i][0].record(stream)
            host_query(chunk)
            e2e_ev[i][1].record(stream)
        torch.cuda.synchronize()
        e2e_ms = sum(a.elapsed_time(b) for a, b in e2e_ev)
        e2e_modes[mode] = {"value": n * world * args.steps / (e2e_ms / 1e3) / 1e6, "chunk_rays": chunk,
                           "hits_equal_device_query": bool(np.array_equal(hits_pinned.numpy(), hits_dev.cpu().numpy()))}
    e2e_value = e2e_modes["direct"]["value"]

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = precision_cpu(sc, rays)
    peak, peak_kind = measured_peaks()
    qa, fa = arms["quantized"], arms["fp32"]
    if rank == 0:
        def summary(a):
            s = a["stats"]
            return {"mrays_s": a["value"], "ms_per_step": a["total_ms"] / args.steps, "gb_s": a["gbs"],
                    "bytes_per_ray": a["bytes_per_launch"] / n, "nodes_per_ray": s["nodes_visited"] / n,
                    "triangles_per_ray": s["triangles_tested"] / n, "node_bytes": a["node_bytes"],
                    "blas_bytes": a["blas_bytes"], "wide_nodes": a["nodes"],
                    "blas_build_ms": a["rebuild_ms"], "scene_setup_ms": a["build_ms"]}

        print(json.dumps({
            "metric": "Mrays/s", "value": qa["value"], "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": qa["total_ms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (procedural mesh and rays from seeds)",
            "config": {"workload": PRECISION_WORKLOAD, "path": "8-bit quantised child boxes (value) vs FP32 boxes",
                       "rays": n, "triangles": int(sum(len(g.indices) for g in sc.models[0].geometries)),
                       "parallelism": f"replicas x{world}",
                       "l2": "flushed between steps (256 MiB write outside the timed events); BVH >> L2",
                       "hits_identical_quantized_vs_fp32": identical, "hit_rate": hit_rate,
                       "quantized": summary(qa), "fp32": summary(fa),
                       "speedup_quantized_over_fp32": qa["value"] / fa["value"],
                       "build_times": "blas_build_ms: median of 3 rebuilds of the BLAS into its own memory "
                                      "(device events, mesh resident, L2 flushed before each); scene_setup_ms: "
                                      "the first GpuScene construction (mesh upload from pageable host memory, "
                                      "allocations, BLAS and TLAS builds)"},
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": n * RAY_BYTES,
                    "d2h_bytes_per_step": n * RAY_HIT_BYTES, "api": "rt_trace_ray_buffer_host",
                    "mode": "direct (pinned host rays / hits read and written by the traversal)",
                    "hits_equal_device_query": e2e_modes["direct"]["hits_equal_device_query"],
                    "staged_copies": e2e_modes["staged"]},
            "roofline": {"bound": "hbm", "achieved": qa["gbs"], "peak": peak, "unit": "GB/s", "frac": qa["gbs"] / peak,
                         "traffic": profiled_traffic("k_trace_ray_buffer_precision.md"),
                         "kernel": "k_trace_ray_buffer (quantised BLAS)",
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "algorithmic_bytes_per_launch": qa["bytes_per_launch"]},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches),
        }))
    dev.close()
    if dist:
        dist.destroy_process_group()


BATCH_METRIC = "Mrays/s quantized+batched vs plain FP32 (exact hit IDs); serve p50/p99 ms"
BATCH_WORKLOAD = ("batch: 64 independent scenes (procedural torus + displaced UV sphere + ground grid, unique "
                  "triangles log-uniform in [10k, 2M], resolutions from {128^2, 256^2, 512^2, 1024^2, 1920x1080}), "
                  "primary + 2 blue-noise soft shadows + 1 reflection bounce each, one batched launch sequence "
                  "replayed from a CUDA graph")


def batch_setup(dev, scs, quantized: bool = False, width4: bool = False, radiance: bool = False):
    """GPU scenes and frames of the batch: BLASes with FP32 boxes or 8-bit
    quantised child boxes, 8 or at most 4 children per node."""
    from rtgallery import host

    w = abi.RT_BUILD_EXT_NODE_WIDTH_4 if width4 else 0
    q = abi.RT_BUILD_QUANTIZED_NODES if quantized else 0
    frames = []
    for sc in scs:
        gs = host.GpuScene(dev, sc, own_textures=True, blas_flags=abi.RT_BUILD_PREFER_FAST_TRACE | q | w,
                           tlas_flags=abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_ALLOW_UPDATE | w)
        fr = host.PerFrameResources(dev, gs, sc.width, sc.height, radiance=radiance)
        fr.write_uniforms(sc.uniforms)
        frames.append(fr)
    return frames


def build_oracles(scs, threads: int | None = None):
    """One oracle per scene, built on a thread pool (the oracle's BVH build
    runs in C with the interpreter lock released)."""
    from concurrent.futures import ThreadPoolExecutor

    from oracle.oracle import OracleScene, default_threads

    with ThreadPoolExecutor(max_workers=threads or default_threads()) as ex:
        return list(ex.map(OracleScene, scs))


def batch_cpu(scs, oracles, budget_s: float = 12.0) -> dict:
    """The oracle (FP32, all host threads) rendering row bands of the batch's
    scenes in turn until about `budget_s` seconds of CPU work (the oracles'
    BVH builds are not timed)."""
    from oracle.oracle import default_threads

    threads = default_threads()
    rays, t_total, done = 0, 0.0, 0
    for k in range(len(scs) * 16):
        sc, o = scs[k % len(scs)], oracles[k % len(scs)]
        band = max(4, sc.height // 16)
        y0 = ((k // len(scs)) * band) % max(1, sc.height - band)
        t = time.perf_counter()
        _, _, st = o.render(rows=(y0, y0 + band), threads=threads)
        t_total += time.perf_counter() - t
        rays += st["traversals"]
        done += 1
        if t_total >= budget_s:
            break
    return {"value": rays / t_total / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
            "sample": f"{done} row bands of 1/16 of a scene's rows, the 64 scenes in turn ({rays} traversals, "
                      f"{t_total:.1f} s)"}


def radiance_error_bands(scs, oracles, radiance_host) -> dict:
    """Per image: max-abs linear radiance error of the GPU against the FP32
    oracle (the <= 1e-3 tolerance) and against the FP64 oracle (reported), on
    the central 1/16 of its rows."""
    from oracle.oracle import default_threads

    err32, err64 = [], []
    for sc, o, rad in zip(scs, oracles, radiance_host):
        band = max(4, sc.height // 16)
        y0 = (sc.height - band) // 2
        _, r32, _ = o.render(rows=(y0, y0 + band), threads=default_threads())
        _, r64, _ = o.render(rows=(y0, y0 + band), double=True, threads=default_threads())
        g = rad[y0:y0 + band, :, :3]
        err32.append(float(np.abs(g - r32[y0:y0 + band, :, :3]).max()))
        err64.append(float(np.abs(g - r64[y0:y0 + band, :, :3]).max()))
    return {"rows": "central 1/16 of each image's rows", "tolerance_vs_fp32_oracle": 1e-3,
            "max_abs_vs_fp32_oracle": max(err32), "max_abs_vs_fp64_oracle": max(err64),
            "per_image_max_abs_vs_fp64_oracle": err64, "per_image_max_abs_vs_fp32_oracle": err32}


def camera_ray_sample(sc, step: int) -> np.ndarray:
    """The camera rays (ray_generation's formula, in float32) of every
    `step`-th pixel in x and y of scene `sc`."""
    u = sc.uniforms
    vi = np.array(u.view_inverse, np.float32).reshape(4, 4).T  # column-major -> [row, col]
    pi = np.array(u.proj_inverse, np.float32).reshape(4, 4).T
    ys, xs = np.mgrid[0:sc.height:step, 0:sc.width:step]
    xs, ys = xs.ravel().astype(np.float32), ys.ravel().astype(np.float32)
    ndc = np.stack([(xs + 0.5) / sc.width * 2 - 1, (ys + 0.5) / sc.height * 2 - 1,
                    np.ones_like(xs), np.ones_like(xs)], 1).astype(np.float32)
    tgt = (ndc @ pi.T)[:, :3]
    loc = tgt / np.linalg.norm(tgt, axis=1, keepdims=True)
    d = loc @ vi[:3, :3].T
    rays = np.zeros(len(xs), abi.RAY_DTYPE)
    rays["origin"] = vi[:3, 3]
    rays["direction"] = d.astype(np.float32)
    rays["tmin"] = 0.01
    rays["tmax"] = 10000.0
    return rays


def bench_batch_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import default_threads

    threads = default_threads()
    scs = scenes.batch_scenes(args.batch_scenes)
    oracles = build_oracles(scs)
    times, rays = [], 0
    for k in range(args.warmup + args.steps):
        sc, o = scs[k % len(scs)], oracles[k % len(scs)]
        band = max(4, sc.height // 32)
        y0 = (k * band) % max(1, sc.height - band)
        t = time.perf_counter()
        _, _, st = o.render(rows=(y0, y0 + band), threads=threads)
        dt = time.perf_counter() - t
        if k >= args.warmup:
            times.append(dt)
            rays += st["traversals"]
    total = sum(times)
    value = rays / total / 1e6
    print(json.dumps({
        "impl": "reference", "metric": BATCH_METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "sample": "a 1/32 row band of one scene per step",
                   "path": "the reference's shader logic on the host (oracle port), FP32, one scene at a time"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"1/32 row band of one scene per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def bench_batch(args):
    """The headline: 64 scenes rendered by the quantised + batched path (8-bit
    child boxes, one batched launch sequence replayed from a CUDA graph, the
    launch shape and node width from rt_ctx_autotune) against the plain FP32
    path (FP32 boxes, one rt_cmd_trace_rays per scene, the library's default
    launch shape), with every image and a sample of hits compared between the
    two; then the serving stream's latency percentiles."""
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    from rtgallery import host

    dev = host.Device()
    lib = dev.lib
    scs = scenes.batch_scenes(args.batch_scenes)
    t0 = time.perf_counter()
    fr32 = batch_setup(dev, scs)
    frq8 = batch_setup(dev, scs, quantized=True)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    note(f"batch: 64 scenes built twice (FP32, quantised) in {setup_s:.1f} s")
    stream = torch.cuda.Stream()
    sh = host.Device.stream_handle(stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    default_cfg = abi.RtTraversalConfig(128, 0, 20, 0)

    def items_of(frames, **kw):
        its = [host.batch_scene(fr, sc.max_trace_depth, sc.shadow_ray_count, **kw) for fr, sc in zip(frames, scs)]
        return (abi.RtBatchScene * len(its))(*its)

    arr32, arrq8 = items_of(fr32), items_of(frq8)

    def batched(arr, flags=0):
        dev.check(lib.rt_cmd_trace_rays_batched(dev.ctx, arr, len(scs), None, flags, sh))

    def plain():
        # the drop-in: one rt_cmd_trace_rays per scene (PerFrameResources::record), FP32 nodes
        for fr, sc in zip(fr32, scs):
            fr.gpu_scene.bind_textures()
            fr.record(sc.max_trace_depth, sc.shadow_ray_count, stream=stream)

    def timed(fn, steps):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        with torch.cuda.stream(stream):
            for i in range(steps):
                flush.fill_(i & 0xFF)
                ev[i][0].record(stream)
                fn()
                ev[i][1].record(stream)
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in ev)

    def set_cfg(cfg):
        dev.check(lib.rt_ctx_set_traversal_config(dev.ctx, C.byref(cfg)))

    def autotune(arr):
        rep = abi.RtAutotuneReport()
        dev.check(lib.rt_ctx_autotune(dev.ctx, arr, len(scs), None, 3, sh, C.byref(rep)))
        return rep.median_ms[rep.best], abi.RtTraversalConfig(*rep.configs[rep.best].as_tuple()), rep

    set_cfg(default_cfg)
    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            plain()
            batched(arr32)
            batched(arrq8)
    torch.cuda.synchronize()
    dev.read_stats(reset=True)
    with torch.cuda.stream(stream):
        batched(arrq8)
    torch.cuda.synchronize()
    rays_per_step = dev.read_stats(reset=True)["traversals"]

    # ---- the plain FP32 path: per-scene calls, default launch shape ----
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    ms_plain = timed(plain, args.steps)
    note(f"plain FP32 per-scene: {ms_plain / args.steps:.2f} ms per step")
    plain_images = [fr.image.clone() for fr in fr32]

    # ---- the autotuner: launch shape for the FP32 batch (decomposition only), and launch shape x node
    # width {8, 4} for the quantised batch; the graph is captured with the quantised winner ----
    t_tune = time.perf_counter()
    if args.traversal:  # a given launch shape for both paths, 8-wide nodes, no tuning
        fixed = abi.RtTraversalConfig(*(int(v) for v in args.traversal.split(",")))
        best32 = best_q8 = best_q4 = (None, fixed, abi.RtAutotuneReport())
        frq4 = arrq4 = None
        width, tuned = 8, fixed
    else:
        best32 = autotune(arr32)
        best_q8 = autotune(arrq8)
        frq4 = batch_setup(dev, scs, quantized=True, width4=True)
        arrq4 = items_of(frq4)
        with torch.cuda.stream(stream):
            batched(arrq4)  # sizes the workspace outside the tuner
        torch.cuda.synchronize()
        best_q4 = autotune(arrq4)
        width = 4 if best_q4[0] < best_q8[0] else 8
        tuned = best_q4[1] if width == 4 else best_q8[1]
    tune_s = time.perf_counter() - t_tune
    frq, arrq = (frq4, arrq4) if width == 4 else (frq8, arrq8)
    note(f"traversal config: quantised width {width} {tuned.as_tuple()} ({tune_s:.1f} s), "
         f"best ms q8 {best_q8[0]} q4 {best_q4[0]} fp32 {best32[0]}")

    # FP32 batched (the batching gain alone), its own tuned launch shape
    set_cfg(best32[1])
    g32 = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g32, stream=stream):
        batched(arr32)
    for _ in range(args.warmup):
        g32.replay()
    torch.cuda.synchronize()
    ms_batch32 = timed(g32.replay, args.steps)
    del g32

    # ---- the quantised + batched path (value) ----
    set_cfg(tuned)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        batched(arrq)
    for _ in range(args.warmup):
        graph.replay()
    torch.cuda.synchronize()
    clocks = ClockSampler(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = lib.rt_kernel_launch_count()
    with torch.cuda.stream(stream):
        batched(arrq)
    torch.cuda.synchronize()
    launches_per_step = lib.rt_kernel_launch_count() - l0
    ms_graph = timed(graph.replay, args.steps)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms_graph, _ = reduce_over_ranks(dist, ms_graph, 0.0)
    value = rays_per_step * world * args.steps / (ms_graph / 1e3) / 1e6
    plain_value = rays_per_step * args.steps / (ms_plain / 1e3) / 1e6
    batch32_value = rays_per_step * args.steps / (ms_batch32 / 1e3) / 1e6
    note(f"quantised+batched {value:.0f} Mrays/s, plain FP32 {plain_value:.0f}, batched FP32 {batch32_value:.0f}")

    # ---- exact hits: every image of the quantised batch equals the plain path's, byte for byte, and
    # the camera rays of every 4th pixel (each axis) hit the same (t, u, v, instance, geometry,
    # primitive, facing) through FP32 and quantised structures ----
    images_identical = all(torch.equal(a, fr.image) for a, fr in zip(plain_images, frq))
    hit_rays, hits_identical = 0, True
    for gs32, gsq, sc in zip([f.gpu_scene for f in fr32], [f.gpu_scene for f in frq], scs):
        rays = camera_ray_sample(sc, 4)
        a = host.trace_ray_buffer(dev, gs32, rays)
        b = host.trace_ray_buffer(dev, gsq, rays)
        hit_rays += len(rays)
        hits_identical = hits_identical and bool(np.array_equal(a.view(np.uint8), b.view(np.uint8)))

    # ---- kernel split and roofline of the traversal (a direct call with per-kernel events; work counts
    # from a statistics run of the per-lane traversal) ----
    with torch.cuda.stream(stream):
        batched(arrq, abi.RT_TRACE_FLAG_KERNEL_TIMINGS)
    tt = abi.RtTraceTimings()
    dev.check(lib.rt_ctx_read_trace_timings(dev.ctx, C.byref(tt)))
    kt = tt.as_dict()
    torch.cuda.synchronize()
    dev.read_stats(reset=True)
    with torch.cuda.stream(stream):
        batched(arrq, abi.RT_TRACE_FLAG_COLLECT_STATS)
    torch.cuda.synchronize()
    s = dev.read_stats(reset=True)
    fp32_nodes = s["nodes_visited"] - s["quantized_nodes_visited"]
    bytes_step = (s["traversals"] * (RAY_BYTES + HIT_BYTES) + fp32_nodes * NODE_BYTES +
                  s["quantized_nodes_visited"] * QNODE_BYTES + s["triangles_tested"] * TRI_BYTES +
                  s["instances_visited"] * INST_BYTES)
    achieved = bytes_step / (kt["trace_ms"] / 1e3) / 1e9
    note(f"hits identical {hits_identical}, images identical {images_identical}; traversal {kt['trace_ms']:.2f} ms")
    peak, peak_kind = measured_peaks()
    prof = profiled_figures("k_trace_batch_quantized.md")

    # ---- end to end: every scene's uniforms in from pinned host memory (one copy into one device array),
    # every image written into its pinned host buffer by the output kernel, inside the timed span ----
    uni_host = torch.from_numpy(np.concatenate([np.frombuffer(bytes(sc.uniforms), np.uint8)
                                                for sc in scs])).pin_memory()
    img_host = [torch.empty_like(fr.image, device="cpu").pin_memory() for fr in frq]
    usz = C.sizeof(abi.RtUniforms)
    uni_dev = torch.empty_like(uni_host, device="cuda")
    arr_e2e = (abi.RtBatchScene * len(scs))(*[
        host.batch_scene(fr, sc.max_trace_depth, sc.shadow_ray_count, uniforms_address=uni_dev.data_ptr() + k * usz,
                         image_address=img_host[k].data_ptr()) for k, (fr, sc) in enumerate(zip(frq, scs))])
    uni_dev.copy_(uni_host)
    graph_e2e = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph_e2e, stream=stream):
        dev.check(lib.rt_cmd_trace_rays_batched(dev.ctx, arr_e2e, len(scs), None, 0, sh))
    for _ in range(args.warmup):
        graph_e2e.replay()
    torch.cuda.synchronize()

    def e2e_step():
        uni_dev.copy_(uni_host, non_blocking=True)
        graph_e2e.replay()

    e2e_ms = timed(e2e_step, args.steps)
    e2e_images_ok = all(torch.equal(a, b.cpu()) for a, b in zip(img_host, plain_images))
    e2e_value = rays_per_step * world * args.steps / (e2e_ms / 1e3) / 1e6
    del graph, graph_e2e

    # ---- radiance against the FP32 and FP64 oracles, and the timed CPU baseline ----
    err = cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rad = [torch.zeros((sc.height, sc.width, 4), dtype=torch.float32, device="cuda") for sc in scs]
        arr_rad = (abi.RtBatchScene * len(scs))(*[
            host.batch_scene(fr, sc.max_trace_depth, sc.shadow_ray_count) for fr, sc in zip(frq, scs)])
        for k in range(len(scs)):
            arr_rad[k].desc.radiance_address = rad[k].data_ptr()
        with torch.cuda.stream(stream):
            batched(arr_rad)
        torch.cuda.synchronize()
        rad_host = [r.cpu().numpy() for r in rad]
        del rad
        oracles = build_oracles(scs)
        err = radiance_error_bands(scs, oracles, rad_host)
        cpu = batch_cpu(scs, oracles)
        del oracles
    pixels = sum(sc.width * sc.height for sc in scs)
    unique_tris = int(sum(m.triangle_count for sc in scs for m in sc.models))
    del fr32, frq8, frq4, frq, arr32, arrq8, arrq4, arrq
    torch.cuda.synchronize()
    torch.cuda.empty_cache()

    note("batch part done; serving stream next")
    serve = serve_measure(args, plain_seconds=args.serve_plain_seconds) if args.serve_seconds > 0 else None
    if rank == 0:
        cfg = {"workload": BATCH_WORKLOAD, "scenes": len(scs), "pixels_per_step": pixels,
               "unique_triangles": unique_tris, "traversals_per_step": rays_per_step,
               "parallelism": f"replicas x{world}",
               "l2": "flushed before every step (256 MiB write on the stream, outside the timed events)",
               "path": "quantised + batched: BLASes with 8-bit child boxes, one batched launch sequence for the "
                       "64 scenes replayed from a CUDA graph, launch shape and node width from rt_ctx_autotune",
               "plain_fp32_path": "FP32 child boxes, one rt_cmd_trace_rays per scene, default launch shape "
                                  "(128, 0, 20, 0)",
               "plain_fp32_mrays_s": plain_value,
               "speedup_over_plain_fp32": value / plain_value,
               "batched_fp32_mrays_s": batch32_value,
               "hits_identical": hits_identical and images_identical,
               "images_identical_to_plain": images_identical,
               "hit_sample": f"{hit_rays} camera rays (every 4th pixel in x and y of all 64 scenes) traced through "
                             f"FP32 and quantised structures: t, u, v, instance, geometry, primitive and facing "
                             f"bit-identical = {hits_identical}",
               "radiance": err,
               "autotuned_config": {"node_width": width, "block_size": tuned.block_size,
                                    "shared_stack_depth": tuned.shared_stack_depth,
                                    "leaf_wait": tuned.leaf_wait, "packet_lists": tuned.packet_lists,
                                    "chosen_by": "--traversal" if args.traversal else "rt_ctx_autotune"},
               "autotune_configs": int(best_q8[2].count + best_q4[2].count + best32[2].count),
               "autotune_s": tune_s,
               "autotune_best_ms": {"quantized_width8": best_q8[0], "quantized_width4": best_q4[0],
                                    "fp32_width8": best32[0]},
               "kernel_launches_per_step": launches_per_step, "scene_setup_s": setup_s,
               "trace_ms_per_step": kt["trace_ms"], "shade_ms_per_step": kt["shade_ms"],
               "pipeline_ms_per_step": kt["total_ms"]}
        if serve is not None:
            cfg["serve"] = serve
        print(json.dumps({
            "metric": BATCH_METRIC, "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_graph / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (procedural scenes from seeds)",
            "config": cfg,
            "e2e": {"value": e2e_value, "unit": "Mrays/s", "h2d_bytes_per_step": usz * len(scs),
                    "d2h_bytes_per_step": pixels * 4,
                    "path": "rt_cmd_trace_rays_batched in a CUDA graph: one copy of the 64 uniform blocks in from "
                            "pinned host memory, every RGBA8 image written into its pinned host buffer by the "
                            "output kernel",
                    "images_identical_to_plain": e2e_images_ok},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": prof.get("dram_bytes_per_launch"),
                         "kernel": "k_trace (every traversal launch of the quantised batch)",
                         "achieved_is": "algorithmic bytes per step (rays, hits, 96-byte quantised BLAS nodes, "
                                        "256-byte TLAS nodes, triangles, instance records, counted by a statistics "
                                        "run) / traversal time per step; most of them are L2 hits",
                         "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "fallback 6.8 TB/s",
                         "algorithmic_bytes_per_step": bytes_step,
                         "bytes_per_ray": bytes_step / max(1, s["traversals"]),
                         "nodes_per_ray": s["nodes_visited"] / max(1, s["traversals"]),
                         "quantized_nodes_per_ray": s["quantized_nodes_visited"] / max(1, s["traversals"]),
                         "dram_frac_of_peak_from_profile": prof.get("dram_frac"),
                         "l2_throughput_pct_from_profile": prof.get("l2_pct"),
                         "profile": "profiles/k_trace_batch_quantized.md" if prof else None},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(launches_per_step) * args.steps,
        }))
    dev.close()
    if dist:
        dist.destroy_process_group()


SERVE_WORKLOAD = ("serve: Poisson request stream (seeded) over 32 device-resident scenes (procedural, unique "
                  "triangles log-uniform in [50k, 4M], RGBA8 textures), each request a random scene, camera and "
                  "light, resolution from {256^2, 512^2, 1024^2, 1280x720, 1920x1080}, 1-8 soft-shadow rays and "
                  "1 reflection bounce; admission by an HBM budget for BVHs + textures + frame buffers; "
                  "continuous batching vs the plain one-request-per-launch path on the same stream")


SERVE_MAX_BATCH, SERVE_IN_FLIGHT = 32, 2
# batch limits of the batched server (ray slots, shadow rays), and of the plain server (one request of the
# largest size: 1920x1080 with 8 shadow rays)
SERVE_BATCH_SLOTS, SERVE_BATCH_SHADOW = 4 << 20, 16 << 20
SERVE_REQUEST_SLOTS, SERVE_REQUEST_SHADOW = 1920 * 1080, 1920 * 1080 * 8


def serve_requests(args, n_scenes):
    """The seeded request stream: (arrival s, scene, w, h, shadows, uniforms)."""
    rng = scenes.Pcg32(4242, 0x77)
    t, out = 0.0, []
    while True:
        t += -math.log(1.0 - rng.uniform()) / args.serve_rate
        if t >= args.serve_seconds:
            break
        sc = int(rng.next_u32() % n_scenes)
        w, h = scenes.SERVE_RESOLUTIONS[int(rng.next_u32() % len(scenes.SERVE_RESOLUTIONS))]
        shadows = 1 + int(rng.next_u32() % 8)
        out.append((t, sc, w, h, shadows, scenes.random_view_uniforms(rng, w, h, frame=len(out))))
    return out


def run_stream(dev, gscenes, reqs, budget, max_batch, in_flight, ring):
    """Replays `reqs` at their arrival times against a fresh server; returns
    (latencies ms, queue ms, batch sizes, wall s, traversals, server stats).
    Batches stay within SERVE_BATCH_SLOTS ray slots and SERVE_BATCH_SHADOW
    shadow rays (a larger request alone), and the server sizes its workspace
    and frame-buffer pool for that at creation."""
    import torch

    from rtgallery import host

    srv = host.Server(dev, budget, max_batch_requests=max_batch, max_in_flight=in_flight,
                      max_batch_pixels=SERVE_BATCH_SLOTS if max_batch > 1 else SERVE_REQUEST_SLOTS,
                      max_batch_shadow_rays=SERVE_BATCH_SHADOW if max_batch > 1 else SERVE_REQUEST_SHADOW)
    ids = [srv.add_scene(g) for g in gscenes]
    tickets = [None] * len(reqs)
    results = [None] * len(reqs)
    slot_owner = [None] * len(ring)
    torch.cuda.synchronize()
    dev.read_stats(reset=True)

    def waiter():
        for i in range(len(reqs)):
            while tickets[i] is None:
                time.sleep(0.0002)
            results[i] = srv.wait(tickets[i], 600000)

    th = threading.Thread(target=waiter)
    th.start()
    t0 = time.perf_counter()
    for i, (t, sc, w, h, shadows, u) in enumerate(reqs):
        k = i % len(ring)
        while slot_owner[k] is not None and results[slot_owner[k]] is None:
            time.sleep(0.0002)  # the pinned slot is still being written by an earlier request
        slot_owner[k] = i
        delay = t0 + t - time.perf_counter()
        if delay > 0:
            time.sleep(delay)
        tickets[i] = srv.submit(ids[sc], u, w, h, 2, shadows, image_host=ring[k].data_ptr())
    th.join()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    torch.cuda.synchronize()
    rays = dev.read_stats(reset=True)["traversals"]
    lat = np.array([r.latency_ms for r in results])
    qms = np.array([r.queue_ms for r in results])
    bs = np.array([r.batch_requests for r in results])
    return lat, qms, bs, wall, rays, st


def run_alone(dev, gscenes, reqs, budget, ring) -> np.ndarray:
    """Each request of `reqs` submitted only after the previous one finished
    (nothing else on the GPU): its service time alone, in ms."""
    from rtgallery import host

    srv = host.Server(dev, budget, max_batch_requests=1, max_in_flight=1, max_batch_pixels=SERVE_REQUEST_SLOTS,
                      max_batch_shadow_rays=SERVE_REQUEST_SHADOW)
    ids = [srv.add_scene(g) for g in gscenes]
    out = []
    for i, (t, sc, w, h, shadows, u) in enumerate(reqs):
        tk = srv.submit(ids[sc], u, w, h, 2, shadows, image_host=ring[i % len(ring)].data_ptr())
        out.append(srv.wait(tk, 600000).latency_ms)
    srv.close()
    return np.array(out)


def bench_serve_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle.oracle import OracleScene, default_threads

    threads = default_threads()
    scs = [scenes.scene_serve_member(i) for i in range(min(args.serve_scenes, 4))]
    oracles = [OracleScene(sc) for sc in scs]  # BVH builds, untimed
    reqs = serve_requests(args, len(scs))
    times, rays = [], 0
    for k in range(args.warmup + args.steps):
        t, sc, w, h, shadows, u = reqs[k % len(reqs)]
        o = oracles[sc]
        band = max(2, h // 64)
        y0 = (k * band) % max(1, h - band)
        t1 = time.perf_counter()
        _, _, st = o.render(uniforms=u, width=w, height=h, max_trace_depth=2, shadow_ray_count=shadows,
                            rows=(y0, y0 + band), threads=threads)
        dt = time.perf_counter() - t1
        if k >= args.warmup:
            times.append(dt)
            rays += st["traversals"]
    total = sum(times)
    value = rays / total / 1e6
    print(json.dumps({
        "impl": "reference", "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": SERVE_WORKLOAD, "sample": "a 1/64 row band of one request per step (4 scenes)"},
        "cpu_baseline": {"value": value, "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": f"1/64 row band of one request per step, {args.steps} steps"},
        "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def serve_measure(args, plain_seconds: float | None = None) -> dict:
    """The serving stream (args.serve_seconds of seeded Poisson arrivals at
    args.serve_rate per second over 32 resident scenes) through the batched
    server, then through the plain one-request-per-launch server over its
    first `plain_seconds` (None = all of it), then a 2000-request burst
    through both (capacity).  Returns the figures of the JSON line."""
    import torch

    from rtgallery import host

    dev = host.Device(threadsafe=True)
    t0 = time.perf_counter()
    scs = [scenes.scene_serve_member(i) for i in range(args.serve_scenes)]
    gscenes = [host.GpuScene(dev, sc, own_textures=True) for sc in scs]
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    reqs = serve_requests(args, len(scs))
    budget = int(args.serve_budget_gb * (1 << 30))
    max_px = max(w * h for w, h in scenes.SERVE_RESOLUTIONS)
    ring = [torch.empty(max_px * 4, dtype=torch.uint8).pin_memory() for _ in range(256)]
    # warm-up: a short stream so kernels, pools and the workspaces exist
    warm = [(0.0005 * i, *r[1:]) for i, r in enumerate(reqs[:64])]
    run_stream(dev, gscenes, warm, budget, SERVE_MAX_BATCH, SERVE_IN_FLIGHT, ring)
    clocks = ClockSampler(torch.cuda.current_device())
    clocks.start()
    lat, qms, bs, wall, rays, st = run_stream(dev, gscenes, reqs, budget, SERVE_MAX_BATCH, SERVE_IN_FLIGHT, ring)
    clk = clocks.stop()
    preqs = reqs if plain_seconds is None else [r for r in reqs if r[0] < plain_seconds]
    p_lat, p_q, p_bs, p_wall, p_rays, p_st = run_stream(dev, gscenes, preqs, budget, 1, 1, ring)
    # capacity: the first 2000 requests all arriving at once, batched and plain
    burst = [(0.0, *r[1:]) for r in reqs[:2000]]
    _, _, c_bs, c_wall, c_rays, _ = run_stream(dev, gscenes, burst, budget, SERVE_MAX_BATCH, SERVE_IN_FLIGHT, ring)
    _, _, _, cp_wall, cp_rays, _ = run_stream(dev, gscenes, burst, budget, 1, 1, ring)
    # the service time of each of the first 1000 requests alone; slowdown = latency in the stream / alone
    alone = run_alone(dev, gscenes, reqs[:1000], budget, ring)
    slow = lat[:len(alone)] / alone

    def pct(a, q):
        return float(np.percentile(a, q))

    out = {"workload": SERVE_WORKLOAD, "requests": len(reqs), "rate_per_s": args.serve_rate,
           "stream_s": args.serve_seconds, "scenes": len(scs),
           "unique_triangles": int(sum(m.triangle_count for sc in scs for m in sc.models)),
           "hbm_budget_bytes": budget, "peak_bytes": st["peak_bytes"], "resident_bytes": st["resident_bytes"],
           "scene_setup_s": setup_s,
           "p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "p999_ms": pct(lat, 99.9),
           "p99_over_p50": pct(lat, 99) / pct(lat, 50),
           "alone_first_1000": {"p50_ms": pct(alone, 50), "p99_ms": pct(alone, 99),
                                "p99_over_p50": pct(alone, 99) / pct(alone, 50),
                                "note": "each of the stream's first 1000 requests rendered with nothing else on "
                                        "the GPU: the spread of the requests' own service times"},
           "slowdown_first_1000": {"p50": pct(slow, 50), "p99": pct(slow, 99), "max": float(slow.max()),
                                   "note": "latency in the batched stream / the same request's time alone"},
           "batched": {"p50_ms": pct(lat, 50), "p99_ms": pct(lat, 99), "p999_ms": pct(lat, 99.9),
                       "queue_p50_ms": pct(qms, 50), "mean_batch": float(bs.mean()), "batches": st["batches"],
                       "mrays_s": rays / wall / 1e6, "wall_s": wall, "rejected": st["rejected"]},
           "plain_per_request": {"p50_ms": pct(p_lat, 50), "p99_ms": pct(p_lat, 99), "p999_ms": pct(p_lat, 99.9),
                                 "mrays_s": p_rays / p_wall / 1e6, "wall_s": p_wall, "requests": len(preqs),
                                 "rejected": p_st["rejected"]},
           "capacity_burst_2000": {"batched_mrays_s": c_rays / c_wall / 1e6, "plain_mrays_s": cp_rays / cp_wall / 1e6,
                                   "batched_req_s": len(burst) / c_wall, "plain_req_s": len(burst) / cp_wall,
                                   "mean_batch": float(c_bs.mean())},
           "max_batch_requests": SERVE_MAX_BATCH, "max_in_flight": SERVE_IN_FLIGHT, "clocks": clk,
           "traversals": rays, "wall_s": wall, "batches": int(st["batches"]),
           "mean_d2h_bytes": float(np.mean([w * h * 4 for _, _, w, h, _, _ in reqs]))}
    del gscenes
    dev.close()
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return out


def bench_serve(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    sv = serve_measure(args)
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from oracle.oracle import OracleScene, default_threads

        threads = default_threads()
        scs = [scenes.scene_serve_member(i) for i in range(args.serve_scenes)]
        reqs = serve_requests(args, len(scs))
        # requests of the four smallest scenes, one oracle BVH each (its build is untimed)
        small = sorted(range(len(scs)), key=lambda i: sum(m.triangle_count for m in scs[i].models))[:4]
        oracles = {i: OracleScene(scs[i]) for i in small}
        sample = [r for r in reqs if r[1] in oracles]
        t_cpu, r_cpu, k = 0.0, 0, 0
        while t_cpu < 10.0 and k < len(sample):
            t, sc, w, h, shadows, u = sample[k]
            o = oracles[sc]
            band = max(2, h // 64)
            t1 = time.perf_counter()
            _, _, s2 = o.render(uniforms=u, width=w, height=h, max_trace_depth=2, shadow_ray_count=shadows,
                                rows=(0, band), threads=threads)
            t_cpu += time.perf_counter() - t1
            r_cpu += s2["traversals"]
            k += 1
        cpu = {"value": r_cpu / t_cpu / 1e6, "unit": "Mrays/s", "cores": threads, "kind": "port",
               "sample": f"1/64 row bands of the first {k} requests on the 4 smallest scenes "
                         f"({r_cpu} traversals, {t_cpu:.1f} s)"}
    if rank == 0:
        value = sv["batched"]["mrays_s"]
        print(json.dumps({
            "metric": "Mrays/s", "value": value, "unit": "Mrays/s", "n_gpus": world, "steps": sv["requests"],
            "warmup": 64, "ms_per_step": 1e3 * sv["wall_s"] / sv["requests"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (procedural scenes and request stream from seeds)",
            "config": {k: v for k, v in sv.items() if k not in ("clocks", "traversals", "wall_s", "mean_d2h_bytes")},
            "e2e": {"value": value, "unit": "Mrays/s", "h2d_bytes_per_step": C.sizeof(abi.RtUniforms),
                    "d2h_bytes_per_step": sv["mean_d2h_bytes"]},
            "roofline": None,
            "cpu_baseline": cpu,
            "clocks": sv["clocks"],
            "gpu_launches": sv["batches"] * 9,
        }))


def main():
    args = parse_args()
    if args.workload == "serve":
        if args.impl == "reference":
            bench_serve_reference(args)
        else:
            bench_serve(args)
        return
    if args.workload == "batch":
        if args.impl == "reference":
            bench_batch_reference(args)
        else:
            bench_batch(args)
    elif args.workload == "precision":
        if args.impl == "reference":
            bench_precision_reference(args)
        else:
            bench_precision(args)
    elif args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
