"""Parity at the benchmarked sizes.

The other GPU tests run reduced configurations; these run the ones the
benchmark times, against the oracle:

* the full plain feature set at 1920x1080 (256 instances, 4 soft shadows,
  one reflection bounce): every ray count equal, radiance within 1e-3 of the
  FP32 oracle and of the FP64 oracle for every pixel, RGBA8 within 1 LSB, per
  lane and with camera-ray packets;
* the precision mesh at full size (level 9: 10,485,760 triangles): a
  100,000-ray sample of the benchmark's 4,194,304 random rays, hits
  bit-identical to the oracle through FP32 and through 8-bit quantised
  nodes;
* the 64 batch scenes (up to 1920x1080 each): the quantised + batched render
  of all 64 equals the plain FP32 per-scene renders byte for byte, and every
  image's radiance is within 1e-3 of the FP32 and the FP64 oracle.

The FP64 oracle shades in double precision over the same hits, so its
difference from the GPU is the error of the FP32 shading.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu

RADIANCE_TOL = 1e-3      # max-abs linear radiance, against the FP32 and the FP64 oracle
PRECISION_RAY_SEED = 2024  # the precision benchmark's ray seed
Q = abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_QUANTIZED_NODES


def _host():
    from rtgallery import host

    return host


def _set_config(device, cfg):
    device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(abi.RtTraversalConfig(*cfg))))


def _counts(st):
    return {k: st[k] for k in ("traversals", "primary_rays", "secondary_rays", "shadow_rays")}


def test_full_frame_1080p_matches_oracle(device):
    host = _host()
    sc = scenes.scene_full(0, 1920, 1080)
    gs = host.GpuScene(device, sc)
    o = O.OracleScene(sc)
    o_img, o_rad, o_st = o.render()
    _, o_rad64, _ = o.render(double=True)
    try:
        for cfg in ((128, 0, 20, 0), (128, 0, 24, abi.RT_TRAVERSAL_PACKET_PRIMARY)):
            _set_config(device, cfg)
            img, rad, st = host.render(device, sc, gpu_scene=gs)
            assert st["status"] == 0
            assert _counts(st) == _counts(o_st), cfg
            e32 = float(np.abs(rad[..., :3] - o_rad[..., :3]).max())
            e64 = float(np.abs(rad[..., :3] - o_rad64[..., :3]).max())
            assert e32 <= RADIANCE_TOL and e64 <= RADIANCE_TOL, (cfg, e32, e64)
            assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1, cfg
    finally:
        _set_config(device, (128, 0, 20, 0))


@pytest.fixture(scope="module")
def level9():
    m = scenes.precision_mesh(level=9)
    sc = scenes.single_mesh_scene(m)
    return sc, O.OracleScene(sc)


@pytest.mark.parametrize("flags", [abi.RT_BUILD_PREFER_FAST_TRACE, Q], ids=["fp32", "quantized"])
def test_precision_mesh_level9_sample_bit_exact(device, level9, flags):
    host = _host()
    sc, o = level9
    assert sc.models[0].triangle_count == 10_485_760
    rays = scenes.random_rays(4 << 20, PRECISION_RAY_SEED, 30.0)[::41][:100_000]
    gs = host.GpuScene(device, sc, blas_flags=flags)
    assert gs.models[0].blas.info(device).node_bytes == (96 if flags & abi.RT_BUILD_QUANTIZED_NODES else 256)
    g = host.trace_ray_buffer(device, gs, rays, with_models=False)
    ref, _ = o.trace(rays, with_models=False)
    same = (g.view(np.uint32).reshape(len(g), -1) == ref.view(np.uint32).reshape(len(ref), -1)).all(axis=1)
    assert same.all(), f"{int((~same).sum())} of {len(g)} hits differ, e.g. {np.nonzero(~same)[0][:5]}"
    assert (g["instance_id"] != 0xFFFFFFFF).sum() > 20_000


def test_batch_64_scenes_quantized_batched_equal_plain_and_oracle(device):
    import torch
    from concurrent.futures import ThreadPoolExecutor

    host = _host()
    scs = scenes.batch_scenes(64)

    def frames(flags):
        out = []
        for sc in scs:
            g = host.GpuScene(device, sc, own_textures=True, blas_flags=flags)
            fr = host.PerFrameResources(device, g, sc.width, sc.height, radiance=True)
            fr.write_uniforms(sc.uniforms)
            out.append(fr)
        return out

    plain = frames(abi.RT_BUILD_PREFER_FAST_TRACE)
    quant = frames(Q)
    # the plain path: one rt_cmd_trace_rays per scene, each scene's textures bound into the context
    for fr, sc in zip(plain, scs):
        fr.gpu_scene.bind_textures()
        fr.record(sc.max_trace_depth, sc.shadow_ray_count)
    # the quantised + batched path: all 64 in one batched call, per lane and with camera-ray packets
    items = [host.batch_scene(fr, sc.max_trace_depth, sc.shadow_ray_count) for fr, sc in zip(quant, scs)]
    try:
        for cfg in ((128, 0, 20, 0), (256, 0, 20, abi.RT_TRAVERSAL_PACKET_PRIMARY)):
            _set_config(device, cfg)
            for fr in quant:
                fr.image.zero_()
            device.read_stats(reset=True)
            host.trace_batch(device, items)
            st = device.read_stats(reset=True)
            assert st["status"] == 0
            for k, (a, b) in enumerate(zip(plain, quant)):
                assert torch.equal(a.image, b.image), (cfg, k)
                assert torch.equal(a.radiance, b.radiance), (cfg, k)
    finally:
        _set_config(device, (128, 0, 20, 0))
    rad = [fr.radiance.cpu().numpy() for fr in quant]
    with ThreadPoolExecutor(max_workers=O.default_threads()) as ex:
        oracles = list(ex.map(O.OracleScene, scs))
    worst32 = worst64 = 0.0
    for k, (sc, o) in enumerate(zip(scs, oracles)):
        _, r32, _ = o.render()
        _, r64, _ = o.render(double=True)
        e32 = float(np.abs(rad[k][..., :3] - r32[..., :3]).max())
        e64 = float(np.abs(rad[k][..., :3] - r64[..., :3]).max())
        assert e32 <= RADIANCE_TOL and e64 <= RADIANCE_TOL, (k, sc.width, sc.height, e32, e64)
        worst32, worst64 = max(worst32, e32), max(worst64, e64)
    print(f"64 batch scenes: worst radiance error {worst32:.2e} vs FP32 oracle, {worst64:.2e} vs FP64 oracle")
