"""rt_cmd_trace_rays_batched: several scenes in one set of persistent launches.

Each scene keeps its own TLAS, uniforms, texture table, size, trace depth and
shadow-ray count; every output must be identical, byte for byte, to what
rt_cmd_trace_rays renders for that scene alone (same kernels, same arithmetic,
only the ray lists are shared), and one scene is also checked against the
oracle.  A CUDA graph capture of a batched call replays to the same images.
"""
import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu


def _host():
    from rtgallery import host

    return host


def _frames(device, specs):
    """specs: (scene, depth, shadows); returns [(frame, depth, shadows)]."""
    host = _host()
    out = []
    for sc, depth, shadows in specs:
        gs = host.GpuScene(device, sc, own_textures=True)
        fr = host.PerFrameResources(device, gs, sc.width, sc.height, radiance=True)
        fr.write_uniforms(sc.uniforms)
        out.append((fr, depth, shadows))
    return out


def _specs():
    return [
        (scenes.scene_small(96, 64), 1, 1),
        (scenes.scene_gallery(160, 100), 3, 2),
        (scenes.scene_full(3, 200, 120), 2, 4),
        (scenes.scene_small(33, 17), 2, 0),
        (scenes.scene_gallery(64, 40), 2, 8),
    ]


def _alone(device, frames):
    """Each frame rendered by its own rt_cmd_trace_rays call (its textures bound
    into the context's table first)."""
    import torch

    host = _host()
    imgs = []
    for fr, depth, shadows in frames:
        host.ImageManager(device).push_images(fr.gpu_scene.scene.textures)
        fr.image.zero_()
        fr.radiance.zero_()
        fr.record(depth, shadows)
        torch.cuda.synchronize()
        imgs.append((fr.image.clone(), fr.radiance.clone()))
    return imgs


def test_batch_matches_individual_frames(device):
    import torch

    host = _host()
    frames = _frames(device, _specs())
    alone = _alone(device, frames)
    device.read_stats(reset=True)
    for fr, _, _ in frames:
        fr.image.zero_()
        fr.radiance.zero_()
    host.trace_batch(device, [host.batch_scene(fr, d, s) for fr, d, s in frames], abi.RT_TRACE_FLAG_COLLECT_STATS)
    torch.cuda.synchronize()
    st = device.read_stats(reset=True)
    assert st["status"] == 0
    for k, ((fr, d, s), (img, rad)) in enumerate(zip(frames, alone)):
        assert torch.equal(fr.image, img), f"scene {k}: image differs from its own launch"
        assert torch.equal(fr.radiance, rad), f"scene {k}: radiance differs from its own launch"
    # the traversal counts add up to the oracle's for every scene
    want = 0
    for (fr, d, s) in frames:
        sc = fr.gpu_scene.scene
        _, _, o_st = O.OracleScene(sc).render(max_trace_depth=d, shadow_ray_count=s)
        want += o_st["traversals"]
    assert st["traversals"] == want


@pytest.mark.parametrize("lane_bounces", [False, True])
def test_packet_traversal_matches_per_lane(device, lane_bounces):
    """Both ray lists as warp packets over a batch of five scenes (mirrors,
    a portal, alpha-clipped geometry, 0 to 8 shadow rays; shadow-list
    chunks that straddle two scenes split into sub-packets; mirror / portal
    continuations as sub-packets or one per lane): every image and radiance
    is bit-identical to the per-lane render of the scene alone, and the
    traversal count is the oracle's."""
    import ctypes as C

    import torch

    host = _host()
    frames = _frames(device, _specs())
    alone = _alone(device, frames)
    pl = abi.RT_TRAVERSAL_PACKET_PRIMARY | abi.RT_TRAVERSAL_PACKET_SHADOW
    cfg = abi.RtTraversalConfig(128, 0, 20, pl | (abi.RT_TRAVERSAL_PACKET_LANE_BOUNCES if lane_bounces else 0))
    default = abi.RtTraversalConfig()
    device.check(device.lib.rt_ctx_get_traversal_config(device.ctx, C.byref(default)))
    try:
        device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(cfg)))
        for fr, _, _ in frames:
            fr.image.zero_()
            fr.radiance.zero_()
        device.read_stats(reset=True)
        host.trace_batch(device, [host.batch_scene(fr, d, s) for fr, d, s in frames])
        torch.cuda.synchronize()
        st = device.read_stats(reset=True)
    finally:
        device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(default)))
    assert st["status"] == 0
    for k, ((fr, d, s), (img, rad)) in enumerate(zip(frames, alone)):
        assert torch.equal(fr.image, img), f"scene {k}: packet image differs"
        assert torch.equal(fr.radiance, rad), f"scene {k}: packet radiance differs"
    want = sum(O.OracleScene(fr.gpu_scene.scene).render(max_trace_depth=d, shadow_ray_count=s)[2]["traversals"]
               for fr, d, s in frames)
    assert st["traversals"] == want


def test_batch_scene_matches_oracle(device):
    import torch

    host = _host()
    sc = scenes.scene_gallery(120, 80)
    other = scenes.scene_full(1, 64, 48)
    frames = _frames(device, [(other, 2, 4), (sc, 3, 2), (other, 1, 1)])
    host.trace_batch(device, [host.batch_scene(fr, d, s) for fr, d, s in frames])
    torch.cuda.synchronize()
    o_img, o_rad, _ = O.OracleScene(sc).render(max_trace_depth=3, shadow_ray_count=2)
    rad = frames[1][0].radiance.cpu().numpy()
    img = frames[1][0].image.cpu().numpy()
    assert np.abs(rad - o_rad).max() <= 1e-3
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1


def test_batch_graph_replay(device):
    import torch

    host = _host()
    frames = _frames(device, _specs()[:3])
    batch = [host.batch_scene(fr, d, s) for fr, d, s in frames]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        host.trace_batch(device, batch, stream=stream)  # sizes the stream's workspace outside the capture
    stream.synchronize()
    direct = [fr.image.clone() for fr, _, _ in frames]
    for fr, _, _ in frames:
        fr.image.zero_()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        host.trace_batch(device, batch, stream=stream)
    for _ in range(2):
        for fr, _, _ in frames:
            fr.image.zero_()
        g.replay()
        torch.cuda.synchronize()
        for k, (fr, _, _) in enumerate(frames):
            assert torch.equal(fr.image, direct[k]), f"scene {k} differs after graph replay"


def test_batch_into_pinned_host_images(device):
    """Uniform blocks read from one shared device array and images written by
    the output kernel straight into pinned host buffers: the same bytes as the
    device images, for a direct call and a graph replay."""
    import ctypes as C

    import torch

    host = _host()
    frames = _frames(device, _specs()[:4])
    host.trace_batch(device, [host.batch_scene(fr, d, s) for fr, d, s in frames])
    torch.cuda.synchronize()
    want = [fr.image.cpu() for fr, _, _ in frames]
    usz = C.sizeof(abi.RtUniforms)
    uni = torch.from_numpy(np.concatenate(
        [np.frombuffer(bytes(fr.gpu_scene.scene.uniforms), np.uint8) for fr, _, _ in frames])).cuda()
    out = [torch.zeros_like(fr.image, device="cpu").pin_memory() for fr, _, _ in frames]
    batch = [host.batch_scene(fr, d, s, uniforms_address=uni.data_ptr() + k * usz, image_address=out[k].data_ptr())
             for k, (fr, d, s) in enumerate(frames)]
    host.trace_batch(device, batch)
    torch.cuda.synchronize()
    for k in range(len(frames)):
        assert torch.equal(out[k], want[k]), f"scene {k}: pinned host image differs"
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        host.trace_batch(device, batch, stream=stream)
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        host.trace_batch(device, batch, stream=stream)
    for t in out:
        t.zero_()
    g.replay()
    torch.cuda.synchronize()
    for k in range(len(frames)):
        assert torch.equal(out[k], want[k]), f"scene {k}: pinned host image differs after graph replay"


def test_batch_rejects_bad_scenes(device):
    host = _host()
    frames = _frames(device, _specs()[:2])
    good = [host.batch_scene(fr, d, s) for fr, d, s in frames]
    bad = host.batch_scene(frames[0][0], 1, 1)
    bad.texture_count = abi.RT_MAX_BOUND_IMAGES + 1
    with pytest.raises(abi.RtError) as e:
        host.trace_batch(device, [good[0], bad])
    assert e.value.status == abi.RT_ERR_INVALID
    bad = host.batch_scene(frames[0][0], 0, 1)
    with pytest.raises(abi.RtError):
        host.trace_batch(device, [bad, good[1]])
    host.trace_batch(device, [])  # an empty batch is a no-op
    host.trace_batch(device, good)  # and a good batch still works after the rejected ones


def _images(frames):
    return [fr.image.clone() for fr, _, _ in frames]


def test_every_traversal_config_gives_identical_images(device):
    import ctypes as C

    import torch

    host = _host()
    frames = _frames(device, _specs()[:3])
    batch = [host.batch_scene(fr, d, s) for fr, d, s in frames]
    host.trace_batch(device, batch)
    torch.cuda.synchronize()
    ref = _images(frames)
    ref_rad = [fr.radiance.clone() for fr, _, _ in frames]
    default = abi.RtTraversalConfig()
    device.check(device.lib.rt_ctx_get_traversal_config(device.ctx, C.byref(default)))
    assert default.as_tuple() == (128, 0, 20, 0)
    # every per-lane launch shape (both lists per lane), then every packet choice on each block size
    configs = [(block, depth, wait, 0) for block in (64, 128, 256) for depth in (0, 16, 24, 32) for wait in (0, 20, 32)]
    configs += [(block, 16, 20, pl) for block in (64, 128, 256) for pl in (1, 2, 3, 5, 7)]
    try:
        for cfg in configs:
            c = abi.RtTraversalConfig(*cfg)
            device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(c)))
            for fr, _, _ in frames:
                fr.image.zero_()
                fr.radiance.zero_()
            host.trace_batch(device, batch)
            torch.cuda.synchronize()
            for k, (fr, _, _) in enumerate(frames):
                assert torch.equal(fr.image, ref[k]), (cfg, k)
                assert torch.equal(fr.radiance, ref_rad[k]), (cfg, k)  # bit-identical radiance: same hits
    finally:
        device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(default)))
    for bad in ((96, 0, 20, 0), (128, 8, 20, 0), (128, 0, 33, 0), (128, 0, 20, 8)):
        with pytest.raises(abi.RtError) as e:
            device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(abi.RtTraversalConfig(*bad))))
        assert e.value.status == abi.RT_ERR_UNSUPPORTED


def test_autotune_picks_a_built_config(device):
    import ctypes as C

    import torch

    host = _host()
    frames = _frames(device, _specs()[:2])
    batch = [host.batch_scene(fr, d, s) for fr, d, s in frames]
    arr = (abi.RtBatchScene * len(batch))(*batch)
    host.trace_batch(device, batch)
    torch.cuda.synchronize()
    ref = _images(frames)
    default = abi.RtTraversalConfig()
    device.check(device.lib.rt_ctx_get_traversal_config(device.ctx, C.byref(default)))
    rep = abi.RtAutotuneReport()
    try:
        device.check(device.lib.rt_ctx_autotune(device.ctx, arr, len(batch), None, 1, host.Device.stream_handle(),
                                                C.byref(rep)))
        # 36 per-lane launch shapes, then the 5 packet choices on the fastest shape
        assert rep.count == 41 and rep.best < rep.count
        cfgs = [rep.configs[i].as_tuple() for i in range(rep.count)]
        assert all(c[3] == 0 for c in cfgs[:36]) and (128, 0, 20, 0) in cfgs[:36]
        assert sorted(c[3] for c in cfgs[36:]) == [1, 2, 3, 5, 7] and len({c[:3] for c in cfgs[36:]}) == 1
        ms = [rep.median_ms[i] for i in range(rep.count)]
        assert all(m > 0 for m in ms) and ms[rep.best] == min(ms)
        chosen = abi.RtTraversalConfig()
        device.check(device.lib.rt_ctx_get_traversal_config(device.ctx, C.byref(chosen)))
        assert chosen.as_tuple() == rep.configs[rep.best].as_tuple()
        for fr, _, _ in frames:
            fr.image.zero_()
        host.trace_batch(device, batch)
        torch.cuda.synchronize()
        for k, (fr, _, _) in enumerate(frames):
            assert torch.equal(fr.image, ref[k])
    finally:
        device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(default)))


def test_batch_of_more_scenes_than_one_setup_chunk(device):
    """70 scenes: their records are written by two setup launches (64 + 6);
    every image equals the same scene rendered as a batch of one."""
    import torch

    host = _host()
    base = scenes.scene_small(24, 16)
    gs = host.GpuScene(device, base, own_textures=True)
    rng = scenes.Pcg32(77, 0x70)
    frames = []
    for i in range(70):
        w, h = 8 + int(rng.next_u32() % 40), 4 + int(rng.next_u32() % 30)
        fr = host.PerFrameResources(device, gs, w, h)
        fr.write_uniforms(scenes.random_view_uniforms(rng, w, h, frame=i, distance=(6.0, 12.0), height_range=(2.0, 6.0)))
        frames.append((fr, 1 + i % 3, i % 5))
    for fr, d, s in frames:
        host.trace_batch(device, [host.batch_scene(fr, d, s)])
    torch.cuda.synchronize()
    alone = _images(frames)
    for fr, _, _ in frames:
        fr.image.zero_()
    host.trace_batch(device, [host.batch_scene(fr, d, s) for fr, d, s in frames])
    torch.cuda.synchronize()
    for k, (fr, _, _) in enumerate(frames):
        assert torch.equal(fr.image, alone[k]), f"scene {k}"
    assert sum(int(a.float().sum() > 0) for a in alone) > 60
