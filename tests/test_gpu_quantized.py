"""BLASes built with RT_BUILD_QUANTIZED_NODES (8-bit child boxes).

A quantised node stores each child box as bytes on a per-node power-of-two
grid, rounded outwards with a quarter grid step to spare, so the boxes only
grow: traversal may visit more nodes, never fewer, and the closest hit is
decided by the same watertight triangle test and the same (t, instance,
geometry, primitive) order.  Every hit must therefore be bit-identical to
the FP32-node build and to the oracle.  Rays from far away take the exact
plane decode instead of the fast one; both are covered.  The same holds for
structures collapsed to at most 4 children per node.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu
Q = abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_QUANTIZED_NODES


def _host():
    from rtgallery import host

    return host


def _same(g, o, what):
    same = (g.view(np.uint32).reshape(len(g), -1) == o.view(np.uint32).reshape(len(o), -1)).all(axis=1)
    assert same.all(), f"{what}: {int((~same).sum())} of {len(g)} hits differ, e.g. {np.nonzero(~same)[0][:5]}"


def _aimed_rays(count, seed, distance, radius):
    """Origins on a sphere of `distance`, aimed at points within `radius` of
    the centre (the exact-decode case once distance / grid step > 2^19)."""
    rng = scenes.Pcg32(seed, 0x51)
    u = rng.uniform_array(count * 6).reshape(count, 6)
    def on_sphere(a, b):
        z = 2.0 * a - 1.0
        r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
        return np.stack([r * np.cos(2 * np.pi * b), r * np.sin(2 * np.pi * b), z], 1)
    org = on_sphere(u[:, 0], u[:, 1]) * distance
    tgt = on_sphere(u[:, 2], u[:, 3]) * radius * u[:, 4:5]
    d = tgt - org
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros(count, abi.RAY_DTYPE)
    rays["origin"] = org.astype(np.float32)
    rays["direction"] = d.astype(np.float32)
    rays["tmin"] = 0.0
    rays["tmax"] = np.inf
    return rays


SCENES = {
    "small": lambda: scenes.scene_small(64, 64),
    "gallery": lambda: scenes.scene_gallery(96, 64),
    "full": lambda: scenes.scene_full(0, 96, 54),
}


@pytest.mark.parametrize("name", list(SCENES))
def test_quantized_blas_hits_bit_exact(device, name):
    host = _host()
    sc = SCENES[name]()
    gq = host.GpuScene(device, sc, blas_flags=Q)
    gf = host.GpuScene(device, sc)
    for m in gq.models:
        inf = m.blas.info(device)
        assert inf.status == abi.RT_OK and inf.node_bytes == 96 and inf.build_flags & abi.RT_BUILD_QUANTIZED_NODES
    for m in gf.models:
        assert m.blas.info(device).node_bytes == 256
    o = O.OracleScene(sc)
    rays = scenes.random_rays(20000, 41, 60.0 if name == "full" else 16.0)
    rays["tmax"] = 1e4
    for flags in (abi.RT_RAY_FLAG_NONE, abi.RT_RAY_FLAG_OPAQUE, abi.RT_RAY_FLAG_CULL_BACK_FACING,
                  abi.RT_RAY_FLAG_CULL_OPAQUE, abi.RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT):
        q = host.trace_ray_buffer(device, gq, rays, ray_flags=flags)
        h, _ = o.trace(rays, ray_flags=flags)
        if flags & abi.RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT:
            assert ((q["instance_id"] == 0xFFFFFFFF) == (h["instance_id"] == 0xFFFFFFFF)).all()
            continue
        _same(q, h, f"{name} quantised vs oracle, flags {flags:#x}")
        _same(q, host.trace_ray_buffer(device, gf, rays, ray_flags=flags), f"{name} quantised vs fp32")


def test_quantized_render_matches_oracle(device):
    host = _host()
    sc = scenes.scene_gallery(96, 64)
    gq = host.GpuScene(device, sc, blas_flags=Q)
    img, rad, st = host.render(device, sc, radiance=True, gpu_scene=gq)
    o_img, o_rad, o_st = O.OracleScene(sc).render()
    for k in ("traversals", "primary_rays", "secondary_rays", "shadow_rays"):
        assert st[k] == o_st[k], (k, st[k], o_st[k])
    assert st["status"] == 0
    assert np.abs(rad - o_rad).max() <= 1e-3
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1


@pytest.mark.parametrize("formats", ["quantised", "mixed"])
def test_quantized_scenes_render_identically_per_lane_and_as_packets(device, formats):
    """A scene of quantised BLASes (the quantised-only kernels) and one mixing
    quantised and FP32 BLASes in one TLAS (the kernels decoding both): the
    per-lane traversal and both lists as warp packets give bit-identical
    images and radiance, equal to the oracle's within its tolerance."""
    import torch

    host = _host()
    sc = scenes.scene_full(0, 96, 54)
    flags = Q if formats == "quantised" else [Q if i % 2 == 0 else abi.RT_BUILD_PREFER_FAST_TRACE
                                              for i in range(len(sc.models))]
    g = host.GpuScene(device, sc, blas_flags=flags)
    sizes = {m.blas.info(device).node_bytes for m in g.models}
    assert sizes == ({96} if formats == "quantised" else {96, 256})
    out = []
    default = abi.RtTraversalConfig()
    device.check(device.lib.rt_ctx_get_traversal_config(device.ctx, C.byref(default)))
    try:
        for packets in (0, abi.RT_TRAVERSAL_PACKET_PRIMARY | abi.RT_TRAVERSAL_PACKET_SHADOW):
            cfg = abi.RtTraversalConfig(128, 0, 20, packets)
            device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(cfg)))
            img, rad, st = host.render(device, sc, radiance=True, gpu_scene=g)
            assert st["status"] == 0
            out.append((img, rad, st["traversals"]))
    finally:
        device.check(device.lib.rt_ctx_set_traversal_config(device.ctx, C.byref(default)))
    (img0, rad0, n0), (img1, rad1, n1) = out
    assert np.array_equal(img0, img1) and np.array_equal(rad0.view(np.uint32), rad1.view(np.uint32)) and n0 == n1
    o_img, o_rad, o_st = O.OracleScene(sc).render()
    assert n0 == o_st["traversals"]
    assert np.abs(rad0 - o_rad).max() <= 1e-3
    torch.cuda.synchronize()


@pytest.mark.parametrize("distance",[30.0, 3.0e5])
def test_quantized_mesh_near_and_far_rays(device, distance):
    """655,360 triangles; rays from 30 units use the fast plane decode, rays
    from 3e5 units the exact one (the origin is over 2^19 grid steps away)."""
    host = _host()
    sc = scenes.single_mesh_scene(scenes.precision_mesh(level=7))
    gq = host.GpuScene(device, sc, blas_flags=Q)
    gf = host.GpuScene(device, sc)
    rays = _aimed_rays(60000, 17, distance, 12.0)
    q = host.trace_ray_buffer(device, gq, rays, with_models=False)
    f = host.trace_ray_buffer(device, gf, rays, with_models=False)
    _same(q, f, f"quantised vs fp32 from {distance}")
    sub = slice(0, 6000)
    o, _ = O.OracleScene(sc).trace(rays[sub], with_models=False)
    _same(q[sub], o, f"quantised vs oracle from {distance}")
    assert (q["instance_id"] != 0xFFFFFFFF).mean() > 0.5
    info_q, info_f = gq.models[0].blas.info(device), gf.models[0].blas.info(device)
    assert info_q.node_count == info_f.node_count
    assert info_q.total_size < info_f.total_size


def test_quantized_blas_clone_and_compact(device):
    import torch

    host = _host()
    sc = scenes.single_mesh_scene(scenes.precision_mesh(level=5))
    gq = host.GpuScene(device, sc, blas_flags=Q)
    rays = _aimed_rays(20000, 3, 40.0, 12.0)
    ref = host.trace_ray_buffer(device, gq, rays, with_models=False)
    blas = gq.models[0].blas
    info = blas.info(device)
    compact = host.Device.alloc(info.compacted_size)
    device.check(device.lib.rt_cmd_copy_acceleration_structure(device.ctx, blas.device_address(), compact.data_ptr(),
                                                               info.compacted_size, abi.RT_COPY_MODE_COMPACT, None))
    clone = blas.clone(device, "clone")
    torch.cuda.synchronize()
    for copy in (compact, clone.buffer):
        cinfo = abi.RtAccelerationStructureInfo()
        device.check(device.lib.rt_get_acceleration_structure_info(copy.data_ptr(), C.byref(cinfo), None))
        assert cinfo.node_bytes == 96 and cinfo.node_count == info.node_count and cinfo.status == abi.RT_OK
        inst = sc.instances.copy()
        inst["blas"] = copy.data_ptr()
        buf = host.Device.upload(inst)
        tlas = host.AccelerationStructure.build_tlas(device, buf, len(inst), gq.scratch)
        saved = gq.tlas
        gq.tlas = tlas
        try:
            _same(host.trace_ray_buffer(device, gq, rays, with_models=False), ref, "copied quantised blas")
        finally:
            gq.tlas = saved
    assert info.compacted_size <= info.total_size


def test_quantized_build_sizes_are_smaller(device):
    host = _host()
    model = scenes.precision_mesh(level=4)
    gm = host.GpuScene(device, scenes.single_mesh_scene(model)).models[0]
    geo = (abi.RtGeometryTriangles * 1)()
    geo[0].vertex_address = gm.position_buffer.data_ptr()
    geo[0].index_address = gm.index_buffers[0].data_ptr()
    geo[0].vertex_stride = 12
    geo[0].max_vertex = len(model.positions) - 1
    geo[0].primitive_count = len(model.geometries[0].indices)
    s_f, s_q = abi.RtBuildSizes(), abi.RtBuildSizes()
    device.check(device.lib.rt_get_blas_build_sizes(geo, 1, abi.RT_BUILD_PREFER_FAST_TRACE, C.byref(s_f)))
    device.check(device.lib.rt_get_blas_build_sizes(geo, 1, Q, C.byref(s_q)))
    assert s_q.acceleration_structure_size < s_f.acceleration_structure_size
    assert s_q.build_scratch_size >= s_f.build_scratch_size


W4 = abi.RT_BUILD_EXT_NODE_WIDTH_4


@pytest.mark.parametrize("name", list(SCENES))
def test_node_width_4_hits_bit_exact(device, name):
    """BLASes and TLAS collapsed to at most 4 children per node (FP32 and
    quantised): same hits as the oracle; a TLAS refit of the 4-wide TLAS too."""
    import torch

    host = _host()
    sc = SCENES[name]()
    o = O.OracleScene(sc)
    rays = scenes.random_rays(20000, 43, 60.0 if name == "full" else 16.0)
    rays["tmax"] = 1e4
    ref, _ = o.trace(rays)
    tlas_flags = abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_ALLOW_UPDATE | W4
    for blas_flags in (abi.RT_BUILD_PREFER_FAST_TRACE | W4, Q | W4):
        g = host.GpuScene(device, sc, blas_flags=blas_flags, tlas_flags=tlas_flags)
        _same(host.trace_ray_buffer(device, g, rays), ref, f"{name} width 4, blas flags {blas_flags:#x}")
        info_t = g.tlas.info(device)
        assert info_t.status == abi.RT_OK
        if len(sc.instances) > 4:
            assert info_t.tree_depth >= 2
    # refit the 4-wide TLAS after moving instances
    g = host.GpuScene(device, sc, blas_flags=abi.RT_BUILD_PREFER_FAST_TRACE | W4, tlas_flags=tlas_flags)
    inst = sc.instances.copy()
    rng = scenes.Pcg32(5, 9)
    for i in range(0, len(inst), 2):
        inst["transform"][i, :, 3] += np.array([rng.uniform_range(-1, 1), 0.5, rng.uniform_range(-1, 1)], np.float32)
    g.instances_buffer.copy_(torch.from_numpy(g.patch_instances(inst).view(np.uint8).reshape(-1)).cuda())
    g.tlas.update_tlas(device, g.instances_buffer, len(inst), g.scratch)
    assert g.tlas.info(device).status == abi.RT_OK
    o.set_instances(inst)
    _same(host.trace_ray_buffer(device, g, rays), o.trace(rays)[0], f"{name} width 4 after refit")


def test_node_width_4_render_matches_oracle(device):
    host = _host()
    sc = scenes.scene_gallery(96, 64)
    g = host.GpuScene(device, sc, blas_flags=abi.RT_BUILD_PREFER_FAST_TRACE | W4,
                      tlas_flags=abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_ALLOW_UPDATE | W4)
    img, rad, st = host.render(device, sc, radiance=True, gpu_scene=g)
    o_img, o_rad, o_st = O.OracleScene(sc).render()
    assert st["traversals"] == o_st["traversals"] and st["status"] == 0
    assert np.abs(rad - o_rad).max() <= 1e-3
