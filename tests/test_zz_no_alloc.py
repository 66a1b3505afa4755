"""The allocation-free BLAS build (rt_cmd_build_blas_static_scratch).

Some callers may not allocate device memory when they build a BLAS: their
device memory belongs to another allocator that hands this library only
the destination buffer, or their frame loop has a memory budget fixed at
start-up.  For them the library keeps one fixed scratch array on each
device.  This file checks, through the C ABI, that two builds in a row with
that array give the same structure as the caller-scratch build of the same
geometry: identical header (node and triangle counts, bounds, status) and
bit-identical hits for every ray (hit IDs are compared exactly everywhere in
this test suite).  The second build runs over the first build's leftovers
in the shared array.  It also checks that a geometry too big for the array
is rejected before anything is queued.

This file is collected last on purpose (its name sorts last).
"""
import ctypes as C

import numpy as np
import pytest

from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu


def _geometry_array(gm):
    arr = (abi.RtGeometryTriangles * len(gm.index_buffers))()
    for i, (ib, g) in enumerate(zip(gm.index_buffers, gm._model.geometries)):
        arr[i].vertex_address = gm.position_buffer.data_ptr()
        arr[i].index_address = ib.data_ptr()
        arr[i].vertex_stride = 12
        arr[i].max_vertex = len(gm._model.positions) - 1
        arr[i].primitive_count = len(g.indices)
        arr[i].flags = abi.RT_GEOMETRY_OPAQUE if g.opaque else 0
    return arr


def _info(device, addr):
    inf = abi.RtAccelerationStructureInfo()
    device.check(device.lib.rt_get_acceleration_structure_info(addr, C.byref(inf), None))
    return inf


def _scene_for(model: scenes.Model):
    base = scenes.scene_small(8, 8)
    inst = scenes.instance_records(scenes.affine(np.eye(3), [0, 0, 0])[None], [0], [0], 0)
    return scenes.Scene([model], base.textures, inst, base.uniforms, 8, 8)


def _trace_with_blas(device, gs, blas_buffer, blas_size, rays):
    """Rebuilds the scene's TLAS over `blas_buffer` and traces `rays`."""
    import torch

    from rtgallery import host

    inst = gs.scene.instances.copy()
    inst["blas"] = blas_buffer.data_ptr()
    buf = host.Device.upload(inst)
    tlas = host.AccelerationStructure.build_tlas(device, buf, len(inst), gs.scratch)
    saved = gs.tlas
    gs.tlas = tlas
    try:
        hits = host.trace_ray_buffer(device, gs, rays, with_models=False)
    finally:
        gs.tlas = saved
    torch.cuda.synchronize()
    return hits


@pytest.mark.parametrize("call", [0, 1])
def test_static_scratch_build_matches_caller_scratch_build(device, call):
    import torch

    from rtgallery import host

    # two calls in a row with different geometry: a displaced sphere, then an
    # alpha-clipped fence plus a torus in one BLAS (two geometries)
    if call == 0:
        pos, nrm, uv, idx = scenes.uv_sphere(128, 64, 1.0, 0.05, 7)
        model = scenes.Model(pos, nrm, uv, [scenes.Geometry(idx, True)], "sphere")
    else:
        tp, tn, tuv, ti = scenes.torus(1.0, 0.35, 64, 32)
        fp, fn, fuv, fi = scenes.quad_grid(200, 1, 10.0, 2.0, 25.0, 1.0)
        pos = np.concatenate([tp, fp])
        model = scenes.Model(pos, np.concatenate([tn, fn]), np.concatenate([tuv, fuv]),
                             [scenes.Geometry(ti, True), scenes.Geometry(fi + len(tp), False)], "torus+fence")
    gs = host.GpuScene(device, _scene_for(model))
    gm = gs.models[0]
    gm._model = model
    geo = _geometry_array(gm)
    reference = gm.blas  # built by rt_cmd_build_blas with caller scratch

    sizes = abi.RtBuildSizes()
    # sizes for the flags of the build (PREFER_FAST_TRACE builds take more nodes and scratch)
    device.check(device.lib.rt_get_blas_build_sizes(geo, len(geo), abi.RT_BUILD_PREFER_FAST_TRACE, C.byref(sizes)))
    assert sizes.build_scratch_size <= abi.RT_STATIC_SCRATCH_BYTES
    dst = host.Device.alloc(sizes.acceleration_structure_size)
    torch.cuda.synchronize()
    device.check(device.lib.rt_cmd_build_blas_static_scratch(device.ctx, geo, len(geo), abi.RT_BUILD_PREFER_FAST_TRACE,
                                                             dst.data_ptr(), sizes.acceleration_structure_size,
                                                             host.Device.stream_handle()))
    torch.cuda.synchronize()
    a, b = _info(device, reference.device_address()), _info(device, dst.data_ptr())
    assert b.status == abi.RT_OK
    assert (b.node_count, b.primitive_count, b.tree_depth, b.total_size) == \
        (a.node_count, a.primitive_count, a.tree_depth, a.total_size)
    assert list(b.bounds_lo) == list(a.bounds_lo) and list(b.bounds_hi) == list(a.bounds_hi)
    # the triangle records (leaf order) are byte-identical
    hdr = dst[:512].cpu().numpy().view(np.uint64)
    prims_off = int(hdr[6])  # header: 8 x u32, total_size, nodes_offset, prims_offset
    assert int(hdr[5]) == 512 and prims_off % 256 == 0
    n = a.primitive_count
    ref_tris = reference.buffer[prims_off:prims_off + 48 * n].cpu().numpy()
    new_tris = dst[prims_off:prims_off + 48 * n].cpu().numpy()
    assert (ref_tris == new_tris).all()
    # and every ray hits the same thing through either BLAS, bit for bit
    rays = scenes.random_rays(50000, 21 + call, 8.0)
    rays["tmax"] = 1e4
    h_ref = _trace_with_blas(device, gs, reference.buffer, reference.size, rays)
    h_new = _trace_with_blas(device, gs, dst, sizes.acceleration_structure_size, rays)
    assert (h_ref.view(np.uint32) == h_new.view(np.uint32)).all()
    assert (h_ref["instance_id"] != 0xFFFFFFFF).sum() > 1000


def test_static_scratch_rejects_oversized_geometry(device):
    geo = (abi.RtGeometryTriangles * 1)()
    geo[0].vertex_address = 4096
    geo[0].vertex_stride = 12
    geo[0].primitive_count = 2_000_000
    geo[0].max_vertex = 6_000_000
    sizes = abi.RtBuildSizes()
    device.check(device.lib.rt_get_blas_build_sizes(geo, 1, 0, C.byref(sizes)))
    r = device.lib.rt_cmd_build_blas_static_scratch(device.ctx, geo, 1, 0, 1 << 20, sizes.acceleration_structure_size,
                                                    None)
    assert r == abi.RT_ERR_TOO_LARGE
    assert b"static scratch" in device.lib.rt_last_error_string()


def test_static_scratch_rejects_quantized_nodes(device):
    """The static-scratch build writes FP32 nodes only: a request for 8-bit
    quantised nodes is refused before anything is queued."""
    geo = (abi.RtGeometryTriangles * 1)()
    geo[0].vertex_address = 4096
    geo[0].vertex_stride = 12
    geo[0].primitive_count = 100
    geo[0].max_vertex = 300
    flags = abi.RT_BUILD_PREFER_FAST_TRACE | abi.RT_BUILD_QUANTIZED_NODES
    r = device.lib.rt_cmd_build_blas_static_scratch(device.ctx, geo, 1, flags, 1 << 20, 1 << 20, None)
    assert r == abi.RT_ERR_UNSUPPORTED
    assert b"QUANTIZED" in device.lib.rt_last_error_string()
