"""GPU parity: librtcore.so (through the C ABI) against the CPU oracle.

Bit-exact: hit/miss, instance / geometry / primitive IDs, t, u, v for every
ray, the number of rays each program traced.  Tolerance: linear radiance
max-abs 1e-3 (pow/sqrt rounding differs between CUDA and libm), RGBA8 image
1 LSB.  Everything runs on identical inputs generated in-process.
"""
import ctypes as C
import json
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from rtgallery import abi, scenes

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"
RADIANCE_TOL = 1e-3


def _host():
    from rtgallery import host

    return host


def _eval_gpu(device, fn, inputs, count, out_stride):
    import torch

    inp = torch.from_numpy(np.ascontiguousarray(inputs, np.float32).reshape(-1)).cuda()
    out = torch.zeros(count * out_stride, dtype=torch.float32, device="cuda")
    device.check(device.lib.rt_debug_eval(fn, inp.data_ptr(), out.data_ptr(), count, None))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_device_functions_match_oracle(device):
    rng = np.random.default_rng(5)
    n = 4096
    # sincos: bit-exact (the same operation sequence on both sides)
    x = (rng.random(n) * 40 - 20).astype(np.float32)
    g = _eval_gpu(device, abi.RT_FN_SINCOS, x, n, 2)
    o = O.debug_eval(abi.RT_FN_SINCOS, x, n, 2)
    assert (g.view(np.uint32) == o.view(np.uint32)).all()
    # watertight triangle test: bit-exact hit flag, t, u, v
    p = rng.normal(size=(n, 16)).astype(np.float32)
    p[:, 15] = 0.0
    g = _eval_gpu(device, abi.RT_FN_WATERTIGHT, p, n, 4)
    o = O.debug_eval(abi.RT_FN_WATERTIGHT, p, n, 4)
    assert (g.view(np.uint32) == o.view(np.uint32)).all()
    assert (o[0::4] != 0).sum() > 100
    # colour functions: tolerance
    for fn, stride_in, stride_out, gen in [
        (abi.RT_FN_V_SMITH_GGX_CORRELATED, 3, 1, lambda: rng.random((n, 3)) * [1, 1, 1] + [1e-3, 0, 0.01]),
        (abi.RT_FN_D_GGX, 2, 1, lambda: rng.random((n, 2)) * [1, 1] + [0, 0.05]),
        (abi.RT_FN_LINEAR_TO_SRGB, 1, 1, lambda: rng.random(n) * 1.2),
        (abi.RT_FN_HEATMAP, 1, 3, lambda: rng.random(n) * 1.1 - 0.05),
    ]:
        inp = np.asarray(gen(), np.float32)
        g = _eval_gpu(device, fn, inp, n, stride_out)
        o = O.debug_eval(fn, inp, n, stride_out)
        np.testing.assert_allclose(g, o, rtol=2e-6, atol=2e-6)
    bp = np.zeros((n, 16), np.float32)
    for k, sl in enumerate([slice(0, 3), slice(3, 6), slice(6, 9)]):
        v = rng.normal(size=(n, 3))
        bp[:, sl] = v / np.linalg.norm(v, axis=1, keepdims=True)
    bp[:, 9] = rng.random(n) * 0.9 + 0.1
    bp[:, 10:13] = rng.random((n, 3))
    bp[:, 13] = rng.random(n)
    bp[:, 14] = rng.random(n)
    g = _eval_gpu(device, abi.RT_FN_BRDF, bp, n, 3)
    o = O.debug_eval(abi.RT_FN_BRDF, bp, n, 3)
    np.testing.assert_allclose(g, o, rtol=1e-5, atol=1e-5)


def test_ggx_division_by_zero_kat_on_device(device):
    kat = json.loads((GOLDEN / "ggx_division_by_zero.json").read_text())
    for eps in (kat["nov_epsilon_rust"], kat["nov_epsilon_glsl"]):
        g = _eval_gpu(device, abi.RT_FN_V_SMITH_GGX_CORRELATED, np.array([eps, 1.0, kat["roughness"]]), 1, 1)
        assert math.isfinite(g[0])


def _gpu_scene(device, sc):
    return _host().GpuScene(device, sc)


def _assert_hits_equal(g, o, what=""):
    same = (g.view(np.uint32).reshape(len(g), -1) == o.view(np.uint32).reshape(len(o), -1)).all(axis=1)
    if not same.all():
        bad = np.nonzero(~same)[0][:5]
        raise AssertionError(f"{what}: {int((~same).sum())} of {len(g)} hits differ, e.g. {bad}: gpu {g[bad]} "
                             f"oracle {o[bad]}")


def test_golden_small_rays(device):
    g = np.load(GOLDEN / "small_rays.npz")
    tor = scenes.Model(g["torus_positions"], g["torus_normals"], g["torus_uvs"],
                       [scenes.Geometry(g["torus_indices"], True, scenes.TEX_DIFFUSE_A, scenes.TEX_MR_DEFAULT)])
    gnd = scenes.Model(g["ground_positions"], g["ground_normals"], g["ground_uvs"],
                       [scenes.Geometry(g["ground_indices"], True, scenes.TEX_DIFFUSE_B, scenes.TEX_MR_DEFAULT)])
    base = scenes.scene_small(64, 32)
    sc = scenes.Scene([tor, gnd], base.textures, g["instances"], base.uniforms, 64, 32, 3, 1)
    gs = _gpu_scene(device, sc)
    hits = _host().trace_ray_buffer(device, gs, g["rays"])
    _assert_hits_equal(hits, g["hits"], "golden small_rays")


SCENES = {
    "small": lambda: scenes.scene_small(128, 128),
    "gallery": lambda: scenes.scene_gallery(160, 100),
    "full": lambda: scenes.scene_full(0, 192, 108),
}

RAY_FLAG_CASES = [
    abi.RT_RAY_FLAG_NONE,
    abi.RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT | abi.RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER,
    abi.RT_RAY_FLAG_OPAQUE,
    abi.RT_RAY_FLAG_CULL_BACK_FACING,
    abi.RT_RAY_FLAG_CULL_OPAQUE,
]


@pytest.mark.parametrize("name", list(SCENES))
def test_ray_buffer_bit_exact(device, name):
    sc = SCENES[name]()
    gs = _gpu_scene(device, sc)
    o = O.OracleScene(sc)
    box = 60.0 if name == "full" else 16.0
    rays = scenes.random_rays(20000, 31, box)
    rays["tmax"] = 1e4
    for flags in RAY_FLAG_CASES:
        g = _host().trace_ray_buffer(device, gs, rays, ray_flags=flags)
        h, _ = o.trace(rays, ray_flags=flags)
        if flags & abi.RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT:
            # any accepted hit ends the ray: only hit/miss is defined
            assert ((g["instance_id"] == 0xFFFFFFFF) == (h["instance_id"] == 0xFFFFFFFF)).all()
        else:
            _assert_hits_equal(g, h, f"{name} flags {flags:#x}")
        if flags == abi.RT_RAY_FLAG_NONE:
            assert (h["instance_id"] != 0xFFFFFFFF).sum() > 100
    # cull mask: instances whose mask misses the ray's are skipped
    g = _host().trace_ray_buffer(device, gs, rays, cull_mask=0x00)
    assert (g["instance_id"] == 0xFFFFFFFF).all()


@pytest.mark.parametrize("name", list(SCENES))
def test_render_matches_oracle(device, name):
    sc = SCENES[name]()
    img, rad, st = _host().render(device, sc, radiance=True)
    o_img, o_rad, o_st = O.OracleScene(sc).render()
    for k in ("traversals", "primary_rays", "secondary_rays", "shadow_rays"):
        assert st[k] == o_st[k], (k, st[k], o_st[k])
    assert st["status"] == 0
    diff = np.abs(rad - o_rad)
    assert diff.max() <= RADIANCE_TOL, diff.max()
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1


def test_normal_map_branch_matches_oracle(device):
    """closest_hit_textured.glsl:123-157: the gallery's ground names a normal
    map (RGBA8 UNORM, bilinear), so its shading takes the cotangent-frame
    branch; those pixels must match the oracle, and the branch must matter
    (without the map the oracle's radiance there differs)."""
    sc = scenes.scene_gallery(320, 200)
    assert sc.models[1].geometries[0].normal_map_image == scenes.TEX_NORMAL_MAP
    img, rad, st = _host().render(device, sc, radiance=True)
    o_img, o_rad, _ = O.OracleScene(sc).render()
    plain = scenes.scene_gallery(320, 200)
    plain.models[1].geometries[0].normal_map_image = -1
    _, p_rad, _ = O.OracleScene(plain).render()
    mapped = np.abs(o_rad - p_rad)[..., :3].max(-1) > 1e-3
    assert mapped.sum() > 5000, int(mapped.sum())
    assert np.abs(rad - o_rad)[mapped].max() <= RADIANCE_TOL
    assert np.abs(img.astype(int) - o_img.astype(int)).max() <= 1


def test_tlas_update_matches_rebuild(device):
    """DefaultScene::update + write_resources (src/scene.rs:163-204): move one
    instance, refit the TLAS in place, then compare with the oracle."""
    import torch

    host = _host()
    sc = scenes.scene_gallery(96, 64)
    gs = _gpu_scene(device, sc)
    inst = sc.instances.copy()
    rng = scenes.Pcg32(99)
    for i in range(4, len(inst), 3):
        inst["transform"][i] = scenes.affine(scenes.rot_y(rng.uniform() * 6.28), [rng.uniform_range(-5, 5), 1.0,
                                            rng.uniform_range(-5, 5)], 0.4)
    patched = gs.patch_instances(inst)
    gs.instances_buffer.copy_(torch.from_numpy(patched.view(np.uint8).reshape(-1)).cuda())
    gs.tlas.update_tlas(device, gs.instances_buffer, len(inst), gs.scratch)
    info = gs.tlas.info(device)
    assert info.status == 0
    o = O.OracleScene(sc)
    o.set_instances(inst)
    rays = scenes.random_rays(20000, 3, 14.0)
    rays["tmax"] = 1e4
    _assert_hits_equal(host.trace_ray_buffer(device, gs, rays), o.trace(rays)[0], "after in-place update")
    # out-of-place update into a new TLAS, and a full rebuild, agree as well
    gs.tlas.rebuild_tlas(device, gs.instances_buffer, len(inst), gs.scratch)
    _assert_hits_equal(host.trace_ray_buffer(device, gs, rays), o.trace(rays)[0], "after rebuild")


def test_clone_and_compact_copies(device):
    host = _host()
    sc = scenes.scene_gallery(64, 48)
    gs = _gpu_scene(device, sc)
    rays = scenes.random_rays(5000, 4, 14.0)
    rays["tmax"] = 1e4
    ref = host.trace_ray_buffer(device, gs, rays)
    clone = gs.tlas.clone(device, "clone")
    info = gs.tlas.info(device)
    compact = host.Device.alloc(info.compacted_size)
    device.check(device.lib.rt_cmd_copy_acceleration_structure(device.ctx, gs.tlas.device_address(),
                                                               compact.data_ptr(), info.compacted_size,
                                                               abi.RT_COPY_MODE_COMPACT, None))
    for tlas_buf in (clone.buffer, compact):
        saved = gs.tlas
        gs.tlas = host.AccelerationStructure(tlas_buf, info.total_size, saved.flags, 1)
        _assert_hits_equal(host.trace_ray_buffer(device, gs, rays), ref, "copy")
        gs.tlas = saved
    cinfo = abi.RtAccelerationStructureInfo()
    device.check(device.lib.rt_get_acceleration_structure_info(compact.data_ptr(), C.byref(cinfo), None))
    assert cinfo.total_size == info.compacted_size <= info.total_size
    assert cinfo.node_count == info.node_count


def _one_model_scene(positions, indices, instances, opaque=True):
    m = scenes.Model(np.asarray(positions, np.float32), np.zeros((len(positions), 3), np.float32),
                     np.zeros((len(positions), 2), np.float32),
                     [scenes.Geometry(np.asarray(indices, np.uint32).reshape(-1, 3), opaque, 0, 4)])
    base = scenes.scene_small(8, 8)
    return scenes.Scene([m], base.textures, instances, base.uniforms, 8, 8)


def test_edge_cases(device):
    host = _host()
    rays = scenes.random_rays(4000, 8, 6.0)
    rays["tmax"] = 1e4
    tri = [[0, 0, 0], [1, 0, 0], [0, 1, 0]]
    ident = scenes.affine(np.eye(3), [0, 0, 0])
    cases = {
        "one triangle": (tri, [0, 1, 2], scenes.instance_records(ident[None], [0], [0], 0)),
        "empty blas": (np.zeros((0, 3)), np.zeros((0,)), scenes.instance_records(ident[None], [0], [0], 0)),
        "no instances": (tri, [0, 1, 2], scenes.instance_records(np.zeros((0, 3, 4)), [], [], 0)),
        "singular transform": (tri, [0, 1, 2], scenes.instance_records(np.zeros((1, 3, 4)), [0], [0], 0)),
        "masked instance": (tri, [0, 1, 2], scenes.instance_records(ident[None], [0], [0], 0, mask=0)),
        "degenerate + duplicate tris": ([[0, 0, 0], [1, 0, 0], [2, 0, 0], [0, 1, 0]],
                                        [0, 1, 2, 0, 1, 3, 0, 1, 3, 0, 1, 3],
                                        scenes.instance_records(np.stack([ident, scenes.affine(np.eye(3), [0, 0, 0.5])]),
                                                                [0, 0], [0, 0], 0)),
    }
    for name, (pos, idx, inst) in cases.items():
        sc = _one_model_scene(np.asarray(pos).reshape(-1, 3), idx, inst)
        gs = _gpu_scene(device, sc)
        g = host.trace_ray_buffer(device, gs, rays, with_models=False)
        o, _ = O.OracleScene(sc).trace(rays, with_models=False)
        _assert_hits_equal(g, o, name)
        if name in ("empty blas", "no instances", "singular transform", "masked instance"):
            assert (g["instance_id"] == 0xFFFFFFFF).all(), name


def test_instance_boxes_under_shear_and_nonuniform_scale(device):
    """An instance's TLAS box is its transformed BLAS box cut to the box of
    its transformed bounding sphere (an ellipsoid under a general affine
    map).  Sheared, non-uniformly scaled, mirrored and far-translated
    instances of a torus and a displaced sphere, rays grazing them: every hit
    equals the oracle's."""
    host = _host()
    rng = scenes.Pcg32(77, 3)
    tor = scenes.torus(1.0, 0.35, 48, 24)
    sph = scenes.uv_sphere(64, 32, 1.0, 0.05, 5)
    models = [scenes.Model(p, n, u, [scenes.Geometry(i, True)], nm) for (p, n, u, i), nm in ((tor, "torus"), (sph, "sphere"))]
    xf, mdl = [], []
    for k in range(24):
        m = scenes.random_rotation(rng) @ np.diag([rng.uniform_range(0.2, 3.0) * (-1 if k % 5 == 0 else 1),
                                                    rng.uniform_range(0.2, 3.0), rng.uniform_range(0.2, 3.0)])
        m = m @ np.array([[1.0, rng.uniform_range(-1, 1), 0.0], [0.0, 1.0, rng.uniform_range(-1, 1)], [0.0, 0.0, 1.0]])
        t = [rng.uniform_range(-6, 6), rng.uniform_range(-6, 6), rng.uniform_range(-6, 6)]
        if k == 23:  # far away, about 2 units across
            t = [3.0e4, -2.0e4, 1.0e4]
            m = 2.0 * scenes.random_rotation(rng) @ np.array([[1.0, 0.3, 0.0], [0.0, 1.0, 0.0], [0.0, 0.0, 1.0]])
        a = np.zeros((3, 4))
        a[:, :3], a[:, 3] = m, t
        xf.append(a)
        mdl.append(k % 2)
    inst = scenes.instance_records(np.array(xf), np.array(mdl), np.array(mdl), 0,
                                   flags=abi.RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE)
    sc = scenes.Scene(models, {}, inst, scenes.make_uniforms(np.eye(4).reshape(-1), np.eye(4).reshape(-1), (0, 1, 0),
                                                              0.0, 0, 0), 8, 8)
    gs = _gpu_scene(device, sc)
    o = O.OracleScene(sc)
    rays = scenes.random_rays(60000, 13, 9.0)
    rays["tmax"] = 1e4
    # plus rays aimed at the far instance's centre
    far = scenes.random_rays(2000, 14, 2.0)
    far["origin"] += np.float32([3.0e4, -2.0e4, 1.0e4]) + np.float32([0, 0, -20.0])
    far["direction"] = np.float32([0, 0, 1]) + 0.05 * far["direction"]
    far["direction"] /= np.linalg.norm(far["direction"], axis=1, keepdims=True)
    far["tmax"] = 1e4
    for name, rr in (("near", rays), ("far", far)):
        g = host.trace_ray_buffer(device, gs, rr, with_models=False)
        h, _ = o.trace(rr, with_models=False)
        _assert_hits_equal(g, h, name)
        assert (h["instance_id"] != 0xFFFFFFFF).sum() > 50, name


def test_invalid_vertex_index_reports_status(device):
    sc = _one_model_scene([[0, 0, 0], [1, 0, 0], [0, 1, 0]], [0, 1, 7],
                          scenes.instance_records(scenes.affine(np.eye(3), [0, 0, 0])[None], [0], [0], 0))
    gs = _gpu_scene(device, sc)
    info = gs.models[0].blas.info(device)
    assert info.status == abi.RT_ERR_INVALID


def test_host_validation_rejects_bad_launches(device):
    host = _host()
    sc = scenes.scene_small(16, 16)
    gs = _gpu_scene(device, sc)
    fr = host.PerFrameResources(device, gs, 16, 16)
    fr.write_uniforms(sc.uniforms)
    with pytest.raises(abi.RtError) as e:
        fr.record(0, 1)
    assert e.value.status == abi.RT_ERR_INVALID
    s = abi.RtShaderBindingTable()
    s.hit_group_count = 9
    with pytest.raises(abi.RtError):
        fr.record(1, 1, sbt=s)
    fr.record(1, 1)  # a valid launch still works after the rejected ones


def test_mid_size_mesh_bit_exact(device):
    """A 655,360-triangle displaced icosphere (level 7, bisected) with 100k
    random rays: every hit bit-exact."""
    host = _host()
    m = scenes.precision_mesh(level=7)
    sc = scenes.single_mesh_scene(m)
    gs = _gpu_scene(device, sc)
    rays = scenes.random_rays(100000, 12, 30.0)
    g = host.trace_ray_buffer(device, gs, rays, with_models=False)
    o, _ = O.OracleScene(sc).trace(rays, with_models=False)
    _assert_hits_equal(g, o, "icosphere l6")
    assert (g["instance_id"] != 0xFFFFFFFF).mean() > 0.2


@pytest.mark.parametrize("blas_flags", [abi.RT_BUILD_PREFER_FAST_BUILD, 0,
                                        abi.RT_BUILD_PREFER_FAST_BUILD | abi.RT_BUILD_QUANTIZED_NODES],
                         ids=["fast_build", "no_preference", "fast_build_quantized"])
def test_karras_hierarchy_builds_bit_exact(device, blas_flags):
    """BLASes and TLASes built without PREFER_FAST_TRACE take the Karras LBVH
    hierarchy instead of PLOC: every hit of the three parity scenes and of the
    655,360-triangle mesh is still bit-exact against the oracle, and a render
    matches it within the radiance tolerance."""
    host = _host()
    tlas_flags = (blas_flags & ~abi.RT_BUILD_QUANTIZED_NODES) | abi.RT_BUILD_ALLOW_UPDATE
    for name, make in SCENES.items():
        sc = make()
        gs = host.GpuScene(device, sc, blas_flags=blas_flags, tlas_flags=tlas_flags)
        assert all(m.blas.info(device).build_flags & abi.RT_BUILD_PREFER_FAST_TRACE == 0 for m in gs.models)
        o = O.OracleScene(sc)
        rays = scenes.random_rays(20000, 37, 60.0 if name == "full" else 16.0)
        rays["tmax"] = 1e4
        _assert_hits_equal(host.trace_ray_buffer(device, gs, rays), o.trace(rays)[0], f"{name} karras")
        img, rad, st = host.render(device, sc, radiance=True, gpu_scene=gs)
        o_img, o_rad, o_st = o.render()
        assert st["status"] == 0 and st["traversals"] == o_st["traversals"]
        assert np.abs(rad - o_rad).max() <= RADIANCE_TOL
    m = scenes.precision_mesh(level=7)
    sc = scenes.single_mesh_scene(m)
    gs = host.GpuScene(device, sc, blas_flags=blas_flags, tlas_flags=tlas_flags)
    rays = scenes.random_rays(100000, 13, 30.0)
    g = host.trace_ray_buffer(device, gs, rays, with_models=False)
    _assert_hits_equal(g, O.OracleScene(sc).trace(rays, with_models=False)[0], "icosphere l7 karras")
    assert (g["instance_id"] != 0xFFFFFFFF).mean() > 0.2


def test_host_buffer_query_matches_device_query(device):
    """rt_trace_ray_buffer_host returns the same hits as
    rt_cmd_trace_ray_buffer: pinned buffers traced in place (chunk_rays 0),
    staged chunks on two streams with a ragged last chunk, and pageable
    buffers (chunk_rays 0 falls back to the staged copies)."""
    import torch

    host = _host()
    sc = scenes.scene_gallery(64, 48)
    gs = _gpu_scene(device, sc)
    rays = scenes.random_rays(20011, 17, 14.0)
    rays["tmax"] = 1e4
    ref = host.trace_ray_buffer(device, gs, rays)
    rays_h = torch.from_numpy(rays.view(np.uint8).copy()).pin_memory()
    push = gs.push_constants(0)

    def query(rays_ptr, hits_ptr, chunk):
        device.check(device.lib.rt_trace_ray_buffer_host(device.ctx, gs.tlas.device_address(), C.byref(push), None,
                                                         0, 0xFF, 0, rays_ptr, len(rays), hits_ptr, chunk,
                                                         host.Device.stream_handle()))
        torch.cuda.synchronize()

    for chunk in (3000, 0, 20011):
        hits_h = torch.zeros(len(rays) * abi.HIT_DTYPE.itemsize, dtype=torch.uint8).pin_memory()
        query(rays_h.data_ptr(), hits_h.data_ptr(), chunk)
        _assert_hits_equal(hits_h.numpy().view(abi.HIT_DTYPE), ref, f"host query, chunk {chunk}")
    rays_p = np.ascontiguousarray(rays)
    hits_p = np.zeros(len(rays), abi.HIT_DTYPE)
    query(rays_p.ctypes.data, hits_p.ctypes.data, 0)
    _assert_hits_equal(hits_p, ref, "pageable host query")


def test_double_buffered_frame_loop_matches_serial_frames(device):
    """host.FrameLoop (two frames in flight on two streams, each with its own
    TLAS rebuilt from that frame's instances) renders every frame exactly as
    a serial loop over one frame resource does."""
    import torch

    host = _host()
    W, H = 160, 96
    models = scenes.full_scene_models()
    sc0 = scenes.scene_full(0, W, H, models=models)
    gs = _gpu_scene(device, sc0)
    frames = [host.Device.upload(gs.patch_instances(scenes.full_scene_instances(k))) for k in range(6)]
    unis = [host.Device.upload(np.frombuffer(bytes(scenes.scene_full(k, W, H, models=models).uniforms), np.uint8))
            for k in range(6)]
    serial = host.PerFrameResources(device, gs, W, H, clone_tlas=True)
    ref = []
    for k in range(6):
        serial.tlas.rebuild_tlas(device, frames[k], gs.num_instances, gs.scratch)
        serial.uniforms_buffer.copy_(unis[k])
        serial.record(2, 4)
        torch.cuda.synchronize()
        ref.append(serial.image.clone())
    loop = host.FrameLoop(device, gs, W, H, frames_in_flight=2)
    for direct in (False, True):  # image copied after the frame, or written into the pinned buffer
        got = [torch.zeros_like(r, device="cpu").pin_memory() for r in ref]
        loop.begin()
        for k in range(6):
            loop.record(k, 2, 4, instances=frames[k], uniforms_dev=unis[k], image_host=got[k], image_direct=direct)
        loop.end()
        torch.cuda.synchronize()
        for k in range(6):
            assert torch.equal(got[k], ref[k].cpu()), f"frame {k}, direct {direct}"
    assert len({int(r.float().sum()) for r in ref}) > 1  # the frames differ
