"""ctypes mirror of include/rtcore.h and the loader for librtcore.so.

The structs keep the reference's byte layouts (shared-structs/src/lib.rs,
src/gpu_structs.rs); ``check_layouts()`` asserts every size and offset the
header asserts.  ``load_library()`` fails loudly when the CUDA library is
missing: there is no CPU fallback anywhere in the product path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

RT_OK = 0
RT_ERR_INVALID = 1
RT_ERR_OOM = 2
RT_ERR_STACK_OVERFLOW = 3
RT_ERR_TIMEOUT = 4
RT_ERR_CUDA = 5
RT_ERR_UNSUPPORTED = 6
RT_ERR_TOO_LARGE = 7
RT_ERR_BAD_AS = 8

RT_MAX_BOUND_IMAGES = 128
RT_MAX_BLAS_GEOMETRIES = 128
RT_MAX_HIT_GROUPS = 8
RT_AS_ALIGNMENT = 256
RT_STATIC_SCRATCH_BYTES = 64 << 20

RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE = 0x1
RT_INSTANCE_TRIANGLE_FLIP_FACING = 0x2
RT_INSTANCE_FORCE_OPAQUE = 0x4
RT_INSTANCE_FORCE_NO_OPAQUE = 0x8
RT_GEOMETRY_OPAQUE = 0x1
RT_GEOMETRY_NO_DUPLICATE_ANY_HIT_INVOCATION = 0x2
RT_BUILD_ALLOW_UPDATE = 0x1
RT_BUILD_ALLOW_COMPACTION = 0x2
RT_BUILD_PREFER_FAST_TRACE = 0x4
RT_BUILD_PREFER_FAST_BUILD = 0x8
RT_BUILD_LOW_MEMORY = 0x10
RT_BUILD_QUANTIZED_NODES = 0x100
RT_BUILD_EXT_NODE_WIDTH_4 = 0x200
RT_RAY_FLAG_NONE = 0x0
RT_RAY_FLAG_OPAQUE = 0x1
RT_RAY_FLAG_NO_OPAQUE = 0x2
RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT = 0x4
RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER = 0x8
RT_RAY_FLAG_CULL_BACK_FACING = 0x10
RT_RAY_FLAG_CULL_FRONT_FACING = 0x20
RT_RAY_FLAG_CULL_OPAQUE = 0x40
RT_RAY_FLAG_CULL_NO_OPAQUE = 0x80
RT_RAY_FLAG_EXT_COLLECT_STATS = 0x100
RT_COPY_MODE_CLONE = 0
RT_COPY_MODE_COMPACT = 1
RT_FORMAT_R8G8B8A8_UNORM = 37
RT_FORMAT_R8G8B8A8_SRGB = 43
RT_FORMAT_R32G32B32A32_SFLOAT = 109
RT_FILTER_NEAREST = 0
RT_FILTER_LINEAR = 1
RT_PROGRAM_NONE = 0
RT_PROGRAM_CLOSEST_HIT_TEXTURED = 1
RT_PROGRAM_CLOSEST_HIT_MIRROR = 2
RT_PROGRAM_CLOSEST_HIT_PORTAL = 3
RT_PROGRAM_ANY_HIT_ALPHA_CLIP = 1
RT_TRACE_FLAG_COLLECT_STATS = 0x1
RT_TRACE_FLAG_LAMBERT_DIFFUSE = 0x2
RT_TRACE_FLAG_KERNEL_TIMINGS = 0x4
RT_CTX_THREADSAFE = 0x1
RT_FN_V_SMITH_GGX_CORRELATED = 0
RT_FN_D_GGX = 1
RT_FN_LINEAR_TO_SRGB = 2
RT_FN_HEATMAP = 3
RT_FN_SINCOS = 4
RT_FN_BRDF = 5
RT_FN_WATERTIGHT = 6
# per-function (input floats, output floats) per element
RT_FN_STRIDES = {0: (3, 1), 1: (2, 1), 2: (1, 1), 3: (1, 3), 4: (1, 2), 5: (16, 3), 6: (16, 4)}

# hit groups of the reference (src/main.rs:46-50 HitShader, :289-305)
HIT_SHADER_TEXTURED = 0
HIT_SHADER_MIRROR = 1
HIT_SHADER_PORTAL = 2


class RtUniforms(C.Structure):
    _fields_ = [
        ("view_inverse", C.c_float * 16),
        ("proj_inverse", C.c_float * 16),
        ("sun_dir", C.c_float * 3),
        ("_padding0", C.c_uint32),
        ("sun_radius", C.c_float),
        ("blue_noise_texture_index", C.c_uint32),
        ("ggx_lut_texture_index", C.c_uint32),
        ("frame_index", C.c_uint32),
        ("show_heatmap", C.c_uint8),
        ("_padding1", C.c_uint8 * 15),
    ]


class RtModelInfo(C.Structure):
    _fields_ = [
        ("position_buffer_address", C.c_uint64),
        ("normal_buffer_address", C.c_uint64),
        ("uv_buffer_address", C.c_uint64),
        ("geometry_info_address", C.c_uint64),
    ]


class RtGeometryImages(C.Structure):
    _fields_ = [
        ("diffuse_image_index", C.c_uint32),
        ("metallic_roughness_image_index", C.c_uint32),
        ("normal_map_image_index", C.c_int32),
        ("_padding", C.c_uint32),
    ]


class RtGeometryInfo(C.Structure):
    _fields_ = [("index_buffer_address", C.c_uint64), ("images", RtGeometryImages)]


class RtPushConstantBufferAddresses(C.Structure):
    _fields_ = [("model_info", C.c_uint64), ("uniforms", C.c_uint64), ("acceleration_structure", C.c_uint64)]


class RtAccelerationStructureInstance(C.Structure):
    _fields_ = [
        ("transform", (C.c_float * 4) * 3),
        ("instance_custom_index_and_mask", C.c_uint32),
        ("instance_shader_binding_table_record_offset_and_flags", C.c_uint32),
        ("acceleration_structure_reference", C.c_uint64),
    ]


class RtGeometryTriangles(C.Structure):
    _fields_ = [
        ("vertex_address", C.c_uint64),
        ("index_address", C.c_uint64),
        ("vertex_stride", C.c_uint32),
        ("max_vertex", C.c_uint32),
        ("primitive_count", C.c_uint32),
        ("flags", C.c_uint32),
    ]


class RtBuildSizes(C.Structure):
    _fields_ = [
        ("acceleration_structure_size", C.c_uint64),
        ("build_scratch_size", C.c_uint64),
        ("update_scratch_size", C.c_uint64),
    ]


class RtAccelerationStructureInfo(C.Structure):
    _fields_ = [
        ("type", C.c_uint32),
        ("build_flags", C.c_uint32),
        ("node_count", C.c_uint32),
        ("primitive_count", C.c_uint32),
        ("node_bytes", C.c_uint32),
        ("tree_depth", C.c_uint32),
        ("total_size", C.c_uint64),
        ("compacted_size", C.c_uint64),
        ("bounds_lo", C.c_float * 3),
        ("bounds_hi", C.c_float * 3),
        ("status", C.c_uint32),
        ("_padding", C.c_uint32),
    ]


class RtTextureDesc(C.Structure):
    _fields_ = [
        ("address", C.c_uint64),
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("row_pitch", C.c_uint32),
        ("format", C.c_uint32),
        ("filter", C.c_uint32),
        ("_padding", C.c_uint32),
    ]


class RtHitGroup(C.Structure):
    _fields_ = [("closest_hit", C.c_uint32), ("any_hit", C.c_uint32)]


class RtShaderBindingTable(C.Structure):
    _fields_ = [("hit_group_count", C.c_uint32), ("_padding", C.c_uint32), ("hit_groups", RtHitGroup * RT_MAX_HIT_GROUPS)]


class RtTraceRaysDesc(C.Structure):
    _fields_ = [
        ("width", C.c_uint32),
        ("height", C.c_uint32),
        ("max_trace_depth", C.c_uint32),
        ("shadow_ray_count", C.c_uint32),
        ("flags", C.c_uint32),
        ("_padding", C.c_uint32),
        ("image_address", C.c_uint64),
        ("radiance_address", C.c_uint64),
    ]


class RtBatchScene(C.Structure):
    _fields_ = [
        ("push", RtPushConstantBufferAddresses),
        ("texture_count", C.c_uint32),
        ("_padding", C.c_uint32),
        ("texture_table", C.c_uint64),
        ("desc", RtTraceRaysDesc),
    ]


RT_MAX_BATCH_SCENES = 65536


RT_TRAVERSAL_PACKET_PRIMARY = 0x1
RT_TRAVERSAL_PACKET_SHADOW = 0x2
RT_TRAVERSAL_PACKET_LANE_BOUNCES = 0x4


class RtTraversalConfig(C.Structure):
    _fields_ = [("block_size", C.c_uint32), ("shared_stack_depth", C.c_uint32), ("leaf_wait", C.c_uint32),
                ("packet_lists", C.c_uint32)]

    def as_tuple(self) -> tuple:
        return (self.block_size, self.shared_stack_depth, self.leaf_wait, self.packet_lists)


RT_AUTOTUNE_MAX_CONFIGS = 64


class RtAutotuneReport(C.Structure):
    _fields_ = [("count", C.c_uint32), ("best", C.c_uint32),
                ("configs", RtTraversalConfig * RT_AUTOTUNE_MAX_CONFIGS),
                ("median_ms", C.c_float * RT_AUTOTUNE_MAX_CONFIGS)]


class RtServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_batch_requests", C.c_uint32),
                ("max_batch_pixels", C.c_uint32), ("max_in_flight", C.c_uint32),
                ("max_batch_shadow_rays", C.c_uint32)]


class RtServeScene(C.Structure):
    _fields_ = [("acceleration_structure", C.c_uint64), ("model_info", C.c_uint64), ("texture_table", C.c_uint64),
                ("texture_count", C.c_uint32), ("_padding", C.c_uint32), ("resident_bytes", C.c_uint64)]


class RtServeRequest(C.Structure):
    _fields_ = [("uniforms", RtUniforms), ("scene", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32),
                ("max_trace_depth", C.c_uint32), ("shadow_ray_count", C.c_uint32), ("flags", C.c_uint32),
                ("image_device", C.c_uint64), ("image_host", C.c_uint64), ("_padding", C.c_uint32 * 2)]


RT_SERVE_PENDING, RT_SERVE_DONE, RT_SERVE_REJECTED = 0, 1, 2


class RtServeResult(C.Structure):
    _fields_ = [("state", C.c_uint32), ("status", C.c_uint32), ("batch", C.c_uint32), ("batch_requests", C.c_uint32),
                ("queue_ms", C.c_double), ("latency_ms", C.c_double)]


class RtServeStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("rejected", C.c_uint64),
                ("batches", C.c_uint64), ("resident_bytes", C.c_uint64), ("peak_bytes", C.c_uint64),
                ("budget_bytes", C.c_uint64), ("pixels", C.c_uint64)]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_}


# include/rtassets.h
class RtGlbInfo(C.Structure):
    _fields_ = [("vertex_count", C.c_uint32), ("geometry_count", C.c_uint32), ("image_count", C.c_uint32),
                ("primitive_count", C.c_uint32), ("triangle_count", C.c_uint64)]


class RtGlbGeometry(C.Structure):
    _fields_ = [("index_count", C.c_uint32), ("opaque", C.c_uint32), ("diffuse_image", C.c_int32),
                ("metallic_roughness_image", C.c_int32), ("normal_map_image", C.c_int32), ("_padding", C.c_uint32)]


class RtGlbImage(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("format", C.c_uint32), ("filter", C.c_uint32),
                ("byte_size", C.c_uint64)]


class RtRay(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("tmin", C.c_float), ("direction", C.c_float * 3), ("tmax", C.c_float)]


class RtHit(C.Structure):
    _fields_ = [
        ("t", C.c_float),
        ("u", C.c_float),
        ("v", C.c_float),
        ("instance_id", C.c_uint32),
        ("instance_custom_index", C.c_uint32),
        ("geometry_index", C.c_uint32),
        ("primitive_index", C.c_uint32),
        ("hit_kind", C.c_uint32),
    ]


class RtTraceTimings(C.Structure):
    _fields_ = [
        ("total_ms", C.c_float),
        ("trace_ms", C.c_float),
        ("closest_ms", C.c_float),
        ("shadow_ms", C.c_float),
        ("shade_ms", C.c_float),
        ("other_ms", C.c_float),
        ("trace_launches", C.c_uint32),
        ("_padding", C.c_uint32),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("_")}


class RtStats(C.Structure):
    _fields_ = [
        ("traversals", C.c_uint64),
        ("primary_rays", C.c_uint64),
        ("secondary_rays", C.c_uint64),
        ("shadow_rays", C.c_uint64),
        ("nodes_visited", C.c_uint64),
        ("triangles_tested", C.c_uint64),
        ("instances_visited", C.c_uint64),
        ("status", C.c_uint32),
        ("_padding", C.c_uint32),
        ("quantized_nodes_visited", C.c_uint64),
    ]

    def as_dict(self) -> dict:
        return {f: getattr(self, f) for f, _ in self._fields_ if not f.startswith("_")}


# numpy views of the same records (for arrays of them)
INSTANCE_DTYPE = np.dtype(
    [("transform", "<f4", (3, 4)), ("custom_index_and_mask", "<u4"), ("sbt_offset_and_flags", "<u4"), ("blas", "<u8")]
)
RAY_DTYPE = np.dtype([("origin", "<f4", (3,)), ("tmin", "<f4"), ("direction", "<f4", (3,)), ("tmax", "<f4")])
HIT_DTYPE = np.dtype(
    [("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("instance_id", "<u4"), ("instance_custom_index", "<u4"),
     ("geometry_index", "<u4"), ("primitive_index", "<u4"), ("hit_kind", "<u4")]
)
MODEL_INFO_DTYPE = np.dtype([("position", "<u8"), ("normal", "<u8"), ("uv", "<u8"), ("geometry_info", "<u8")])
GEOMETRY_INFO_DTYPE = np.dtype(
    [("index_buffer", "<u8"), ("diffuse", "<u4"), ("metallic_roughness", "<u4"), ("normal_map", "<i4"), ("_pad", "<u4")]
)

EXPORTED_FUNCTIONS = {
    "rt_ctx_create": (C.c_int32, [C.c_uint32, C.POINTER(C.c_void_p)]),
    "rt_ctx_destroy": (C.c_int32, [C.c_void_p]),
    "rt_ctx_set_texture": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(RtTextureDesc)]),
    "rt_ctx_read_stats": (C.c_int32, [C.c_void_p, C.POINTER(RtStats), C.c_int32, C.c_void_p]),
    "rt_ctx_read_trace_timings": (C.c_int32, [C.c_void_p, C.POINTER(RtTraceTimings)]),
    "rt_last_error_string": (C.c_char_p, []),
    "rt_version_string": (C.c_char_p, []),
    "rt_kernel_launch_count": (C.c_uint64, []),
    "rt_get_blas_build_sizes": (C.c_int32, [C.POINTER(RtGeometryTriangles), C.c_uint32, C.c_uint32, C.POINTER(RtBuildSizes)]),
    "rt_cmd_build_blas": (C.c_int32, [C.c_void_p, C.POINTER(RtGeometryTriangles), C.c_uint32, C.c_uint32, C.c_uint64,
                                       C.c_uint64, C.c_uint64, C.c_uint64, C.c_void_p]),
    "rt_cmd_build_blas_static_scratch": (C.c_int32, [C.c_void_p, C.POINTER(RtGeometryTriangles), C.c_uint32,
                                                      C.c_uint32, C.c_uint64, C.c_uint64, C.c_void_p]),
    "rt_get_tlas_build_sizes": (C.c_int32, [C.c_uint32, C.c_uint32, C.POINTER(RtBuildSizes)]),
    "rt_cmd_build_tlas": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint64, C.c_uint64,
                                       C.c_uint64, C.c_uint64, C.c_void_p]),
    "rt_cmd_update_tlas": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint64,
                                        C.c_uint64, C.c_uint64, C.c_void_p]),
    "rt_cmd_copy_acceleration_structure": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint32,
                                                        C.c_void_p]),
    "rt_get_acceleration_structure_info": (C.c_int32, [C.c_uint64, C.POINTER(RtAccelerationStructureInfo), C.c_void_p]),
    "rt_get_acceleration_structure_device_address": (C.c_uint64, [C.c_uint64]),
    "rt_cmd_trace_rays": (C.c_int32, [C.c_void_p, C.POINTER(RtPushConstantBufferAddresses),
                                       C.POINTER(RtShaderBindingTable), C.POINTER(RtTraceRaysDesc), C.c_void_p]),
    "rt_cmd_trace_rays_batched": (C.c_int32, [C.c_void_p, C.POINTER(RtBatchScene), C.c_uint32,
                                               C.POINTER(RtShaderBindingTable), C.c_uint32, C.c_void_p]),
    "rt_ctx_set_traversal_config": (C.c_int32, [C.c_void_p, C.POINTER(RtTraversalConfig)]),
    "rt_ctx_get_traversal_config": (C.c_int32, [C.c_void_p, C.POINTER(RtTraversalConfig)]),
    "rt_trace_ray_buffer_host": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(RtPushConstantBufferAddresses),
                                              C.POINTER(RtShaderBindingTable), C.c_uint32, C.c_uint32, C.c_uint32,
                                              C.c_void_p, C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p]),
    "rt_server_create": (C.c_int32, [C.c_void_p, C.POINTER(RtServerConfig), C.POINTER(C.c_void_p)]),
    "rt_server_destroy": (C.c_int32, [C.c_void_p]),
    "rt_server_add_scene": (C.c_int32, [C.c_void_p, C.POINTER(RtServeScene), C.POINTER(C.c_uint32)]),
    "rt_server_submit": (C.c_int32, [C.c_void_p, C.POINTER(RtServeRequest), C.POINTER(C.c_uint64)]),
    "rt_server_wait": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_uint32, C.POINTER(RtServeResult)]),
    "rt_server_stats": (C.c_int32, [C.c_void_p, C.POINTER(RtServeStats)]),
    "rt_png_decode_rgba8": (C.c_int32, [C.c_void_p, C.c_uint64, C.c_void_p, C.c_uint64, C.POINTER(C.c_uint32),
                                         C.POINTER(C.c_uint32)]),
    "rt_glb_load": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(C.c_void_p)]),
    "rt_glb_info": (C.c_int32, [C.c_void_p, C.POINTER(RtGlbInfo)]),
    "rt_glb_read_vertices": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "rt_glb_read_geometry": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(RtGlbGeometry), C.c_void_p,
                                          C.c_uint64]),
    "rt_glb_read_image": (C.c_int32, [C.c_void_p, C.c_uint32, C.POINTER(RtGlbImage), C.c_void_p, C.c_uint64]),
    "rt_glb_destroy": (C.c_int32, [C.c_void_p]),
    "rt_ctx_autotune": (C.c_int32, [C.c_void_p, C.POINTER(RtBatchScene), C.c_uint32, C.POINTER(RtShaderBindingTable),
                                     C.c_uint32, C.c_void_p, C.POINTER(RtAutotuneReport)]),
    "rt_cmd_trace_ray_buffer": (C.c_int32, [C.c_void_p, C.c_uint64, C.POINTER(RtPushConstantBufferAddresses),
                                             C.POINTER(RtShaderBindingTable), C.c_uint32, C.c_uint32, C.c_uint32,
                                             C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p]),
    "rt_debug_eval": (C.c_int32, [C.c_uint32, C.c_uint64, C.c_uint64, C.c_uint32, C.c_void_p]),
    "rt_debug_sort_pairs": (C.c_int32, [C.c_uint64, C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint64,
                                        C.POINTER(C.c_uint64), C.c_void_p]),
}


class RtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"rtcore error {status}: {message}")
        self.status = status


_LIB = None


def library_path() -> Path:
    return Path(__file__).resolve().parent / "_build" / "librtcore.so"


def load_library(path: str | Path | None = None) -> C.CDLL:
    """Loads librtcore.so; raises if it has not been built (no fallback)."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else library_path()
    if not p.exists():
        raise RuntimeError(
            f"librtcore.so not found at {p}; build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(the CUDA library is required; there is no CPU fallback)"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in EXPORTED_FUNCTIONS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _LIB = lib
    return lib


def check(lib: C.CDLL, status: int) -> None:
    if status != RT_OK:
        raise RtError(status, lib.rt_last_error_string().decode(errors="replace"))


def reference_sbt() -> RtShaderBindingTable:
    """The reference's program table: hit groups {textured, mirror, portal},
    each with the alpha-clip any-hit (src/main.rs:289-305)."""
    s = RtShaderBindingTable()
    s.hit_group_count = 3
    progs = [RT_PROGRAM_CLOSEST_HIT_TEXTURED, RT_PROGRAM_CLOSEST_HIT_MIRROR, RT_PROGRAM_CLOSEST_HIT_PORTAL]
    for i, p in enumerate(progs):
        s.hit_groups[i].closest_hit = p
        s.hit_groups[i].any_hit = RT_PROGRAM_ANY_HIT_ALPHA_CLIP
    return s


def check_layouts() -> None:
    """The byte layouts the reference's Vulkan path relies on."""
    assert C.sizeof(RtUniforms) == 176
    assert RtUniforms.proj_inverse.offset == 64
    assert RtUniforms.sun_dir.offset == 128
    assert RtUniforms.sun_radius.offset == 144
    assert RtUniforms.blue_noise_texture_index.offset == 148
    assert RtUniforms.ggx_lut_texture_index.offset == 152
    assert RtUniforms.frame_index.offset == 156
    assert RtUniforms.show_heatmap.offset == 160
    assert C.sizeof(RtModelInfo) == 32
    assert C.sizeof(RtGeometryInfo) == 24
    assert C.sizeof(RtPushConstantBufferAddresses) == 24
    assert C.sizeof(RtAccelerationStructureInstance) == 64
    assert RtAccelerationStructureInstance.instance_custom_index_and_mask.offset == 48
    assert RtAccelerationStructureInstance.acceleration_structure_reference.offset == 56
    assert INSTANCE_DTYPE.itemsize == 64
    assert MODEL_INFO_DTYPE.itemsize == 32
    assert GEOMETRY_INFO_DTYPE.itemsize == 24
    assert RAY_DTYPE.itemsize == C.sizeof(RtRay) == 32
    assert HIT_DTYPE.itemsize == C.sizeof(RtHit) == 32
    assert C.sizeof(RtGeometryTriangles) == 32
    assert C.sizeof(RtTextureDesc) == 32
    assert C.sizeof(RtShaderBindingTable) == 72
    assert C.sizeof(RtTraceRaysDesc) == 40
    assert C.sizeof(RtTraceTimings) == 32
    assert C.sizeof(RtBatchScene) == 80 and RtBatchScene.desc.offset == 40
    assert C.sizeof(RtTraversalConfig) == 16
    assert C.sizeof(RtAutotuneReport) == 8 + 64 * 16 + 64 * 4
    assert C.sizeof(RtServerConfig) == 24 and C.sizeof(RtServeScene) == 40
    assert C.sizeof(RtServeRequest) == 224 and RtServeRequest.image_device.offset == 200
    assert C.sizeof(RtServeResult) == 32 and C.sizeof(RtServeStats) == 64
    assert C.sizeof(RtGlbInfo) == C.sizeof(RtGlbGeometry) == C.sizeof(RtGlbImage) == 24
