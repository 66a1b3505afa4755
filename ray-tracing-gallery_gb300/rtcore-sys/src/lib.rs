//! Raw bindings to librtcore (`include/rtcore.h`, `include/rtassets.h`): the
//! C ABI that replaces the Vulkan ray-tracing dispatch of
//! expenses/ray-tracing-gallery.
//!
//! Every struct is `#[repr(C)]` with the header's layout (the sizes are
//! checked at compile time below).  `Uniforms`, `ModelInfo`, `GeometryInfo`,
//! `PushConstantBufferAddresses` (shared-structs/src/lib.rs) and
//! `AccelerationStructureInstance` (src/gpu_structs.rs) are not redefined:
//! the host passes its own values of those types, whose layouts the header
//! keeps byte for byte.  Addresses are CUDA device pointers as `u64`;
//! `CudaStream` is a `cudaStream_t` (null = the legacy default stream).
//! Every function returns `RT_OK` (0) or an `RT_ERR_*` code, described by
//! `rt_last_error_string`.
#![allow(non_camel_case_types)]
#![no_std]

use core::ffi::{c_char, c_void};

pub type CudaStream = *mut c_void;

#[repr(C)]
pub struct rt_ctx {
    _private: [u8; 0],
}
#[repr(C)]
pub struct rt_server {
    _private: [u8; 0],
}
#[repr(C)]
pub struct rt_glb_model {
    _private: [u8; 0],
}

// ---- status codes ----
pub const RT_OK: i32 = 0;
pub const RT_ERR_INVALID: i32 = 1;
pub const RT_ERR_OOM: i32 = 2;
pub const RT_ERR_STACK_OVERFLOW: i32 = 3;
pub const RT_ERR_TIMEOUT: i32 = 4;
pub const RT_ERR_CUDA: i32 = 5;
pub const RT_ERR_UNSUPPORTED: i32 = 6;
pub const RT_ERR_TOO_LARGE: i32 = 7;
pub const RT_ERR_BAD_AS: i32 = 8;

pub const RT_MAX_BOUND_IMAGES: u32 = 128;
pub const RT_MAX_BLAS_GEOMETRIES: u32 = 128;
pub const RT_MAX_HIT_GROUPS: usize = 8;
pub const RT_AS_ALIGNMENT: u64 = 256;

// ---- flags (Vulkan values where Vulkan has them) ----
pub const RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE: u32 = 0x1;
pub const RT_INSTANCE_TRIANGLE_FLIP_FACING: u32 = 0x2;
pub const RT_INSTANCE_FORCE_OPAQUE: u32 = 0x4;
pub const RT_INSTANCE_FORCE_NO_OPAQUE: u32 = 0x8;
pub const RT_GEOMETRY_OPAQUE: u32 = 0x1;
pub const RT_GEOMETRY_NO_DUPLICATE_ANY_HIT_INVOCATION: u32 = 0x2;
pub const RT_BUILD_ALLOW_UPDATE: u32 = 0x1;
pub const RT_BUILD_ALLOW_COMPACTION: u32 = 0x2;
pub const RT_BUILD_PREFER_FAST_TRACE: u32 = 0x4;
pub const RT_BUILD_PREFER_FAST_BUILD: u32 = 0x8;
pub const RT_BUILD_LOW_MEMORY: u32 = 0x10;
pub const RT_BUILD_QUANTIZED_NODES: u32 = 0x100;
pub const RT_BUILD_EXT_NODE_WIDTH_4: u32 = 0x200;
pub const RT_RAY_FLAG_NONE: u32 = 0x0;
pub const RT_RAY_FLAG_OPAQUE: u32 = 0x1;
pub const RT_RAY_FLAG_NO_OPAQUE: u32 = 0x2;
pub const RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT: u32 = 0x4;
pub const RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER: u32 = 0x8;
pub const RT_RAY_FLAG_CULL_BACK_FACING: u32 = 0x10;
pub const RT_RAY_FLAG_CULL_FRONT_FACING: u32 = 0x20;
pub const RT_RAY_FLAG_CULL_OPAQUE: u32 = 0x40;
pub const RT_RAY_FLAG_CULL_NO_OPAQUE: u32 = 0x80;
pub const RT_RAY_FLAG_EXT_COLLECT_STATS: u32 = 0x100;
pub const RT_COPY_MODE_CLONE: u32 = 0;
pub const RT_COPY_MODE_COMPACT: u32 = 1;
pub const RT_FORMAT_R8G8B8A8_UNORM: u32 = 37;
pub const RT_FORMAT_R8G8B8A8_SRGB: u32 = 43;
pub const RT_FORMAT_R32G32B32A32_SFLOAT: u32 = 109;
pub const RT_FILTER_NEAREST: u32 = 0;
pub const RT_FILTER_LINEAR: u32 = 1;
pub const RT_PROGRAM_NONE: u32 = 0;
pub const RT_PROGRAM_CLOSEST_HIT_TEXTURED: u32 = 1;
pub const RT_PROGRAM_CLOSEST_HIT_MIRROR: u32 = 2;
pub const RT_PROGRAM_CLOSEST_HIT_PORTAL: u32 = 3;
pub const RT_PROGRAM_ANY_HIT_ALPHA_CLIP: u32 = 1;
pub const RT_TRACE_FLAG_COLLECT_STATS: u32 = 0x1;
pub const RT_TRACE_FLAG_LAMBERT_DIFFUSE: u32 = 0x2;
pub const RT_TRACE_FLAG_KERNEL_TIMINGS: u32 = 0x4;
pub const RT_CTX_THREADSAFE: u32 = 0x1;
pub const RT_STATIC_SCRATCH_BYTES: u64 = 64 << 20;
pub const RT_MAX_BATCH_SCENES: u32 = 65536;
pub const RT_TRAVERSAL_PACKET_PRIMARY: u32 = 0x1;
pub const RT_TRAVERSAL_PACKET_SHADOW: u32 = 0x2;
pub const RT_TRAVERSAL_PACKET_LANE_BOUNCES: u32 = 0x4;
pub const RT_AUTOTUNE_MAX_CONFIGS: usize = 64;
pub const RT_SERVE_PENDING: u32 = 0;
pub const RT_SERVE_DONE: u32 = 1;
pub const RT_SERVE_REJECTED: u32 = 2;

// ---- structs ----
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtGeometryTriangles {
    pub vertex_address: u64,
    pub index_address: u64,
    pub vertex_stride: u32,
    pub max_vertex: u32,
    pub primitive_count: u32,
    pub flags: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtBuildSizes {
    pub acceleration_structure_size: u64,
    pub build_scratch_size: u64,
    pub update_scratch_size: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtAccelerationStructureInfo {
    pub type_: u32,
    pub build_flags: u32,
    pub node_count: u32,
    pub primitive_count: u32,
    pub node_bytes: u32,
    pub tree_depth: u32,
    pub total_size: u64,
    pub compacted_size: u64,
    pub bounds_lo: [f32; 3],
    pub bounds_hi: [f32; 3],
    pub status: u32,
    pub _padding: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtTextureDesc {
    pub address: u64,
    pub width: u32,
    pub height: u32,
    pub row_pitch: u32,
    pub format: u32,
    pub filter: u32,
    pub _padding: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtHitGroup {
    pub closest_hit: u32,
    pub any_hit: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtShaderBindingTable {
    pub hit_group_count: u32,
    pub _padding: u32,
    pub hit_groups: [RtHitGroup; RT_MAX_HIT_GROUPS],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtTraceRaysDesc {
    pub width: u32,
    pub height: u32,
    pub max_trace_depth: u32,
    pub shadow_ray_count: u32,
    pub flags: u32,
    pub _padding: u32,
    pub image_address: u64,
    pub radiance_address: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtRay {
    pub origin: [f32; 3],
    pub tmin: f32,
    pub direction: [f32; 3],
    pub tmax: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtHit {
    pub t: f32,
    pub u: f32,
    pub v: f32,
    pub instance_id: u32,
    pub instance_custom_index: u32,
    pub geometry_index: u32,
    pub primitive_index: u32,
    pub hit_kind: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtTraceTimings {
    pub total_ms: f32,
    pub trace_ms: f32,
    pub closest_ms: f32,
    pub shadow_ms: f32,
    pub shade_ms: f32,
    pub other_ms: f32,
    pub trace_launches: u32,
    pub _padding: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtStats {
    pub traversals: u64,
    pub primary_rays: u64,
    pub secondary_rays: u64,
    pub shadow_rays: u64,
    pub nodes_visited: u64,
    pub triangles_tested: u64,
    pub instances_visited: u64,
    pub status: u32,
    pub _padding: u32,
    pub quantized_nodes_visited: u64,
}

/// The three device addresses of shared_structs::PushConstantBufferAddresses.
#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtPushConstantBufferAddresses {
    pub model_info: u64,
    pub uniforms: u64,
    pub acceleration_structure: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtBatchScene {
    pub push: RtPushConstantBufferAddresses,
    pub texture_count: u32,
    pub _padding: u32,
    pub texture_table: u64,
    pub desc: RtTraceRaysDesc,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtTraversalConfig {
    pub block_size: u32,
    pub shared_stack_depth: u32,
    pub leaf_wait: u32,
    pub packet_lists: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct RtAutotuneReport {
    pub count: u32,
    pub best: u32,
    pub configs: [RtTraversalConfig; RT_AUTOTUNE_MAX_CONFIGS],
    pub median_ms: [f32; RT_AUTOTUNE_MAX_CONFIGS],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtServerConfig {
    pub hbm_budget_bytes: u64,
    pub max_batch_requests: u32,
    pub max_batch_pixels: u32,
    pub max_in_flight: u32,
    pub max_batch_shadow_rays: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtServeScene {
    pub acceleration_structure: u64,
    pub model_info: u64,
    pub texture_table: u64,
    pub texture_count: u32,
    pub _padding: u32,
    pub resident_bytes: u64,
}

/// `uniforms` is the bytes of shared_structs::Uniforms (176 bytes, 16-byte aligned).
#[repr(C, align(16))]
#[derive(Clone, Copy, Debug)]
pub struct RtServeRequest {
    pub uniforms: [u8; 176],
    pub scene: u32,
    pub width: u32,
    pub height: u32,
    pub max_trace_depth: u32,
    pub shadow_ray_count: u32,
    pub flags: u32,
    pub image_device: u64,
    pub image_host: u64,
    pub _padding: [u32; 2],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtServeResult {
    pub state: u32,
    pub status: u32,
    pub batch: u32,
    pub batch_requests: u32,
    pub queue_ms: f64,
    pub latency_ms: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtServeStats {
    pub submitted: u64,
    pub completed: u64,
    pub rejected: u64,
    pub batches: u64,
    pub resident_bytes: u64,
    pub peak_bytes: u64,
    pub budget_bytes: u64,
    pub pixels: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtGlbInfo {
    pub vertex_count: u32,
    pub geometry_count: u32,
    pub image_count: u32,
    pub primitive_count: u32,
    pub triangle_count: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtGlbGeometry {
    pub index_count: u32,
    pub opaque: u32,
    pub diffuse_image: i32,
    pub metallic_roughness_image: i32,
    pub normal_map_image: i32,
    pub _padding: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct RtGlbImage {
    pub width: u32,
    pub height: u32,
    pub format: u32,
    pub filter: u32,
    pub byte_size: u64,
}

// The header's static size checks, restated.
const _: () = {
    assert!(core::mem::size_of::<RtGeometryTriangles>() == 32);
    assert!(core::mem::size_of::<RtTextureDesc>() == 32);
    assert!(core::mem::size_of::<RtRay>() == 32);
    assert!(core::mem::size_of::<RtHit>() == 32);
    assert!(core::mem::size_of::<RtShaderBindingTable>() == 72);
    assert!(core::mem::size_of::<RtTraceRaysDesc>() == 40);
    assert!(core::mem::size_of::<RtBatchScene>() == 80);
    assert!(core::mem::size_of::<RtServerConfig>() == 24);
    assert!(core::mem::size_of::<RtServeScene>() == 40);
    assert!(core::mem::size_of::<RtServeRequest>() == 224);
    assert!(core::mem::size_of::<RtServeResult>() == 32);
    assert!(core::mem::size_of::<RtServeStats>() == 64);
    assert!(core::mem::size_of::<RtTraceTimings>() == 32);
    assert!(core::mem::size_of::<RtStats>() == 72);
};

extern "C" {
    // ---- context ----
    pub fn rt_ctx_create(flags: u32, out: *mut *mut rt_ctx) -> i32;
    pub fn rt_ctx_destroy(ctx: *mut rt_ctx) -> i32;
    pub fn rt_ctx_set_texture(ctx: *mut rt_ctx, index: u32, desc: *const RtTextureDesc) -> i32;
    pub fn rt_ctx_read_stats(ctx: *mut rt_ctx, out: *mut RtStats, reset: i32, stream: CudaStream) -> i32;
    pub fn rt_ctx_read_trace_timings(ctx: *mut rt_ctx, out: *mut RtTraceTimings) -> i32;
    pub fn rt_last_error_string() -> *const c_char;
    pub fn rt_version_string() -> *const c_char;
    pub fn rt_kernel_launch_count() -> u64;

    // ---- acceleration structures (src/util_structs.rs:140-405, src/util_functions.rs:453-510) ----
    pub fn rt_get_blas_build_sizes(geometries: *const RtGeometryTriangles, geometry_count: u32, build_flags: u32,
                                   out: *mut RtBuildSizes) -> i32;
    pub fn rt_cmd_build_blas(ctx: *mut rt_ctx, geometries: *const RtGeometryTriangles, geometry_count: u32,
                             build_flags: u32, dst: u64, dst_size: u64, scratch: u64, scratch_size: u64,
                             stream: CudaStream) -> i32;
    pub fn rt_cmd_build_blas_static_scratch(ctx: *mut rt_ctx, geometries: *const RtGeometryTriangles,
                                            geometry_count: u32, build_flags: u32, dst: u64, dst_size: u64,
                                            stream: CudaStream) -> i32;
    pub fn rt_get_tlas_build_sizes(instance_count: u32, build_flags: u32, out: *mut RtBuildSizes) -> i32;
    pub fn rt_cmd_build_tlas(ctx: *mut rt_ctx, instances: u64, instance_count: u32, build_flags: u32, dst: u64,
                             dst_size: u64, scratch: u64, scratch_size: u64, stream: CudaStream) -> i32;
    pub fn rt_cmd_update_tlas(ctx: *mut rt_ctx, instances: u64, instance_count: u32, src: u64, dst: u64,
                              dst_size: u64, scratch: u64, scratch_size: u64, stream: CudaStream) -> i32;
    pub fn rt_cmd_copy_acceleration_structure(ctx: *mut rt_ctx, src: u64, dst: u64, dst_size: u64, mode: u32,
                                              stream: CudaStream) -> i32;
    pub fn rt_get_acceleration_structure_info(as_: u64, out: *mut RtAccelerationStructureInfo,
                                              stream: CudaStream) -> i32;
    pub fn rt_get_acceleration_structure_device_address(as_memory: u64) -> u64;

    // ---- dispatch (src/command_buffer_recording.rs:79-126) ----
    pub fn rt_cmd_trace_rays(ctx: *mut rt_ctx, push: *const RtPushConstantBufferAddresses,
                             sbt: *const RtShaderBindingTable, desc: *const RtTraceRaysDesc,
                             stream: CudaStream) -> i32;
    pub fn rt_cmd_trace_rays_batched(ctx: *mut rt_ctx, scenes: *const RtBatchScene, scene_count: u32,
                                     sbt: *const RtShaderBindingTable, flags: u32, stream: CudaStream) -> i32;
    pub fn rt_ctx_set_traversal_config(ctx: *mut rt_ctx, config: *const RtTraversalConfig) -> i32;
    pub fn rt_ctx_get_traversal_config(ctx: *mut rt_ctx, out: *mut RtTraversalConfig) -> i32;
    pub fn rt_ctx_autotune(ctx: *mut rt_ctx, scenes: *const RtBatchScene, scene_count: u32,
                           sbt: *const RtShaderBindingTable, reps: u32, stream: CudaStream,
                           report: *mut RtAutotuneReport) -> i32;
    pub fn rt_cmd_trace_ray_buffer(ctx: *mut rt_ctx, tlas: u64, push: *const RtPushConstantBufferAddresses,
                                   sbt: *const RtShaderBindingTable, ray_flags: u32, cull_mask: u32,
                                   sbt_offset: u32, rays: u64, ray_count: u32, hits: u64, stream: CudaStream) -> i32;
    pub fn rt_trace_ray_buffer_host(ctx: *mut rt_ctx, tlas: u64, push: *const RtPushConstantBufferAddresses,
                                    sbt: *const RtShaderBindingTable, ray_flags: u32, cull_mask: u32,
                                    sbt_offset: u32, host_rays: *const RtRay, ray_count: u32,
                                    host_hits: *mut RtHit, chunk_rays: u32, stream: CudaStream) -> i32;

    // ---- serving ----
    pub fn rt_server_create(ctx: *mut rt_ctx, config: *const RtServerConfig, out: *mut *mut rt_server) -> i32;
    pub fn rt_server_destroy(server: *mut rt_server) -> i32;
    pub fn rt_server_add_scene(server: *mut rt_server, scene: *const RtServeScene, id: *mut u32) -> i32;
    pub fn rt_server_submit(server: *mut rt_server, request: *const RtServeRequest, ticket: *mut u64) -> i32;
    pub fn rt_server_wait(server: *mut rt_server, ticket: u64, timeout_ms: u32, out: *mut RtServeResult) -> i32;
    pub fn rt_server_stats(server: *mut rt_server, out: *mut RtServeStats) -> i32;

    // ---- self-tests ----
    pub fn rt_debug_eval(function: u32, in_: u64, out: u64, count: u32, stream: CudaStream) -> i32;
    pub fn rt_debug_sort_pairs(keys: u64, values: u64, count: u32, scratch: u64, scratch_size: u64,
                               scratch_needed: *mut u64, stream: CudaStream) -> i32;

    // ---- assets (include/rtassets.h; host memory only) ----
    pub fn rt_png_decode_rgba8(bytes: *const c_void, size: u64, rgba8_out: *mut c_void, out_bytes: u64,
                               width: *mut u32, height: *mut u32) -> i32;
    pub fn rt_glb_load(bytes: *const c_void, size: u64, out: *mut *mut rt_glb_model) -> i32;
    pub fn rt_glb_info(model: *const rt_glb_model, info: *mut RtGlbInfo) -> i32;
    pub fn rt_glb_read_vertices(model: *const rt_glb_model, positions: *mut f32, normals: *mut f32,
                                uvs: *mut f32) -> i32;
    pub fn rt_glb_read_geometry(model: *const rt_glb_model, index: u32, info: *mut RtGlbGeometry,
                                indices: *mut u32, capacity: u64) -> i32;
    pub fn rt_glb_read_image(model: *const rt_glb_model, index: u32, info: *mut RtGlbImage, texels: *mut c_void,
                             capacity: u64) -> i32;
    pub fn rt_glb_destroy(model: *mut rt_glb_model) -> i32;
}
