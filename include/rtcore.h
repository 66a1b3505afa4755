/*
 * rtcore.h — C ABI of the GB300 ray-tracing core.
 *
 * This header is the drop-in boundary for the Vulkan ray-tracing dispatch of
 * expenses/ray-tracing-gallery.  It keeps the byte layouts of the reference's
 * host<->device structs and mirrors the Vulkan acceleration-structure model:
 * the caller queries sizes, allocates acceleration-structure (AS) and scratch
 * memory, and the library writes into it on the caller's CUDA stream.
 *
 * Conventions
 *  - Every "address" is a CUDA device pointer carried as uint64_t, exactly as
 *    the reference carries VkDeviceAddress values in its push constants.
 *  - `stream` is a cudaStream_t passed as void* (NULL = legacy default stream).
 *  - Every function returns an int32_t status (RT_OK = 0).  Nothing throws or
 *    aborts across the ABI; rt_last_error_string() describes the last failure
 *    of the calling thread.
 *  - Calls are asynchronous on `stream` unless documented otherwise.
 *
 * Reference interfaces replaced (paths inside the reference project):
 *  - rt_get_blas_build_sizes / rt_cmd_build_blas
 *      AccelerationStructure::build_blas   src/util_structs.rs:140-224
 *      AccelerationStructure::new          src/util_structs.rs:226-283
 *  - rt_get_tlas_build_sizes / rt_cmd_build_tlas
 *      build_tlas                           src/util_functions.rs:453-510
 *  - rt_cmd_update_tlas
 *      AccelerationStructure::update_tlas  src/util_structs.rs:285-357
 *  - rt_cmd_copy_acceleration_structure (CLONE)
 *      AccelerationStructure::clone        src/util_structs.rs:359-405
 *  - rt_cmd_trace_rays
 *      PerFrameResources::record -> cmd_trace_rays
 *                                           src/command_buffer_recording.rs:79-126
 *      and the device programs it runs: shaders/ray-tracing/src/lib.rs:33-312,
 *      shaders/closest_hit_textured.glsl, shaders/closest_hit_mirror.glsl,
 *      shaders/any_hit_alpha_clip.glsl, shaders/pbr.glsl
 *  - rt_ctx_set_texture
 *      ImageManager::push_image            src/util_structs.rs:1296-1377
 *      (bindless `textures[]`, shaders/hit_shader_common.glsl:67)
 */
#ifndef RTCORE_H
#define RTCORE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define RTCORE_API __attribute__((visibility("default")))
#else
#define RTCORE_API
#endif

/* ------------------------------------------------------------------------ */
/* Status codes                                                              */
/* ------------------------------------------------------------------------ */
#define RT_OK 0
#define RT_ERR_INVALID 1          /* bad argument, size or alignment        */
#define RT_ERR_OOM 2              /* an internal pool could not be allocated */
#define RT_ERR_STACK_OVERFLOW 3   /* a traversal stack overflowed (result incomplete) */
#define RT_ERR_TIMEOUT 4          /* a bounded device wait gave up           */
#define RT_ERR_CUDA 5             /* a CUDA runtime call failed              */
#define RT_ERR_UNSUPPORTED 6      /* feature or format not supported         */
#define RT_ERR_TOO_LARGE 7        /* input exceeds a documented maximum      */
#define RT_ERR_BAD_AS 8           /* address is not an AS written by this library */

#define RT_MAX_BOUND_IMAGES 128u  /* src/main.rs:44 MAX_BOUND_IMAGES */
#define RT_MAX_BLAS_GEOMETRIES 128u
#define RT_MAX_HIT_GROUPS 8u
#define RT_AS_ALIGNMENT 256u      /* Vulkan: AS offsets are 256-byte aligned */

/* ------------------------------------------------------------------------ */
/* L0 structs, byte-identical to the reference                              */
/* ------------------------------------------------------------------------ */

/* shared-structs/src/lib.rs:10-19 (glam Mat4 is 16-byte aligned; Vec3A is
 * 16 bytes).  Matrices are column-major: element (row r, column c) is at
 * index c*4 + r. */
typedef struct RtUniforms {
    float view_inverse[16];            /* @0   */
    float proj_inverse[16];            /* @64  */
    float sun_dir[3];                  /* @128 direction TOWARD the sun     */
    uint32_t _padding0;                /* @140 (Vec3A / GLSL `uint _padding`) */
    float sun_radius;                  /* @144 */
    uint32_t blue_noise_texture_index; /* @148 */
    uint32_t ggx_lut_texture_index;    /* @152 */
    uint32_t frame_index;              /* @156 */
    uint8_t show_heatmap;              /* @160 (Rust bool / GLSL uint8_t)   */
    uint8_t _padding1[15];             /* struct align 16 -> 176 bytes      */
} RtUniforms;

/* shared-structs/src/lib.rs:24-29 */
typedef struct RtModelInfo {
    uint64_t position_buffer_address;  /* float3[], stride 12 */
    uint64_t normal_buffer_address;    /* float3[], stride 12 */
    uint64_t uv_buffer_address;        /* float2[], stride 8  */
    uint64_t geometry_info_address;    /* RtGeometryInfo[]    */
} RtModelInfo;

/* shared-structs/src/lib.rs:42-47 */
typedef struct RtGeometryImages {
    uint32_t diffuse_image_index;
    uint32_t metallic_roughness_image_index;
    int32_t normal_map_image_index;    /* < 0: no normal map */
    uint32_t _padding;
} RtGeometryImages;

/* shared-structs/src/lib.rs:34-37 */
typedef struct RtGeometryInfo {
    uint64_t index_buffer_address;     /* uint32 triples */
    RtGeometryImages images;
} RtGeometryInfo;

/* shared-structs/src/lib.rs:52-56 — the reference's push constants */
typedef struct RtPushConstantBufferAddresses {
    uint64_t model_info;               /* RtModelInfo[] indexed by instance custom index */
    uint64_t uniforms;                 /* RtUniforms */
    uint64_t acceleration_structure;   /* TLAS address */
} RtPushConstantBufferAddresses;

/* src/gpu_structs.rs:20-25 == VkAccelerationStructureInstanceKHR.
 * transform: row-major 3x4 object->world matrix.
 * instance_custom_index_and_mask: low 24 bits custom index, high 8 bits mask.
 * instance_shader_binding_table_record_offset_and_flags: low 24 bits SBT
 *   record offset (hit-group base), high 8 bits RT_INSTANCE_* flags.
 * acceleration_structure_reference: BLAS address. */
typedef struct RtAccelerationStructureInstance {
    float transform[3][4];
    uint32_t instance_custom_index_and_mask;
    uint32_t instance_shader_binding_table_record_offset_and_flags;
    uint64_t acceleration_structure_reference;
} RtAccelerationStructureInstance;

/* VkGeometryInstanceFlagBitsKHR */
#define RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE 0x1u
#define RT_INSTANCE_TRIANGLE_FLIP_FACING 0x2u
#define RT_INSTANCE_FORCE_OPAQUE 0x4u
#define RT_INSTANCE_FORCE_NO_OPAQUE 0x8u

/* VkGeometryFlagBitsKHR */
#define RT_GEOMETRY_OPAQUE 0x1u
#define RT_GEOMETRY_NO_DUPLICATE_ANY_HIT_INVOCATION 0x2u

/* VkBuildAccelerationStructureFlagBitsKHR, plus one extension bit */
#define RT_BUILD_ALLOW_UPDATE 0x1u
#define RT_BUILD_ALLOW_COMPACTION 0x2u
#define RT_BUILD_PREFER_FAST_TRACE 0x4u
#define RT_BUILD_PREFER_FAST_BUILD 0x8u
#define RT_BUILD_LOW_MEMORY 0x10u
#define RT_BUILD_QUANTIZED_NODES 0x100u /* 8-bit conservatively quantised child boxes */
#define RT_BUILD_EXT_NODE_WIDTH_4 0x200u /* at most 4 children per node (same node layout) */

/* gl_RayFlags*EXT */
#define RT_RAY_FLAG_NONE 0x0u
#define RT_RAY_FLAG_OPAQUE 0x1u
#define RT_RAY_FLAG_NO_OPAQUE 0x2u
#define RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT 0x4u
#define RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER 0x8u
#define RT_RAY_FLAG_CULL_BACK_FACING 0x10u
#define RT_RAY_FLAG_CULL_FRONT_FACING 0x20u
#define RT_RAY_FLAG_CULL_OPAQUE 0x40u
#define RT_RAY_FLAG_CULL_NO_OPAQUE 0x80u
/* Extension bit for rt_cmd_trace_ray_buffer only: also count nodes,
 * triangles and instances visited into the context statistics. */
#define RT_RAY_FLAG_EXT_COLLECT_STATS 0x100u

/* ------------------------------------------------------------------------ */
/* Acceleration structures                                                   */
/* ------------------------------------------------------------------------ */

/* One triangle geometry of a BLAS (VkAccelerationStructureGeometryTrianglesDataKHR
 * + build range), as filled at src/util_structs.rs:151-186: R32G32B32_SFLOAT
 * positions, UINT32 indices, OPAQUE per geometry. */
typedef struct RtGeometryTriangles {
    uint64_t vertex_address;   /* device float3 positions                      */
    uint64_t index_address;    /* device uint32 triples; 0 = non-indexed        */
    uint32_t vertex_stride;    /* bytes between positions (>= 12, multiple of 4) */
    uint32_t max_vertex;       /* highest addressable vertex index              */
    uint32_t primitive_count;  /* triangles                                     */
    uint32_t flags;            /* RT_GEOMETRY_*                                 */
} RtGeometryTriangles;

/* VkAccelerationStructureBuildSizesInfoKHR */
typedef struct RtBuildSizes {
    uint64_t acceleration_structure_size;
    uint64_t build_scratch_size;
    uint64_t update_scratch_size;
} RtBuildSizes;

/* Read back by rt_get_acceleration_structure_info (synchronises `stream`). */
typedef struct RtAccelerationStructureInfo {
    uint32_t type;              /* 0 = bottom level, 1 = top level            */
    uint32_t build_flags;
    uint32_t node_count;        /* wide nodes in use                          */
    uint32_t primitive_count;   /* triangles (BLAS) or instances (TLAS)       */
    uint32_t node_bytes;        /* 256 (FP32 boxes) or 96 (quantised)         */
    uint32_t tree_depth;        /* wide levels                                */
    uint64_t total_size;        /* bytes this AS occupies as built            */
    uint64_t compacted_size;    /* bytes a COMPACT copy needs                 */
    float bounds_lo[3];
    float bounds_hi[3];
    uint32_t status;            /* RT_OK or the build's device-side error      */
    uint32_t _padding;
} RtAccelerationStructureInfo;

#define RT_COPY_MODE_CLONE 0u
#define RT_COPY_MODE_COMPACT 1u

/* ------------------------------------------------------------------------ */
/* Textures (the bindless `textures[]` array)                                */
/* ------------------------------------------------------------------------ */
#define RT_FORMAT_R8G8B8A8_UNORM 37u       /* VkFormat values */
#define RT_FORMAT_R8G8B8A8_SRGB 43u
#define RT_FORMAT_R32G32B32A32_SFLOAT 109u
#define RT_FILTER_NEAREST 0u
#define RT_FILTER_LINEAR 1u

/* Address mode is always REPEAT (the reference's samplers use the Vulkan
 * default, src/util_structs.rs:1306-1320). Sampling is done in software with
 * a fixed arithmetic order so host and device agree bit for bit. */
typedef struct RtTextureDesc {
    uint64_t address;     /* device pointer to texel rows */
    uint32_t width;
    uint32_t height;
    uint32_t row_pitch;   /* bytes between rows */
    uint32_t format;      /* RT_FORMAT_* */
    uint32_t filter;      /* RT_FILTER_* */
    uint32_t _padding;
} RtTextureDesc;

/* ------------------------------------------------------------------------ */
/* Programs and the shader binding table                                     */
/* ------------------------------------------------------------------------ */
#define RT_PROGRAM_NONE 0u
#define RT_PROGRAM_CLOSEST_HIT_TEXTURED 1u  /* shaders/closest_hit_textured.glsl */
#define RT_PROGRAM_CLOSEST_HIT_MIRROR 2u    /* shaders/closest_hit_mirror.glsl   */
#define RT_PROGRAM_CLOSEST_HIT_PORTAL 3u    /* shaders/ray-tracing/src/lib.rs:300-312 */
#define RT_PROGRAM_ANY_HIT_ALPHA_CLIP 1u    /* shaders/any_hit_alpha_clip.glsl  */

typedef struct RtHitGroup {
    uint32_t closest_hit;  /* RT_PROGRAM_CLOSEST_HIT_* or NONE */
    uint32_t any_hit;      /* RT_PROGRAM_ANY_HIT_ALPHA_CLIP or NONE */
} RtHitGroup;

/* Hit group index = instance SBT record offset + ray SBT offset (stride 0),
 * as in src/main.rs:289-305.  Indices >= hit_group_count run no program. */
typedef struct RtShaderBindingTable {
    uint32_t hit_group_count;
    uint32_t _padding;
    RtHitGroup hit_groups[RT_MAX_HIT_GROUPS];
} RtShaderBindingTable;

/* ------------------------------------------------------------------------ */
/* Dispatch                                                                  */
/* ------------------------------------------------------------------------ */
#define RT_TRACE_FLAG_COLLECT_STATS 0x1u    /* count nodes/triangles visited   */
#define RT_TRACE_FLAG_LAMBERT_DIFFUSE 0x2u  /* Fd_Lambert instead of Fd_Burley */
#define RT_TRACE_FLAG_KERNEL_TIMINGS 0x4u   /* record CUDA events around each kernel (rt_ctx_read_trace_timings) */

typedef struct RtTraceRaysDesc {
    uint32_t width;
    uint32_t height;
    uint32_t max_trace_depth;   /* iterations of the raygen bounce loop (reference: 3) */
    uint32_t shadow_ray_count;  /* shadow rays per textured hit (reference: 2)      */
    uint32_t flags;             /* RT_TRACE_FLAG_*                                  */
    uint32_t _padding;
    uint64_t image_address;     /* RGBA8, row-major width*height*4 bytes, row 0 = top */
    uint64_t radiance_address;  /* optional float4 linear colour per pixel, 0 = none  */
} RtTraceRaysDesc;

/* One ray of a ray-buffer query. */
typedef struct RtRay {
    float origin[3];
    float tmin;
    float direction[3];
    float tmax;
} RtRay;

/* Result of a ray-buffer query.  instance_id == 0xFFFFFFFF means miss. */
typedef struct RtHit {
    float t;
    float u;                      /* barycentric weight of vertex 1 */
    float v;                      /* barycentric weight of vertex 2 */
    uint32_t instance_id;         /* gl_InstanceID (index in the instance array) */
    uint32_t instance_custom_index;
    uint32_t geometry_index;
    uint32_t primitive_index;
    uint32_t hit_kind;            /* 0xFE front face, 0xFF back face (gl_HitKind*) */
} RtHit;

/* Kernel times of the last rt_cmd_trace_rays launched with
 * RT_TRACE_FLAG_KERNEL_TIMINGS (CUDA events on the launch's stream). */
typedef struct RtTraceTimings {
    float total_ms;        /* first kernel start .. last kernel end */
    float trace_ms;        /* all traversal launches */
    float closest_ms;      /* closest-hit traversal launches (one per bounce) */
    float shadow_ms;       /* the shadow-ray traversal launch */
    float shade_ms;        /* closest-hit / miss program launches */
    float other_ms;        /* raygen, resolve, output */
    uint32_t trace_launches;
    uint32_t _padding;
} RtTraceTimings;

typedef struct RtStats {
    uint64_t traversals;          /* rays traced (each traceRay counted once) */
    uint64_t primary_rays;        /* first iteration of the bounce loop        */
    uint64_t secondary_rays;      /* mirror / portal continuation rays         */
    uint64_t shadow_rays;
    uint64_t nodes_visited;       /* only with RT_TRACE_FLAG_COLLECT_STATS     */
    uint64_t triangles_tested;    /* only with RT_TRACE_FLAG_COLLECT_STATS     */
    uint64_t instances_visited;   /* only with RT_TRACE_FLAG_COLLECT_STATS     */
    uint32_t status;              /* bit (1 << RT_ERR_*) set for every kind of
                                     device-side error seen; 0 = none          */
    uint32_t _padding;
    uint64_t quantized_nodes_visited; /* of nodes_visited: 96-byte quantised BLAS
                                     nodes (the rest are 256-byte FP32 nodes)  */
} RtStats;

/* ------------------------------------------------------------------------ */
/* Context                                                                   */
/* ------------------------------------------------------------------------ */
typedef struct rt_ctx rt_ctx;

#define RT_CTX_THREADSAFE 0x1u

/* Creates a context on the current CUDA device.  The context owns only a
 * small device block (statistics and status words) and the texture table. */
RTCORE_API int32_t rt_ctx_create(uint32_t flags, rt_ctx** out);
RTCORE_API int32_t rt_ctx_destroy(rt_ctx* ctx);
/* Binds textures[index] (index < RT_MAX_BOUND_IMAGES).  Host-side state,
 * captured by value at each rt_cmd_trace_* call. */
RTCORE_API int32_t rt_ctx_set_texture(rt_ctx* ctx, uint32_t index, const RtTextureDesc* desc);
/* Reads (and optionally zeroes) the statistics; synchronises `stream`. */
RTCORE_API int32_t rt_ctx_read_stats(rt_ctx* ctx, RtStats* out, int32_t reset, void* stream);
/* Waits for and reads the kernel times of the last timed trace launch. */
RTCORE_API int32_t rt_ctx_read_trace_timings(rt_ctx* ctx, RtTraceTimings* out);
RTCORE_API const char* rt_last_error_string(void);
RTCORE_API const char* rt_version_string(void);
/* Kernels this library has launched in this process (diagnostics). */
RTCORE_API uint64_t rt_kernel_launch_count(void);

/* ---- acceleration structures (ctx may be NULL for build/copy calls) ---- */
RTCORE_API int32_t rt_get_blas_build_sizes(const RtGeometryTriangles* geometries, uint32_t geometry_count,
                                           uint32_t build_flags, RtBuildSizes* out);
/* `geometries` is a HOST array, read before the call returns. */
RTCORE_API int32_t rt_cmd_build_blas(rt_ctx* ctx, const RtGeometryTriangles* geometries,
                                     uint32_t geometry_count, uint32_t build_flags, uint64_t dst,
                                     uint64_t dst_size, uint64_t scratch, uint64_t scratch_size,
                                     void* stream);
/* Builds a BLAS exactly like rt_cmd_build_blas, but allocates nothing and
 * takes no scratch argument: the build scratch is one fixed device array
 * inside librtcore of RT_STATIC_SCRATCH_BYTES, which every GPU that loads
 * the library holds until the process exits.  No counterpart in the
 * reference (its Vulkan path always receives caller-allocated scratch).
 * It is for callers that may not allocate device memory when they build:
 * a host whose device memory belongs to another allocator that hands this
 * library only the destination buffer, or a frame loop whose memory budget
 * is fixed at start-up.
 * FP32 nodes only: RT_BUILD_QUANTIZED_NODES returns RT_ERR_UNSUPPORTED.
 * Limit: geometries whose rt_get_blas_build_sizes().build_scratch_size (with
 * the same flags) is above RT_STATIC_SCRATCH_BYTES are rejected with
 * RT_ERR_TOO_LARGE before anything is queued.  That is about 288k triangles
 * with RT_BUILD_PREFER_FAST_TRACE (its PLOC hierarchy needs more scratch)
 * and about 462k otherwise; the size query is the exact check.  Every call uses the same
 * array, so calls whose GPU work can overlap (different streams with no
 * ordering between them) race and corrupt each other's builds; order them.
 * The first call on each device looks the array's device address up
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. */
#define RT_STATIC_SCRATCH_BYTES (64ull << 20)
RTCORE_API int32_t rt_cmd_build_blas_static_scratch(rt_ctx* ctx, const RtGeometryTriangles* geometries,
                                                    uint32_t geometry_count, uint32_t build_flags, uint64_t dst,
                                                    uint64_t dst_size, void* stream);
RTCORE_API int32_t rt_get_tlas_build_sizes(uint32_t instance_count, uint32_t build_flags, RtBuildSizes* out);
/* `instances` is a DEVICE array of RtAccelerationStructureInstance. */
RTCORE_API int32_t rt_cmd_build_tlas(rt_ctx* ctx, uint64_t instances, uint32_t instance_count,
                                     uint32_t build_flags, uint64_t dst, uint64_t dst_size,
                                     uint64_t scratch, uint64_t scratch_size, void* stream);
/* In-place (src == dst) or out-of-place refit of a TLAS built with
 * RT_BUILD_ALLOW_UPDATE; topology is kept, every instance record is re-read. */
RTCORE_API int32_t rt_cmd_update_tlas(rt_ctx* ctx, uint64_t instances, uint32_t instance_count,
                                      uint64_t src, uint64_t dst, uint64_t dst_size, uint64_t scratch,
                                      uint64_t scratch_size, void* stream);
RTCORE_API int32_t rt_cmd_copy_acceleration_structure(rt_ctx* ctx, uint64_t src, uint64_t dst,
                                                      uint64_t dst_size, uint32_t mode, void* stream);
/* Synchronises `stream`, then reads the AS header. */
RTCORE_API int32_t rt_get_acceleration_structure_info(uint64_t as, RtAccelerationStructureInfo* out,
                                                      void* stream);
/* The AS device address is the address of its memory (checked for alignment). */
RTCORE_API uint64_t rt_get_acceleration_structure_device_address(uint64_t as_memory);

/* ---- dispatch ---- */
/* The reference's cmd_trace_rays with its pipeline: raygen -> traversal ->
 * any-hit / closest-hit / miss programs, writing an RGBA8 image.  sbt may be
 * NULL for the reference's table (textured, mirror, portal; alpha-clip any-hit
 * in every group). */
RTCORE_API int32_t rt_cmd_trace_rays(rt_ctx* ctx, const RtPushConstantBufferAddresses* push,
                                     const RtShaderBindingTable* sbt, const RtTraceRaysDesc* desc,
                                     void* stream);

/* One scene of rt_cmd_trace_rays_batched: the arguments of one
 * rt_cmd_trace_rays call, plus the scene's own bindless texture table. */
typedef struct RtBatchScene {
    RtPushConstantBufferAddresses push;  /* model_info, uniforms, acceleration_structure */
    uint32_t texture_count;              /* entries at texture_table (1..RT_MAX_BOUND_IMAGES) */
    uint32_t _padding;
    uint64_t texture_table;              /* device RtTextureDesc[texture_count]; 0 = the context's table */
    RtTraceRaysDesc desc;                /* size, depth, shadow rays, outputs; desc.flags: LAMBERT only */
} RtBatchScene;
#define RT_MAX_BATCH_SCENES 65536u
/* Many scenes (each its own TLAS, uniforms, textures, size, depth and shadow
 * count) rendered by one set of persistent launches: the primary, shadow and
 * reflection wavefronts of all scenes share each traversal launch, so a batch
 * of small frames fills the GPU that one small frame cannot.  Every scene's
 * image is identical to what rt_cmd_trace_rays gives for it alone.  No
 * counterpart in the reference, which records one vkCmdTraceRaysKHR per
 * frame (src/command_buffer_recording.rs:116-126).  `flags`:
 * RT_TRACE_FLAG_COLLECT_STATS / RT_TRACE_FLAG_KERNEL_TIMINGS.  The launch
 * sequence is fixed by the scenes' sizes alone (ray counts stay on the
 * device), so it can be captured into a CUDA graph and replayed; trace the
 * same sizes once outside the capture first, since the per-stream workspace
 * cannot grow inside one (RT_ERR_INVALID then).  At most 2^31 ray slots and
 * 2^31 shadow rays per batch. */
RTCORE_API int32_t rt_cmd_trace_rays_batched(rt_ctx* ctx, const RtBatchScene* scenes, uint32_t scene_count,
                                             const RtShaderBindingTable* sbt, uint32_t flags, void* stream);

/* Launch shape of the wavefront traversal kernels (rt_cmd_trace_rays and
 * rt_cmd_trace_rays_batched).  Every configuration gives identical results;
 * they differ only in speed.  No counterpart in the reference (the driver
 * schedules its own traversal).
 *   block_size          threads per block: 64, 128 or 256 (24 warps per SM each;
 *                       packet kernels 20 for 64 / 128)
 *   shared_stack_depth  traversal-stack entries kept in shared memory: 0, 16,
 *                       24 or 32 (the rest of the 64 live in local memory)
 *   leaf_wait           0..32: a warp runs leaf steps once leaf_wait/32 of its
 *                       lanes wait on one, else node steps
 *   packet_lists        RT_TRAVERSAL_PACKET_* bits: the ray lists a warp
 *                       traverses as one packet of 32 neighbouring rays (one
 *                       node sequence for the union of their box hits, stack
 *                       in shared memory); the other lists run one ray per
 *                       lane with the three fields above.  Packets pay on
 *                       large coherent frames; for small images a request
 *                       lasts as long as its slowest tile, so they are
 *                       opt-in (rt_ctx_autotune tries them)
 * Default {128, 0, 20, 0}. */
#define RT_TRAVERSAL_PACKET_PRIMARY 0x1u /* camera rays (8x4 pixel tiles) and their mirror / portal bounces */
#define RT_TRAVERSAL_PACKET_SHADOW 0x2u  /* the shadow rays of each shaded pixel, appended per shading warp */
/* with PACKET_PRIMARY: the mirror / portal continuation rays of a packet are
 * traced one per lane inside the packet launch instead of as further
 * sub-packets (pays when many pixels see curved mirrors) */
#define RT_TRAVERSAL_PACKET_LANE_BOUNCES 0x4u
typedef struct RtTraversalConfig {
    uint32_t block_size;
    uint32_t shared_stack_depth;
    uint32_t leaf_wait;
    uint32_t packet_lists;
} RtTraversalConfig;
RTCORE_API int32_t rt_ctx_set_traversal_config(rt_ctx* ctx, const RtTraversalConfig* config);
RTCORE_API int32_t rt_ctx_get_traversal_config(rt_ctx* ctx, RtTraversalConfig* out);

#define RT_AUTOTUNE_MAX_CONFIGS 64u
typedef struct RtAutotuneReport {
    uint32_t count;                                  /* configurations timed */
    uint32_t best;                                   /* index of the fastest */
    RtTraversalConfig configs[RT_AUTOTUNE_MAX_CONFIGS];
    float median_ms[RT_AUTOTUNE_MAX_CONFIGS];        /* of `reps` batched launches each */
} RtAutotuneReport;
/* Times rt_cmd_trace_rays_batched(scenes) under the traversal configurations
 * and makes the fastest the context's configuration: first the 36 per-lane
 * launch shapes (block size x shared stack depth x leaf_wait in {16, 20,
 * 24}), then packet_lists 1, 2, 3, 5 and 7 on the fastest shape (41 in all),
 * `reps` timed launches each after one warm-up.  Synchronises `stream`; not allowed while it
 * is being captured.  The scenes' output buffers are overwritten.  `report`
 * may be NULL. */
RTCORE_API int32_t rt_ctx_autotune(rt_ctx* ctx, const RtBatchScene* scenes, uint32_t scene_count,
                                   const RtShaderBindingTable* sbt, uint32_t reps, void* stream,
                                   RtAutotuneReport* report);
/* ---- serving: a request loop over device-resident scenes ----
 * No counterpart in the reference (a single-window renderer).  A server owns
 * one stream and a worker thread.  Scenes stay resident (their BVHs, buffers
 * and textures are the caller's, registered with their byte size); requests
 * (scene, camera/light uniforms, size, depth, shadow rays) are admitted in
 * arrival order while resident scenes + frame buffers + the batch workspace
 * fit the HBM budget, and the admitted ones are rendered together by
 * rt_cmd_trace_rays_batched as soon as one of `max_in_flight` batch slots is
 * free (continuous batching: requests that arrive while a batch runs join the
 * next one).  A batch also stays within max_batch_pixels ray slots and
 * max_batch_shadow_rays shadow rays (a request beyond a limit on its own is
 * rendered alone).  With both limits set, rt_server_create sizes the
 * stream's wavefront workspace and the frame-buffer pool for the largest
 * batch they allow (counted in the budget from then on), so batches within
 * the limits allocate nothing while requests stream.  A request whose
 * image_host is page-locked has its image written there by the output
 * kernel; a pageable image_host gets a copy from a server frame buffer.  A
 * request's image is identical to rendering it alone. */
typedef struct rt_server rt_server;
typedef struct RtServerConfig {
    uint64_t hbm_budget_bytes;    /* resident scenes + frame buffers + workspace */
    uint32_t max_batch_requests;  /* 1 = the plain per-request path */
    uint32_t max_batch_pixels;    /* ray slots per batch (pixels padded to 8x4 tiles); 0 = no limit */
    uint32_t max_in_flight;       /* batches queued on the GPU at once, >= 1 */
    uint32_t max_batch_shadow_rays; /* pixels x shadow rays per batch; 0 = no limit */
} RtServerConfig;
typedef struct RtServeScene {
    uint64_t acceleration_structure;  /* TLAS device address */
    uint64_t model_info;              /* device RtModelInfo[] */
    uint64_t texture_table;           /* device RtTextureDesc[texture_count] */
    uint32_t texture_count;
    uint32_t _padding;
    uint64_t resident_bytes;          /* device bytes the scene keeps resident */
} RtServeScene;
typedef struct RtServeRequest {
    RtUniforms uniforms;              /* copied at submit */
    uint32_t scene;                   /* rt_server_add_scene id */
    uint32_t width, height;
    uint32_t max_trace_depth;
    uint32_t shadow_ray_count;
    uint32_t flags;                   /* RT_TRACE_FLAG_LAMBERT_DIFFUSE */
    uint64_t image_device;            /* 0 = a server frame buffer (counted in the budget) */
    uint64_t image_host;              /* optional: RGBA8 copied here (pinned memory recommended) */
    uint32_t _padding[2];
} RtServeRequest;
#define RT_SERVE_PENDING 0u
#define RT_SERVE_DONE 1u
#define RT_SERVE_REJECTED 2u
typedef struct RtServeResult {
    uint32_t state;                   /* RT_SERVE_* */
    uint32_t status;                  /* RT_OK or why it failed / was rejected */
    uint32_t batch;                   /* sequence number of its batch */
    uint32_t batch_requests;          /* requests in that batch */
    double queue_ms;                  /* submit -> its batch was launched */
    double latency_ms;                /* submit -> image complete (and copied to image_host) */
} RtServeResult;
typedef struct RtServeStats {
    uint64_t submitted, completed, rejected, batches;
    uint64_t resident_bytes, peak_bytes, budget_bytes;
    uint64_t pixels;                  /* rendered */
} RtServeStats;
RTCORE_API int32_t rt_server_create(rt_ctx* ctx, const RtServerConfig* config, rt_server** out);
/* Finishes every admitted request, then releases the server's memory. */
RTCORE_API int32_t rt_server_destroy(rt_server* server);
/* RT_ERR_OOM if the scene would exceed the budget. */
RTCORE_API int32_t rt_server_add_scene(rt_server* server, const RtServeScene* scene, uint32_t* id);
/* Queues a request; RT_ERR_TOO_LARGE if it cannot fit the budget even alone. */
RTCORE_API int32_t rt_server_submit(rt_server* server, const RtServeRequest* request, uint64_t* ticket);
/* Waits up to timeout_ms for `ticket` (RT_ERR_TIMEOUT if still pending); a
 * finished result is returned once and then forgotten. */
RTCORE_API int32_t rt_server_wait(rt_server* server, uint64_t ticket, uint32_t timeout_ms, RtServeResult* out);
RTCORE_API int32_t rt_server_stats(rt_server* server, RtServeStats* out);

/* Traversal only: one traceRay per RtRay against `tlas`, writing RtHit.
 * `push` may be NULL (then any-hit programs cannot run and candidates are
 * accepted as if opaque). */
RTCORE_API int32_t rt_cmd_trace_ray_buffer(rt_ctx* ctx, uint64_t tlas, const RtPushConstantBufferAddresses* push,
                                           const RtShaderBindingTable* sbt, uint32_t ray_flags,
                                           uint32_t cull_mask, uint32_t sbt_offset, uint64_t rays,
                                           uint32_t ray_count, uint64_t hits, void* stream);

/* rt_cmd_trace_ray_buffer from host memory.  With chunk_rays = 0 and both
 * buffers page-locked (cudaHostAlloc / cudaHostRegister), one traversal
 * launch reads the rays from and writes the hits to host memory directly
 * (mapped host memory; NVLink-C2C on Grace systems).  Otherwise the rays are
 * copied in, traced and their hits copied out in chunks of `chunk_rays`
 * (0 = 1M), alternating two internal streams so that one chunk's copies
 * overlap another chunk's traversal.  Ordered after the work already queued
 * on `stream`; on return everything is queued and `stream` waits for it
 * (synchronise `stream` before reading host_hits).  Pageable buffers take
 * the copy path and their copies do not overlap.  No counterpart in the
 * reference, whose rays never leave the GPU. */
RTCORE_API int32_t rt_trace_ray_buffer_host(rt_ctx* ctx, uint64_t tlas, const RtPushConstantBufferAddresses* push,
                                            const RtShaderBindingTable* sbt, uint32_t ray_flags,
                                            uint32_t cull_mask, uint32_t sbt_offset, const RtRay* host_rays,
                                            uint32_t ray_count, RtHit* host_hits, uint32_t chunk_rays,
                                            void* stream);

/* ---- device math self-test (evaluates shader functions element-wise) ---- */
#define RT_FN_V_SMITH_GGX_CORRELATED 0u  /* in: NoV, NoL, roughness            -> out: V  */
#define RT_FN_D_GGX 1u                   /* in: NoH, roughness                 -> out: D  */
#define RT_FN_LINEAR_TO_SRGB 2u          /* in: x                              -> out: y  */
#define RT_FN_HEATMAP 3u                 /* in: heat                           -> out: rgb */
#define RT_FN_SINCOS 4u                  /* in: angle                          -> out: sin, cos */
#define RT_FN_BRDF 5u                    /* in: 16 floats (see oracle)         -> out: rgb */
#define RT_FN_WATERTIGHT 6u              /* in: ray + triangle (16 floats)     -> out: hit, t, u, v */
/* `in` and `out` are device float arrays with the per-function stride. */
RTCORE_API int32_t rt_debug_eval(uint32_t function, uint64_t in, uint64_t out, uint32_t count, void* stream);
/* Self-test of the BVH builder's key sort (the Morton-code sort inside
 * rt_cmd_build_blas / rt_cmd_build_tlas): sorts `count` device (uint32 key,
 * uint32 value) pairs in place, stably by key.  `scratch` (256-byte aligned,
 * scratch_size bytes) holds the second buffers and the sort state; with
 * scratch = 0 only *scratch_needed is written.  Synchronises `stream`;
 * RT_ERR_TIMEOUT if a bounded wait of the sort gave up.  No counterpart in
 * the reference (the driver's build is closed). */
RTCORE_API int32_t rt_debug_sort_pairs(uint64_t keys, uint64_t values, uint32_t count, uint64_t scratch,
                                       uint64_t scratch_size, uint64_t* scratch_needed, void* stream);

#ifdef __cplusplus
} /* extern "C" */
#endif

#ifdef __cplusplus
#define RT_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define RT_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif
RT_STATIC_ASSERT(sizeof(RtUniforms) == 176, "Uniforms is 176 bytes");
RT_STATIC_ASSERT(offsetof(RtUniforms, proj_inverse) == 64, "Uniforms.proj_inverse @64");
RT_STATIC_ASSERT(offsetof(RtUniforms, sun_dir) == 128, "Uniforms.sun_dir @128");
RT_STATIC_ASSERT(offsetof(RtUniforms, sun_radius) == 144, "Uniforms.sun_radius @144");
RT_STATIC_ASSERT(offsetof(RtUniforms, blue_noise_texture_index) == 148, "@148");
RT_STATIC_ASSERT(offsetof(RtUniforms, ggx_lut_texture_index) == 152, "@152");
RT_STATIC_ASSERT(offsetof(RtUniforms, frame_index) == 156, "@156");
RT_STATIC_ASSERT(offsetof(RtUniforms, show_heatmap) == 160, "@160");
RT_STATIC_ASSERT(sizeof(RtModelInfo) == 32, "ModelInfo is 32 bytes");
RT_STATIC_ASSERT(sizeof(RtGeometryImages) == 16, "GeometryImages is 16 bytes");
RT_STATIC_ASSERT(sizeof(RtGeometryInfo) == 24, "GeometryInfo is 24 bytes");
RT_STATIC_ASSERT(sizeof(RtPushConstantBufferAddresses) == 24, "push constants are 24 bytes");
RT_STATIC_ASSERT(sizeof(RtAccelerationStructureInstance) == 64, "instance record is 64 bytes");
RT_STATIC_ASSERT(offsetof(RtAccelerationStructureInstance, instance_custom_index_and_mask) == 48, "@48");
RT_STATIC_ASSERT(offsetof(RtAccelerationStructureInstance, acceleration_structure_reference) == 56, "@56");
RT_STATIC_ASSERT(sizeof(RtGeometryTriangles) == 32, "geometry desc is 32 bytes");
RT_STATIC_ASSERT(sizeof(RtTextureDesc) == 32, "texture desc is 32 bytes");
RT_STATIC_ASSERT(sizeof(RtRay) == 32, "ray is 32 bytes");
RT_STATIC_ASSERT(sizeof(RtHit) == 32, "hit is 32 bytes");
RT_STATIC_ASSERT(sizeof(RtShaderBindingTable) == 72, "sbt is 72 bytes");
RT_STATIC_ASSERT(sizeof(RtTraceRaysDesc) == 40, "trace desc is 40 bytes");
RT_STATIC_ASSERT(sizeof(RtBatchScene) == 80, "batch scene is 80 bytes");
RT_STATIC_ASSERT(offsetof(RtBatchScene, desc) == 40, "RtBatchScene.desc @40");
RT_STATIC_ASSERT(sizeof(RtServerConfig) == 24, "server config is 24 bytes");
RT_STATIC_ASSERT(sizeof(RtServeScene) == 40, "serve scene is 40 bytes");
RT_STATIC_ASSERT(sizeof(RtServeRequest) == 224, "serve request is 224 bytes");
RT_STATIC_ASSERT(offsetof(RtServeRequest, image_device) == 200, "RtServeRequest.image_device @200");
RT_STATIC_ASSERT(sizeof(RtServeResult) == 32, "serve result is 32 bytes");
RT_STATIC_ASSERT(sizeof(RtServeStats) == 64, "serve stats are 64 bytes");
RT_STATIC_ASSERT(sizeof(RtTraceTimings) == 32, "timings are 32 bytes");
RT_STATIC_ASSERT(sizeof(RtStats) == 72, "stats are 72 bytes");

#endif /* RTCORE_H */
