/*
 * rt_oracle.h — CPU oracle for the ray-tracing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * cpu_baseline / reference legs of bench.py may load this library; the product
 * library (librtcore) never links or calls it.
 *
 * What it restates (paths inside the reference project expanded in
 * rt_oracle.c next to each function):
 *   - ray_generation, primary_ray_miss, shadow_ray_miss, closest_hit_portal
 *       shaders/ray-tracing/src/lib.rs
 *   - closest_hit_textured, closest_hit_mirror, any_hit_alpha_clip, pbr
 *       shaders/ (the GLSL hit shaders)
 *   - heatmap_temperature              shaders/ray-tracing/src/heatmap.rs
 *   - V_SmithGGXCorrelated unit test   shaders/ray-tracing/src/pbr.rs:52-69
 * The reference's BVH build and traversal live in the closed Vulkan driver;
 * the oracle defines them as: a binary binned-SAH BVH (its own, independent of
 * the product's LBVH), a watertight FP32 ray/triangle test (Woop, Benthin &
 * Wald, JCGT 2013) and a closest hit under the total order
 * (t, instance index, geometry index, primitive index).
 *
 * Parity of hit IDs and images against the reference itself is UNPINNED: the
 * reference needs a Vulkan ray-tracing driver, which does not exist here.
 */
#ifndef RT_ORACLE_H
#define RT_ORACLE_H

#include <stdint.h>
#include "../include/rtcore.h"

#ifdef __cplusplus
extern "C" {
#endif

/* A BLAS geometry in host memory (positions stride in floats). */
typedef struct OGeometry {
    const float* positions;
    uint32_t stride_floats;
    uint32_t max_vertex;
    const uint32_t* indices; /* NULL = non-indexed */
    uint32_t primitive_count;
    uint32_t flags;          /* RT_GEOMETRY_* */
} OGeometry;

/* Host-memory mirror of RtGeometryInfo. */
typedef struct OGeometryInfo {
    const uint32_t* indices;
    uint32_t diffuse_image_index;
    uint32_t metallic_roughness_image_index;
    int32_t normal_map_image_index;
    uint32_t _padding;
} OGeometryInfo;

/* Host-memory mirror of RtModelInfo. */
typedef struct OModelInfo {
    const float* positions;  /* float3 */
    const float* normals;    /* float3 */
    const float* uvs;        /* float2 */
    const OGeometryInfo* geometries;
    uint32_t geometry_count;
    uint32_t _padding;
} OModelInfo;

typedef struct OTexture {
    const void* texels;
    uint32_t width, height, row_pitch, format, filter, _padding;
} OTexture;

typedef struct ORenderDesc {
    uint32_t width, height;
    uint32_t max_trace_depth;
    uint32_t shadow_ray_count;
    uint32_t flags;          /* RT_TRACE_FLAG_* */
    uint32_t row_begin;      /* render rows [row_begin, row_end) only */
    uint32_t row_end;
    uint32_t double_shading; /* 1 = shading arithmetic in FP64 */
} ORenderDesc;

typedef struct OStats {
    uint64_t traversals, primary_rays, secondary_rays, shadow_rays;
    uint64_t nodes_visited, triangles_tested, instances_visited;
} OStats;

typedef struct OScene OScene;

OScene* o_scene_create(void);
void o_scene_destroy(OScene* s);
/* Returns the BLAS id (used as acceleration_structure_reference). */
int32_t o_scene_add_blas(OScene* s, const OGeometry* geoms, uint32_t count);
/* Instance records; acceleration_structure_reference holds a BLAS id. */
int32_t o_scene_set_instances(OScene* s, const RtAccelerationStructureInstance* inst, uint32_t count);
int32_t o_scene_set_models(OScene* s, const OModelInfo* models, uint32_t count);
int32_t o_scene_set_texture(OScene* s, uint32_t index, const OTexture* tex);
/* Builds every BLAS BVH that is not built yet and rebuilds the TLAS. */
int32_t o_scene_build(OScene* s);
/* 1 = test every instance and triangle (no BVH); for small cases. */
void o_scene_set_bruteforce(OScene* s, int32_t on);

/* Traversal-only query; same semantics as rt_cmd_trace_ray_buffer. */
int32_t o_trace_ray_buffer(OScene* s, const RtShaderBindingTable* sbt, int32_t have_models,
                           uint32_t ray_flags, uint32_t cull_mask, uint32_t sbt_offset,
                           const RtRay* rays, uint32_t count, RtHit* hits, int32_t threads,
                           OStats* stats);
/* The reference's pipeline; image is RGBA8 width*height*4, radiance float4 per
 * pixel (either may be NULL).  Only rows [row_begin,row_end) are written. */
int32_t o_render(OScene* s, const RtUniforms* u, const RtShaderBindingTable* sbt,
                 const ORenderDesc* desc, uint8_t* image, float* radiance, int32_t threads,
                 OStats* stats);

/* Element-wise evaluation of shader functions (same ids as rt_debug_eval). */
int32_t o_debug_eval(uint32_t function, const float* in, float* out, uint32_t count, int32_t dbl);

/* Precomputed world-to-object matrix of an instance (row-major 3x4); returns
 * 0 for a singular transform. */
int32_t o_instance_world_to_object(const float object_to_world[12], float out[12]);

#ifdef __cplusplus
}
#endif
#endif
