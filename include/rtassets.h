/*
 * rtassets.h — host-side asset decoding for the ray-tracing core.
 *
 * The reference feeds its BLAS builds and its bindless texture array from
 * glTF-binary models and PNG images decoded on the CPU.  These entry points do
 * the same decoding natively, producing exactly the arrays the rest of the ABI
 * consumes: vertex / index arrays for rt_cmd_build_blas and the model-info
 * table, RGBA8 (or one RGBA32F texel) images for rt_ctx_set_texture /
 * per-scene texture tables.  They are host code only: nothing here touches
 * the GPU, and every call is synchronous and thread-safe (a model handle may
 * be read from several threads; rt_glb_destroy must not race with readers).
 *
 * Reference interfaces replaced (paths inside the reference project):
 *  - rt_png_decode_rgba8
 *      load_png_image_from_bytes          src/util_functions.rs:239-265
 *      (image 0.23.14 load_from_memory_with_format(Png) then to_rgba8)
 *  - rt_glb_load, rt_glb_info, rt_glb_read_vertices, rt_glb_read_geometry,
 *    rt_glb_read_image, rt_glb_destroy
 *      Model::load_gltf                   src/util_structs.rs:1049-1156
 *      load_images_from_material          src/util_structs.rs:982-1024
 *      load_image_from_gltf_texture       src/util_structs.rs:934-980
 *      metallic_roughness_to_rgba         src/util_structs.rs:1027-1029
 *      create_single_colour_image         src/util_functions.rs:216-237
 *
 * Decoding rules (each restates the reference's behaviour):
 *  - PNG: every colour type and bit depth of the PNG specification, Adam7
 *    interlacing, PLTE and tRNS; CRC-32 and Adler-32 are verified.  The result
 *    is RGBA8: grey g -> (g, g, g, 255); grey+alpha -> (g, g, g, a); RGB adds
 *    alpha 255; palette entries expand through PLTE and tRNS; grey below 8 bits
 *    is scaled to 0..255; tRNS colour keys give alpha 0; 16-bit samples keep
 *    their high byte.
 *  - GLB: node transforms are ignored (the mesh data is used as stored, as
 *    the reference does).  One geometry per material, in material order; a
 *    file without materials has one opaque geometry.  Every primitive of every
 *    mesh appends its vertices and its indices (offset by the vertices already
 *    read) to the geometry of its material (material 0 when it names none).
 *    A geometry is opaque when its material's alphaMode is OPAQUE.
 *  - Images are numbered in the order the reference pushes them into its
 *    image manager: per material its diffuse image (the baseColorTexture as
 *    R8G8B8A8_SRGB, else one R32G32B32A32_SFLOAT texel of baseColorFactor),
 *    its metallic-roughness image (the metallicRoughnessTexture as
 *    R8G8B8A8_SRGB, else one texel [1, roughness, metallic, 1]) and, when the
 *    material has one, its normal map (R8G8B8A8_UNORM).  A decoded texture is
 *    sampled with RT_FILTER_LINEAR unless its sampler's magFilter is NEAREST;
 *    single-colour images use RT_FILTER_NEAREST.  A file without materials
 *    has one image: the texel [1, 1, 0, 1] (metallic 0, roughness 1); its
 *    diffuse image is the caller's fallback image (diffuse_image = -1).
 *  - Unsupported (RT_ERR_UNSUPPORTED): images given by URI, buffers other than
 *    the GLB's binary chunk, sparse accessors, primitives that are not indexed
 *    triangle lists.  Missing NORMAL or TEXCOORD_0, out-of-range accessors and
 *    indices past the primitive's vertices are RT_ERR_INVALID.
 */
#ifndef RTASSETS_H
#define RTASSETS_H

#include "rtcore.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Decodes a PNG file held in memory to RGBA8, row-major, no row padding.
 * With rgba8_out == NULL only *width / *height are written (header parse).
 * out_bytes must be at least width * height * 4. */
RTCORE_API int32_t rt_png_decode_rgba8(const void* bytes, uint64_t size, void* rgba8_out, uint64_t out_bytes,
                                       uint32_t* width, uint32_t* height);

typedef struct rt_glb_model rt_glb_model;   /* decoded model, host memory */

typedef struct RtGlbInfo {
    uint32_t vertex_count;      /* positions, normals and uvs each hold this many */
    uint32_t geometry_count;    /* one per material (1 without materials) */
    uint32_t image_count;       /* images in the reference's push order */
    uint32_t primitive_count;   /* mesh primitives read */
    uint64_t triangle_count;    /* over all geometries */
} RtGlbInfo;

typedef struct RtGlbGeometry {
    uint32_t index_count;               /* 3 per triangle */
    uint32_t opaque;                    /* 1: alphaMode OPAQUE (or no material) */
    int32_t diffuse_image;              /* model image slot; -1 = the caller's fallback image */
    int32_t metallic_roughness_image;   /* model image slot */
    int32_t normal_map_image;           /* model image slot; -1 = none */
    uint32_t _padding;
} RtGlbGeometry;

typedef struct RtGlbImage {
    uint32_t width;
    uint32_t height;
    uint32_t format;            /* RT_FORMAT_R8G8B8A8_SRGB / _UNORM or RT_FORMAT_R32G32B32A32_SFLOAT */
    uint32_t filter;            /* RT_FILTER_* */
    uint64_t byte_size;         /* width * height * 4 (RGBA8) or 16 (one RGBA32F texel) */
} RtGlbImage;

/* Parses a GLB file and decodes its images.  *out is released with
 * rt_glb_destroy. */
RTCORE_API int32_t rt_glb_load(const void* bytes, uint64_t size, rt_glb_model** out);
RTCORE_API int32_t rt_glb_info(const rt_glb_model* model, RtGlbInfo* info);
/* Copies the vertex arrays: positions and normals 3 floats per vertex, uvs
 * 2 floats per vertex.  Any pointer may be NULL to skip that array. */
RTCORE_API int32_t rt_glb_read_vertices(const rt_glb_model* model, float* positions, float* normals, float* uvs);
/* Describes geometry `index`; with indices != NULL also copies its index
 * array (capacity in elements, at least info->index_count). */
RTCORE_API int32_t rt_glb_read_geometry(const rt_glb_model* model, uint32_t index, RtGlbGeometry* info,
                                        uint32_t* indices, uint64_t capacity);
/* Describes image slot `index`; with texels != NULL also copies its texels
 * (capacity in bytes, at least info->byte_size). */
RTCORE_API int32_t rt_glb_read_image(const rt_glb_model* model, uint32_t index, RtGlbImage* info, void* texels,
                                     uint64_t capacity);
RTCORE_API int32_t rt_glb_destroy(rt_glb_model* model);

RT_STATIC_ASSERT(sizeof(RtGlbInfo) == 24, "RtGlbInfo is 24 bytes");
RT_STATIC_ASSERT(sizeof(RtGlbGeometry) == 24, "RtGlbGeometry is 24 bytes");
RT_STATIC_ASSERT(sizeof(RtGlbImage) == 24, "RtGlbImage is 24 bytes");

#ifdef __cplusplus
}
#endif

#endif /* RTASSETS_H */
