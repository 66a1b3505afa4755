// rt_shade.cuh — the reference's shader arithmetic on the device: software
// texture sampling, the alpha-clip any-hit, and the colour / ray-construction
// parts of the textured, mirror and portal closest-hits.  Included by
// rt_trace.cu only (anonymous-namespace definitions).
#pragma once

#include <cfloat>

#include "rt_device.cuh"

namespace rt {

// sRGB -> linear for 8-bit channels, filled once per context from the
// IEC 61966-2-1 formula evaluated in double (upload_srgb_table).
__constant__ float c_srgb_lut[256];

namespace {

constexpr float kPi = 3.141592653589793f;
constexpr uint32_t kNoHit = 0xFFFFFFFFu;

// What the device programs need about one scene: its TLAS, the push-constant
// model table and its bindless textures.  A batched launch keeps one per
// scene in device memory; the ray-buffer query holds its one in registers.
struct Env {
    const WideNode* tnodes;
    const InstRecord* insts;
    const RtModelInfo* models;      // may be null (no any-hit / closest-hit programs then)
    const RtTextureDesc* textures;  // texture_count entries
    uint32_t tnode_count;
    uint32_t inst_count;
    uint32_t texture_count;
    uint32_t blas_kinds;            // kBlasKind* bits of the TLAS's instances
};

__device__ __forceinline__ Env make_env(uint64_t tlas, uint64_t model_info, const RtTextureDesc* tex,
                                        uint32_t texture_count, uint32_t* status) {
    Env e;
    const uint8_t* base = reinterpret_cast<const uint8_t*>(tlas);
    const AsHeader* h = reinterpret_cast<const AsHeader*>(base);
    const bool ok = base != nullptr && h->magic == kAsMagic && h->type == kAsTypeTop;
    e.tnodes = ok ? reinterpret_cast<const WideNode*>(base + h->nodes_offset) : nullptr;
    e.insts = ok ? reinterpret_cast<const InstRecord*>(base + h->prims_offset) : nullptr;
    e.tnode_count = ok ? h->node_count : 0u;
    e.inst_count = ok ? h->prim_count : 0u;
    e.blas_kinds = ok ? h->blas_kinds : 0u;
    if (!ok) atomicOr(status, 1u << RT_ERR_BAD_AS);
    e.models = reinterpret_cast<const RtModelInfo*>(model_info);
    e.textures = tex;
    e.texture_count = tex ? texture_count : 0u;
    return e;
}

// ---------------------------------------------------------------------------
// Textures: software sampling, REPEAT, fixed arithmetic order (oracle twin).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int wrap_i(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

__device__ __forceinline__ float4 texel_fetch(const RtTextureDesc& t, int x, int y) {
    const uint8_t* row = reinterpret_cast<const uint8_t*>(t.address) + (size_t)y * t.row_pitch;
    if (t.format == RT_FORMAT_R32G32B32A32_SFLOAT) {
        return __ldg(reinterpret_cast<const float4*>(row) + x);
    }
    uint32_t p = __ldg(reinterpret_cast<const uint32_t*>(row) + x);
    uint32_t r = p & 0xFFu, g = (p >> 8) & 0xFFu, b = (p >> 16) & 0xFFu, a = p >> 24;
    float4 o;
    if (t.format == RT_FORMAT_R8G8B8A8_SRGB) {
        o.x = c_srgb_lut[r];
        o.y = c_srgb_lut[g];
        o.z = c_srgb_lut[b];
    } else {
        o.x = (float)r / 255.0f;
        o.y = (float)g / 255.0f;
        o.z = (float)b / 255.0f;
    }
    o.w = (float)a / 255.0f;
    return o;
}

__device__ float4 tex_sample(const RtTextureDesc& t, float u, float v) {
    if (t.address == 0 || t.width == 0 || t.height == 0) return make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    int w = (int)t.width, h = (int)t.height;
    if (t.filter == RT_FILTER_LINEAR) {
        float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
        float x0 = floorf(x), y0 = floorf(y);
        float fx = x - x0, fy = y - y0;
        int ix = wrap_i((int)fmaxf(fminf(x0, 2.0e9f), -2.0e9f), w);
        int iy = wrap_i((int)fmaxf(fminf(y0, 2.0e9f), -2.0e9f), h);
        int ix1 = ix + 1 == w ? 0 : ix + 1, iy1 = iy + 1 == h ? 0 : iy + 1;
        float4 t00 = texel_fetch(t, ix, iy), t10 = texel_fetch(t, ix1, iy);
        float4 t01 = texel_fetch(t, ix, iy1), t11 = texel_fetch(t, ix1, iy1);
        float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy);
        float w01 = (1.0f - fx) * fy, w11 = fx * fy;
        float4 o;
        o.x = ((w00 * t00.x + w10 * t10.x) + w01 * t01.x) + w11 * t11.x;
        o.y = ((w00 * t00.y + w10 * t10.y) + w01 * t01.y) + w11 * t11.y;
        o.z = ((w00 * t00.z + w10 * t10.z) + w01 * t01.z) + w11 * t11.z;
        o.w = ((w00 * t00.w + w10 * t10.w) + w01 * t01.w) + w11 * t11.w;
        return o;
    }
    float x = floorf(u * (float)w), y = floorf(v * (float)h);
    int ix = wrap_i((int)fmaxf(fminf(x, 2.0e9f), -2.0e9f), w);
    int iy = wrap_i((int)fmaxf(fminf(y, 2.0e9f), -2.0e9f), h);
    return texel_fetch(t, ix, iy);
}

__device__ __forceinline__ const RtHitGroup* hit_group(const RtShaderBindingTable* sbt, uint32_t sbt_flags,
                                                       uint32_t ray_sbt_offset) {
    if (!sbt) return nullptr;
    uint32_t gi = (sbt_flags & 0xFFFFFFu) + ray_sbt_offset;
    if (gi >= sbt->hit_group_count || gi >= RT_MAX_HIT_GROUPS) return nullptr;
    return &sbt->hit_groups[gi];
}

// any_hit_alpha_clip.glsl:11-29
__device__ __noinline__ bool alpha_clip_accepts(const RtModelInfo* models, const RtTextureDesc* textures,
                                                uint32_t texture_count, uint32_t custom, uint32_t geom, uint32_t prim,
                                                float u, float v) {
    const RtModelInfo m = models[custom];
    const RtGeometryInfo* gis = reinterpret_cast<const RtGeometryInfo*>(m.geometry_info_address);
    const RtGeometryInfo gi = gis[geom];
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(gi.index_buffer_address) + 3 * (size_t)prim;
    const float* uvs = reinterpret_cast<const float*>(m.uv_buffer_address);
    uint32_t i0 = idx[0], i1 = idx[1], i2 = idx[2];
    float w0 = (1.0f - u) - v;
    float uvx = (uvs[2 * i0] * w0 + uvs[2 * i1] * u) + uvs[2 * i2] * v;
    float uvy = (uvs[2 * i0 + 1] * w0 + uvs[2 * i1 + 1] * u) + uvs[2 * i2 + 1] * v;
    uint32_t ti = gi.images.diffuse_image_index;
    if (ti >= texture_count) return true;
    float4 c = tex_sample(textures[ti], uvx, uvy);
    return !(c.w < 0.5f);
}

// ---------------------------------------------------------------------------
// Shading (colour arithmetic; compared with a tolerance against the oracle)
// ---------------------------------------------------------------------------
__device__ __forceinline__ float clampf(float x, float lo, float hi) { return fminf(fmaxf(x, lo), hi); }

// pbr.glsl:56-65
__device__ __forceinline__ float v_smith_ggx_correlated(float NoV, float NoL, float roughness) {
    float a2 = roughness * roughness;
    float GGXV = NoL * sqrtf(NoV * NoV * (1.0f - a2) + a2);
    float GGXL = NoV * sqrtf(NoL * NoL * (1.0f - a2) + a2);
    return 0.5f / (GGXV + GGXL);
}
// pbr.glsl:44-51
__device__ __forceinline__ float d_ggx(float NoH, float roughness) {
    float a = NoH * roughness;
    float k = roughness / (1.0f - NoH * NoH + a * a);
    return k * k * (1.0f / kPi);
}
// pbr.glsl:74-76
__device__ __forceinline__ float f_schlick1(float u, float f0, float f90) {
    return f0 + (f90 - f0) * powf(1.0f - u, 5.0f);
}
// lib.rs:85-92
__device__ __forceinline__ float linear_to_srgb(float x) {
    if (x <= 0.0031308f) return x * 12.92f;
    return 1.055f * powf(x, 1.0f / 2.4f) - 0.055f;
}
__device__ __forceinline__ uint32_t to_unorm8(float x) {
    float c = fminf(fmaxf(x, 0.0f), 1.0f);
    return (uint32_t)(c * 255.0f + 0.5f);
}
// heatmap.rs:44-47
__device__ __forceinline__ float smoothstep(float e0, float e1, float x) {
    float t = clampf((x - e0) / (e1 - e0), 0.0f, 1.0f);
    return t * t * (3.0f - 2.0f * t);
}
// heatmap.rs:5-38 (index clamped to 9 at heat == 1)
__constant__ float c_heat_palette[10][3] = {
    {0.0f / 255.0f, 2.0f / 255.0f, 91.0f / 255.0f},     {0.0f / 255.0f, 108.0f / 255.0f, 251.0f / 255.0f},
    {0.0f / 255.0f, 221.0f / 255.0f, 221.0f / 255.0f},  {51.0f / 255.0f, 221.0f / 255.0f, 0.0f / 255.0f},
    {255.0f / 255.0f, 252.0f / 255.0f, 0.0f / 255.0f},  {255.0f / 255.0f, 180.0f / 255.0f, 0.0f / 255.0f},
    {255.0f / 255.0f, 104.0f / 255.0f, 0.0f / 255.0f},  {226.0f / 255.0f, 22.0f / 255.0f, 0.0f / 255.0f},
    {191.0f / 255.0f, 0.0f / 255.0f, 83.0f / 255.0f},   {145.0f / 255.0f, 0.0f / 255.0f, 65.0f / 255.0f},
};
__device__ V3 heatmap_temperature(float heat) {
    const float(*C)[3] = c_heat_palette;
    float h = clampf(heat, 0.0f, 1.0f) * 10.0f;
    int hi = (int)h;
    int cur = hi > 9 ? 9 : hi;
    int prv = hi - 1 > 0 ? hi - 1 : 0;
    if (prv > 9) prv = 9;
    int nxt = hi + 1 < 9 ? hi + 1 : 9;
    float hf = floorf(h), hc = -floorf(-h);
    float blur = 0.8f;
    float wc = smoothstep(hf - blur, hf + blur, h) * (1.0f - smoothstep(hc - blur, hc + blur, h));
    float wp = 1.0f - smoothstep(hf - blur, hf + blur, h);
    float wn = smoothstep(hc - blur, hc + blur, h);
    float r[3];
    for (int k = 0; k < 3; k++) r[k] = clampf(wc * C[cur][k] + wp * C[prv][k] + wn * C[nxt][k], 0.0f, 1.0f);
    return mk3(r[0], r[1], r[2]);
}

// pbr.glsl:174-211 split at the light intensity: out = (I * NoL) * comb.
__device__ void brdf_parts(V3 n, V3 v, V3 l, float pr, V3 base, float metallic, bool lambert, float* NoL_out,
                           V3* comb_out) {
    V3 h = normalize3(add3(v, l));
    float rough = pr * pr;
    float NoV = clampf(dot3(n, v), 10.0e-10f, 1.0f);
    float NoH = clampf(dot3(n, h), 0.0f, 1.0f);
    float NoL = clampf(dot3(n, l), 0.0f, 1.0f);
    float LoH = clampf(dot3(l, h), 0.0f, 1.0f);
    float D = d_ggx(NoH, rough);
    float dielectric_f0 = 0.16f * 0.5f * 0.5f;
    float f90 = 0.5f + 2.0f * rough * LoH * LoH;
    float V = v_smith_ggx_correlated(NoV, NoL, rough);
    float fd = lambert ? (1.0f / kPi) : f_schlick1(NoL, 1.0f, f90) * f_schlick1(NoV, 1.0f, f90) * (1.0f / kPi);
    float p5 = powf(1.0f - LoH, 5.0f);
    float b3[3] = {base.x, base.y, base.z};
    float c3[3];
    for (int k = 0; k < 3; k++) {
        float f0 = dielectric_f0 * (1.0f - metallic) + b3[k] * metallic;
        float F = f0 + (f90 - f0) * p5;
        float spec = (D * V) * F;
        float diff = b3[k] * fd;
        c3[k] = diff + spec;
    }
    *NoL_out = NoL;
    *comb_out = mk3(c3[0], c3[1], c3[2]);
}

struct TriData {
    V3 p[3], n[3];
    float uv[3][2];
    RtGeometryInfo gi;
};

// hit_shader_common.glsl:83-87,144-154
__device__ __forceinline__ bool load_triangle(const Env& e, uint32_t custom, uint32_t geom, uint32_t prim, TriData* td) {
    if (!e.models) return false;
    const RtModelInfo m = e.models[custom];
    const RtGeometryInfo* gis = reinterpret_cast<const RtGeometryInfo*>(m.geometry_info_address);
    td->gi = gis[geom];
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(td->gi.index_buffer_address) + 3 * (size_t)prim;
    const float* P = reinterpret_cast<const float*>(m.position_buffer_address);
    const float* N = reinterpret_cast<const float*>(m.normal_buffer_address);
    const float* UV = reinterpret_cast<const float*>(m.uv_buffer_address);
    for (int k = 0; k < 3; k++) {
        uint32_t i = idx[k];
        td->p[k] = mk3(P[3 * (size_t)i], P[3 * (size_t)i + 1], P[3 * (size_t)i + 2]);
        td->n[k] = mk3(N[3 * (size_t)i], N[3 * (size_t)i + 1], N[3 * (size_t)i + 2]);
        td->uv[k][0] = UV[2 * (size_t)i];
        td->uv[k][1] = UV[2 * (size_t)i + 1];
    }
    return true;
}

// closest_hit_textured.glsl:13-19
__device__ __forceinline__ V3 project_onto_tangent_plane(V3 point, V3 vp, V3 vn) {
    V3 vtp = sub3(point, vp);
    float dp = fminf(0.0f, dot3(vtp, vn));
    return sub3(vtp, mul3s(vn, dp));
}

// closest_hit_textured.glsl:99-111 (nearest-sampled texel of a 64-wide tile)
__device__ __forceinline__ float blue_noise_r(const Env& e, uint32_t tex, uint32_t x, uint32_t y, uint32_t ox,
                                              uint32_t oy) {
    if (tex >= e.texture_count) return 0.0f;
    float4 c = tex_sample(e.textures[tex], (float)(x + ox) / 64.0f, (float)(y + oy) / 64.0f);
    return c.x;
}

// closest_hit_textured.glsl:77-120: blue noise -> animated -> light sample
__device__ V3 shadow_direction(const Env& e, const RtUniforms& U, uint32_t x, uint32_t y, uint32_t i, V3 sun_dir) {
    float bx = blue_noise_r(e, U.blue_noise_texture_index, x, y, i * 2u * 13u, i * 2u * 41u);
    float by = blue_noise_r(e, U.blue_noise_texture_index, x, y, (i * 2u + 1u) * 13u, (i * 2u + 1u) * 41u);
    float g = (float)(U.frame_index % 32u) * 0.618033988749f;
    float sx = bx + g, sy = by + g;
    float rx = sx - floorf(sx), ry = sy - floorf(sy);
    float rad = sqrtf(rx);
    float ang = (ry * 2.0f) * kPi;
    float sn, cs;
    rt_sincos(ang, &sn, &cs);
    float px = (rad * cs) * U.sun_radius, py = (rad * sn) * U.sun_radius;
    V3 tangent = normalize3(cross3(sun_dir, mk3(0.0f, 1.0f, 0.0f)));
    V3 bitangent = normalize3(cross3(tangent, sun_dir));
    return normalize3(add3(add3(sun_dir, mul3s(tangent, px)), mul3s(bitangent, py)));
}

// Material + normal + BRDF terms of closest_hit_textured.glsl:174-226.
__device__ void shade_textured(const Env& e, const TriData& td, V3 inrm, float u_, float v_, const float* w2o,
                               V3 dir, V3 sun_dir, bool lambert, float* NoL, V3* comb, V3* amb) {
    const RtGeometryInfo& gi = td.gi;
    float4 dtex = make_float4(0, 0, 0, 0), mr = make_float4(0, 0, 0, 0);
    if (gi.images.diffuse_image_index < e.texture_count)
        dtex = tex_sample(e.textures[gi.images.diffuse_image_index], u_, v_);
    if (gi.images.metallic_roughness_image_index < e.texture_count)
        mr = tex_sample(e.textures[gi.images.metallic_roughness_image_index], u_, v_);
    float metallic = mr.z, roughness = mr.y;
    V3 base = mk3(dtex.x, dtex.y, dtex.z);
    V3 normal;
    int nmi = gi.images.normal_map_image_index;
    if (nmi < 0 || (uint32_t)nmi >= e.texture_count) {
        normal = normalize3(xform_normal_w2o_t(w2o, inrm));
    } else {
        float4 nm = tex_sample(e.textures[nmi], u_, v_);
        V3 map = mk3(nm.x * 2.0f - 1.0f, nm.y * 2.0f - 1.0f, nm.z * 2.0f - 1.0f);
        V3 dp1 = sub3(td.p[1], td.p[0]), dp2 = sub3(td.p[2], td.p[0]);
        float du1x = td.uv[1][0] - td.uv[0][0], du1y = td.uv[1][1] - td.uv[0][1];
        float du2x = td.uv[2][0] - td.uv[0][0], du2y = td.uv[2][1] - td.uv[0][1];
        V3 dp2perp = cross3(dp2, inrm), dp1perp = cross3(inrm, dp1);
        V3 T = add3(mul3s(dp2perp, du1x), mul3s(dp1perp, du2x));
        V3 B = add3(mul3s(dp2perp, du1y), mul3s(dp1perp, du2y));
        float tt = dot3(T, T), bb = dot3(B, B);
        float invmax = 1.0f / sqrtf(tt > bb ? tt : bb);
        V3 m = normalize3(map);
        V3 local = mk3((T.x * invmax * m.x + B.x * invmax * m.y) + inrm.x * m.z,
                       (T.y * invmax * m.x + B.y * invmax * m.y) + inrm.y * m.z,
                       (T.z * invmax * m.x + B.z * invmax * m.y) + inrm.z * m.z);
        normal = normalize3(xform_normal_w2o_t(w2o, local));
    }
    V3 view = mk3(-dir.x, -dir.y, -dir.z);
    brdf_parts(normal, view, sun_dir, roughness, base, metallic, lambert, NoL, comb);
    *amb = mk3(0.1f * base.x, 0.1f * base.y, 0.1f * base.z);
}

}  // namespace
}  // namespace rt
