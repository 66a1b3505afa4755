// rt_trace.cu — traversal and the reference's ray-tracing programs.
//
// Traversal (replaces the driver's traceRayEXT, called at
// shaders/ray-tracing/src/lib.rs:67-82,151-163 and
// shaders/closest_hit_textured.glsl:159-172): one ray per thread, explicit
// stack in local memory, 8-wide nodes read with 128-bit loads, the eight
// child slab tests sorted front-to-back with a 19-comparator network on
// (tnear bits | slot) keys, the watertight FP32 triangle test, alpha-clip
// any-hit inline for non-opaque geometry, and the closest hit chosen under
// the total order (t, instance index, geometry index, primitive index) so the
// result does not depend on the BVH or the visit order.
//
// Pipeline (replaces cmd_trace_rays with the reference's programs,
// src/command_buffer_recording.rs:116-126): a persistent kernel whose
// threads each run one pixel's raygen loop as a state machine — every loop
// iteration is exactly one traversal (bounce ray or shadow ray), so the warp
// stays in the traversal code regardless of which program each lane is in.
// Idle lanes fetch new pixels (warp-aggregated atomic on 8x4 pixel tiles).
#include <algorithm>
#include <cfloat>

#include "rt_internal.h"

namespace rt {

__constant__ float c_srgb_lut[256];

namespace {

constexpr uint32_t kStackSize = 64;
// Stack entries: internal node index (bit 31 clear, < 2^30); leaf =
// bit 31 | (count - 1) << 28 | first primitive; kMarker = return to the
// TLAS.  kNoEntry would be a leaf of 8 primitives starting at 2^28 - 1,
// which no structure can hold (primitive counts are < 2^28), so it is free
// to mean "stack empty".
constexpr uint32_t kMarker = 0x7FFFFFFFu;
constexpr uint32_t kLeafEntry = 0x80000000u;
constexpr uint32_t kNoEntry = 0xFFFFFFFFu;
constexpr float kPi = 3.141592653589793f;

struct Counters {
    uint32_t primary, secondary, shadow;
    uint32_t nodes, tris, insts;
};

struct Hit {
    float t, u, v;
    uint32_t inst;    // sorted TLAS index (kNoHit when none)
    uint32_t geom, prim;
    uint32_t inst_id; // caller's instance index (tie-break key)
    bool front;
};
constexpr uint32_t kNoHit = 0xFFFFFFFFu;

struct Env {
    const WideNode* tnodes;
    const InstRecord* insts;
    const RtModelInfo* models;   // may be null
    const RtShaderBindingTable* sbt;
    const RtTextureDesc* textures;
    uint32_t* status;
    uint32_t tnode_count;
    uint32_t inst_count;
};

// Upper bound of loop iterations of one traversal; reaching it means a
// malformed structure: the ray stops and RT_ERR_TIMEOUT is recorded.
constexpr uint32_t kMaxTraversalSteps = 1u << 22;

__device__ __forceinline__ Env make_env(uint64_t tlas, const RtPushConstantBufferAddresses& push,
                                        const RtShaderBindingTable* sbt, const RtTextureDesc* tex, uint32_t* status) {
    Env e;
    const uint8_t* base = reinterpret_cast<const uint8_t*>(tlas);
    const AsHeader* h = reinterpret_cast<const AsHeader*>(base);
    e.tnodes = reinterpret_cast<const WideNode*>(base + h->nodes_offset);
    e.insts = reinterpret_cast<const InstRecord*>(base + h->prims_offset);
    bool ok = h->magic == kAsMagic && h->type == kAsTypeTop;
    e.tnode_count = ok ? h->node_count : 0u;
    e.inst_count = ok ? h->prim_count : 0u;
    if (!ok) atomicOr(status, 1u << RT_ERR_BAD_AS);
    e.models = reinterpret_cast<const RtModelInfo*>(push.model_info);
    e.sbt = sbt;
    e.textures = tex;
    e.status = status;
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

__device__ __forceinline__ const RtHitGroup* hit_group(const Env& e, uint32_t sbt_flags, uint32_t ray_sbt_offset) {
    if (!e.sbt) return nullptr;
    uint32_t gi = (sbt_flags & 0xFFFFFFu) + ray_sbt_offset;
    if (gi >= e.sbt->hit_group_count || gi >= RT_MAX_HIT_GROUPS) return nullptr;
    return &e.sbt->hit_groups[gi];
}

// any_hit_alpha_clip.glsl:11-29
__device__ bool alpha_clip_accepts(const Env& e, uint32_t custom, uint32_t geom, uint32_t prim, float u, float v) {
    const RtModelInfo m = e.models[custom];
    const RtGeometryInfo* gis = reinterpret_cast<const RtGeometryInfo*>(m.geometry_info_address);
    const RtGeometryInfo gi = gis[geom];
    const uint32_t* idx = reinterpret_cast<const uint32_t*>(gi.index_buffer_address) + 3 * (size_t)prim;
    const float* uvs = reinterpret_cast<const float*>(m.uv_buffer_address);
    uint32_t i0 = idx[0], i1 = idx[1], i2 = idx[2];
    float w0 = (1.0f - u) - v;
    float uvx = (uvs[2 * i0] * w0 + uvs[2 * i1] * u) + uvs[2 * i2] * v;
    float uvy = (uvs[2 * i0 + 1] * w0 + uvs[2 * i1 + 1] * u) + uvs[2 * i2 + 1] * v;
    uint32_t ti = gi.images.diffuse_image_index;
    if (ti >= RT_MAX_BOUND_IMAGES) return true;
    float4 c = tex_sample(e.textures[ti], uvx, uvy);
    return !(c.w < 0.5f);
}

__device__ __forceinline__ bool id_less(uint32_t i, uint32_t g, uint32_t p, const Hit& b) {
    if (i != b.inst_id) return i < b.inst_id;
    if (g != b.geom) return g < b.geom;
    return p < b.prim;
}

__device__ __forceinline__ uint32_t pick8(const uint32_t v[8], uint32_t s) {
    uint32_t r = v[0];
#pragma unroll
    for (int j = 1; j < 8; j++) r = (s == (uint32_t)j) ? v[j] : r;
    return r;
}

#define RT_CSWAP(a, b)               \
    {                                \
        uint32_t lo_ = min(k[a], k[b]); \
        uint32_t hi_ = max(k[a], k[b]); \
        k[a] = lo_;                  \
        k[b] = hi_;                  \
    }

// Optimal 19-comparator sorting network for 8 keys.
__device__ __forceinline__ void sort8(uint32_t k[8]) {
    RT_CSWAP(0, 2) RT_CSWAP(1, 3) RT_CSWAP(4, 6) RT_CSWAP(5, 7)
    RT_CSWAP(0, 4) RT_CSWAP(1, 5) RT_CSWAP(2, 6) RT_CSWAP(3, 7)
    RT_CSWAP(0, 1) RT_CSWAP(2, 3) RT_CSWAP(4, 5) RT_CSWAP(6, 7)
    RT_CSWAP(2, 4) RT_CSWAP(3, 5)
    RT_CSWAP(1, 4) RT_CSWAP(3, 6)
    RT_CSWAP(1, 2) RT_CSWAP(3, 4) RT_CSWAP(5, 6)
}

// One traceRayEXT.  Returns with best.inst == kNoHit on a miss.
template <bool STATS>
__device__ void traverse(const Env& e, V3 wo, V3 wd, float tmin, float tmax, uint32_t ray_flags, uint32_t cull_mask,
                         uint32_t ray_sbt_offset, Hit& best, Counters& cnt) {
    best.t = tmax;
    best.u = best.v = 0.0f;
    best.inst = kNoHit;
    best.inst_id = kNoHit;
    best.geom = kNoHit;
    best.prim = kNoHit;
    best.front = false;
    const bool terminate_first = (ray_flags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT) != 0;

    uint2 stack[kStackSize];
    int sp = 0;

    V3 winv = safe_inv(wd);
    V3 o = wo, d = wd, inv = winv;
    WtRay wt;
    wt.kx = wt.ky = wt.kz = 0;
    wt.sx = wt.sy = wt.sz = 0.0f;
    const WideNode* nodes = e.tnodes;
    const TriRecord* tris = nullptr;
    uint32_t node_count = e.tnode_count, tri_count = 0;
    bool in_blas = false;
    // current instance
    uint32_t c_inst = 0, c_inst_id = 0, c_custom = 0, c_sbt_flags = 0;

    uint32_t entry = 0;  // TLAS root node
    if (node_count == 0) return;
    for (uint32_t steps = 0;; steps++) {
        if (steps >= kMaxTraversalSteps) {
            atomicOr(e.status, 1u << RT_ERR_TIMEOUT);
            return;
        }
        if (entry == kMarker) {
            in_blas = false;
            nodes = e.tnodes;
            node_count = e.tnode_count;
            o = wo;
            d = wd;
            inv = winv;
        } else if ((entry & kLeafEntry) == 0 && entry >= node_count) {
            atomicOr(e.status, 1u << RT_ERR_BAD_AS);  // malformed reference: skip it
        } else if ((entry & kLeafEntry) == 0) {
            // ---- wide node ----
            if (STATS) cnt.nodes++;
            const float4* np = reinterpret_cast<const float4*>(nodes + entry);
            float4 a0 = __ldg(np + 0), a1 = __ldg(np + 1), b0 = __ldg(np + 2), b1 = __ldg(np + 3);
            float4 c0 = __ldg(np + 4), c1 = __ldg(np + 5), d0 = __ldg(np + 6), d1 = __ldg(np + 7);
            float4 e0 = __ldg(np + 8), e1 = __ldg(np + 9), f0 = __ldg(np + 10), f1 = __ldg(np + 11);
            uint4 r0 = __ldg(reinterpret_cast<const uint4*>(np + 12));
            uint4 r1 = __ldg(reinterpret_cast<const uint4*>(np + 13));
            uint4 mm = __ldg(reinterpret_cast<const uint4*>(np + 14));
            const float lox[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
            const float hix[8] = {b0.x, b0.y, b0.z, b0.w, b1.x, b1.y, b1.z, b1.w};
            const float loy[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
            const float hiy[8] = {d0.x, d0.y, d0.z, d0.w, d1.x, d1.y, d1.z, d1.w};
            const float loz[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
            const float hiz[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
            const uint32_t refs[8] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w};
            const float tcap = best.t;
            uint32_t keys[8];
            uint32_t ents[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                float t0x = (lox[k] - o.x) * inv.x, t1x = (hix[k] - o.x) * inv.x;
                float t0y = (loy[k] - o.y) * inv.y, t1y = (hiy[k] - o.y) * inv.y;
                float t0z = (loz[k] - o.z) * inv.z, t1z = (hiz[k] - o.z) * inv.z;
                float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
                float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tcap));
                uint32_t m = node_meta(mm.x, mm.y, k);
                bool hit = (m != 0u) && (tn <= tf * kBoxFarScale);
                // key: tnear bits rounded down to 8 ulps | slot (ascending = near first)
                keys[k] = hit ? ((__float_as_uint(fmaxf(tn, 0.0f)) & ~7u) | (uint32_t)k) : 0xFFFFFFFFu;
                ents[k] = (m == kMetaInternal) ? refs[k] : (kLeafEntry | ((m - 1u) << 28) | refs[k]);
            }
            sort8(keys);
            if (keys[0] != 0xFFFFFFFFu) {
                // push the hit children farthest first; the nearest is next.
                // The stored tnear (key with the slot bits cleared) is rounded
                // down, so culling on pop stays conservative.
#pragma unroll
                for (int q = 7; q >= 1; q--) {
                    uint32_t key = keys[q];
                    if (key == 0xFFFFFFFFu) continue;
                    if (sp < (int)kStackSize) {
                        stack[sp++] = make_uint2(pick8(ents, key & 7u), key & ~7u);
                    } else {
                        atomicOr(e.status, 1u << RT_ERR_STACK_OVERFLOW);
                    }
                }
                entry = pick8(ents, keys[0] & 7u);
                continue;
            }
        } else {
            // ---- leaf ----
            uint32_t first = entry & 0x0FFFFFFFu;
            uint32_t count = ((entry >> 28) & 7u) + 1u;
            if (first + count > (in_blas ? tri_count : e.inst_count)) {
                atomicOr(e.status, 1u << RT_ERR_BAD_AS);  // malformed leaf: skip it
            } else if (!in_blas) {
                // instance leaf (one instance per TLAS leaf)
                const InstRecord* ir = &e.insts[first];
                uint32_t valid = __ldg(&ir->valid);
                uint32_t cm = __ldg(&ir->custom_mask);
                if (valid && ((cm >> 24) & cull_mask) != 0u) {
                    if (STATS) cnt.insts++;
                    const float4* wp = reinterpret_cast<const float4*>(ir->w2o);
                    float4 w0 = __ldg(wp), w1 = __ldg(wp + 1), w2 = __ldg(wp + 2);
                    const float w[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
                    o = xform_point(w, wo);
                    d = xform_dir(w, wd);
                    inv = safe_inv(d);
                    wt = wt_setup(d);
                    uint64_t blas = __ldg(reinterpret_cast<const unsigned long long*>(&ir->blas));
                    const uint8_t* bb = reinterpret_cast<const uint8_t*>(blas);
                    const AsHeader* bh = reinterpret_cast<const AsHeader*>(bb);
                    nodes = reinterpret_cast<const WideNode*>(bb + __ldg(reinterpret_cast<const unsigned long long*>(&bh->nodes_offset)));
                    tris = reinterpret_cast<const TriRecord*>(bb + __ldg(reinterpret_cast<const unsigned long long*>(&bh->prims_offset)));
                    node_count = __ldg(&bh->node_count);
                    tri_count = __ldg(&bh->prim_count);
                    c_inst = first;
                    c_inst_id = __ldg(&ir->instance_id);
                    c_custom = cm & 0xFFFFFFu;
                    c_sbt_flags = __ldg(&ir->sbt_flags);
                    in_blas = true;
                    if (sp < (int)kStackSize) {
                        stack[sp++] = make_uint2(kMarker, __float_as_uint(-INFINITY));
                        entry = 0;  // BLAS root
                        continue;
                    }
                    atomicOr(e.status, 1u << RT_ERR_STACK_OVERFLOW);
                    in_blas = false;
                    nodes = e.tnodes;
                    node_count = e.tnode_count;
                    o = wo;
                    d = wd;
                    inv = winv;
                }
            } else {
                const uint32_t iflags = c_sbt_flags >> 24;
                for (uint32_t q = 0; q < count; q++) {
                    if (STATS) cnt.tris++;
                    const float4* tp = reinterpret_cast<const float4*>(tris + first + q);
                    float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
                    uint32_t prim = __float_as_uint(p0.w), geom = __float_as_uint(p1.w), tf = __float_as_uint(p2.w);
                    bool opaque = (tf & 1u) != 0u;
                    if (iflags & RT_INSTANCE_FORCE_OPAQUE) opaque = true;
                    if (iflags & RT_INSTANCE_FORCE_NO_OPAQUE) opaque = false;
                    if (ray_flags & RT_RAY_FLAG_OPAQUE) opaque = true;
                    if (ray_flags & RT_RAY_FLAG_NO_OPAQUE) opaque = false;
                    if ((ray_flags & RT_RAY_FLAG_CULL_OPAQUE) && opaque) continue;
                    if ((ray_flags & RT_RAY_FLAG_CULL_NO_OPAQUE) && !opaque) continue;
                    float t, u, v;
                    bool front;
                    if (!tri_intersect(o, wt, mk3(p0.x, p0.y, p0.z), mk3(p1.x, p1.y, p1.z), mk3(p2.x, p2.y, p2.z), tmin,
                                       best.t, &t, &u, &v, &front))
                        continue;
                    if (iflags & RT_INSTANCE_TRIANGLE_FLIP_FACING) front = !front;
                    if (!(iflags & RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE)) {
                        if ((ray_flags & RT_RAY_FLAG_CULL_BACK_FACING) && !front) continue;
                        if ((ray_flags & RT_RAY_FLAG_CULL_FRONT_FACING) && front) continue;
                    }
                    if (t == best.t && best.inst != kNoHit && !id_less(c_inst_id, geom, prim, best)) continue;
                    if (!opaque && e.models) {
                        const RtHitGroup* g = hit_group(e, c_sbt_flags, ray_sbt_offset);
                        if (g && g->any_hit == RT_PROGRAM_ANY_HIT_ALPHA_CLIP &&
                            !alpha_clip_accepts(e, c_custom, geom, prim, u, v))
                            continue;
                    }
                    best.t = t;
                    best.u = u;
                    best.v = v;
                    best.inst = c_inst;
                    best.inst_id = c_inst_id;
                    best.geom = geom;
                    best.prim = prim;
                    best.front = front;
                    if (terminate_first) return;
                }
            }
        }
        // ---- pop ----
        entry = kNoEntry;
        const float cull = best.t * kBoxFarScale;
        while (sp > 0) {
            uint2 s = stack[--sp];
            if (s.x != kMarker && __uint_as_float(s.y) > cull) continue;
            entry = s.x;
            break;
        }
        if (entry == kNoEntry) return;
    }
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
    if (tex >= RT_MAX_BOUND_IMAGES) return 0.0f;
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
    if (gi.images.diffuse_image_index < RT_MAX_BOUND_IMAGES)
        dtex = tex_sample(e.textures[gi.images.diffuse_image_index], u_, v_);
    if (gi.images.metallic_roughness_image_index < RT_MAX_BOUND_IMAGES)
        mr = tex_sample(e.textures[gi.images.metallic_roughness_image_index], u_, v_);
    float metallic = mr.z, roughness = mr.y;
    V3 base = mk3(dtex.x, dtex.y, dtex.z);
    V3 normal;
    int nmi = gi.images.normal_map_image_index;
    if (nmi < 0 || (uint32_t)nmi >= RT_MAX_BOUND_IMAGES) {
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

__device__ __forceinline__ void flush_counters(RtStats* st, const Counters& c) {
    atomicAdd(reinterpret_cast<unsigned long long*>(&st->traversals),
              (unsigned long long)(c.primary + c.secondary + c.shadow));
    atomicAdd(reinterpret_cast<unsigned long long*>(&st->primary_rays), (unsigned long long)c.primary);
    atomicAdd(reinterpret_cast<unsigned long long*>(&st->secondary_rays), (unsigned long long)c.secondary);
    atomicAdd(reinterpret_cast<unsigned long long*>(&st->shadow_rays), (unsigned long long)c.shadow);
    if (c.nodes | c.tris | c.insts) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->nodes_visited), (unsigned long long)c.nodes);
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->triangles_tested), (unsigned long long)c.tris);
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->instances_visited), (unsigned long long)c.insts);
    }
}

struct TraceParams {
    TraceLaunch L;
    uint32_t tiles_x;
    uint32_t total;        // tiles * 32
    uint32_t* work;        // fetch counter (zeroed before launch)
};

constexpr uint32_t kPhaseRay = 0;
constexpr uint32_t kPhaseShadow = 1;

// ray_generation (lib.rs:95-191) as a per-pixel state machine.
template <bool STATS>
__global__ void __launch_bounds__(128) k_trace_rays(const __grid_constant__ TraceParams P) {
    const TraceLaunch& L = P.L;
    const RtUniforms& U = *reinterpret_cast<const RtUniforms*>(L.push.uniforms);
    const Env e = make_env(L.push.acceleration_structure, L.push, &L.sbt, L.textures, L.status);
    const uint32_t W = L.desc.width, H = L.desc.height;
    const uint32_t max_depth = L.desc.max_trace_depth;
    const uint32_t nshadow = L.desc.shadow_ray_count;
    const bool lambert = (L.desc.flags & RT_TRACE_FLAG_LAMBERT_DIFFUSE) != 0;
    const V3 sun_dir = mk3(U.sun_dir[0], U.sun_dir[1], U.sun_dir[2]);
    float sun_s, sun_c;
    rt_sincos(U.sun_radius, &sun_s, &sun_c);
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    uint32_t* img = reinterpret_cast<uint32_t*>(L.desc.image_address);
    float4* rad = reinterpret_cast<float4*>(L.desc.radiance_address);

    Counters cnt = {0, 0, 0, 0, 0, 0};
    bool has = false;
    uint32_t x = 0, y = 0, phase = kPhaseRay, bounce = 0, shadow_i = 0;
    V3 ro = mk3(0, 0, 0), rd = mk3(0, 0, 0), so = mk3(0, 0, 0), comb = mk3(0, 0, 0), amb = mk3(0, 0, 0);
    V3 col = mk3(0, 0, 0);
    float NoL = 0.0f, lit = 0.0f;
    long long t_start = 0;

    for (;;) {
        // ---- refill idle lanes (warp-aggregated fetch of tile pixels) ----
        unsigned m = __activemask();
        unsigned idle = __ballot_sync(m, !has);
        if (idle) {
            int leader = __ffs(idle) - 1;
            uint32_t base = 0;
            if ((int)lane == leader) base = atomicAdd(P.work, (uint32_t)__popc(idle));
            base = __shfl_sync(m, base, leader);
            if (!has) {
                uint32_t my = base + __popc(idle & lanemask_lt);
                while (my < P.total) {
                    uint32_t tile = my >> 5, l = my & 31u;
                    uint32_t tx = tile % P.tiles_x, ty = tile / P.tiles_x;
                    x = tx * 8u + (l & 7u);
                    y = ty * 4u + (l >> 3);
                    if (x < W && y < H) {
                        has = true;
                        break;
                    }
                    my = atomicAdd(P.work, 1u);  // outside the image: take another
                }
                if (has) {
                    if (U.show_heatmap) t_start = clock64();
                    // lib.rs:126-142
                    float pcx = (float)x + 0.5f, pcy = (float)y + 0.5f;
                    float tcx = pcx / (float)W, tcy = pcy / (float)H;
                    float rx = tcx * 2.0f - 1.0f, ry = tcy * 2.0f - 1.0f;
                    const float* VI = U.view_inverse;
                    const float* PI = U.proj_inverse;
                    ro = mk3(mat4_row(VI, 0, 0.0f, 0.0f, 0.0f, 1.0f), mat4_row(VI, 1, 0.0f, 0.0f, 0.0f, 1.0f),
                             mat4_row(VI, 2, 0.0f, 0.0f, 0.0f, 1.0f));
                    V3 target = mk3(mat4_row(PI, 0, rx, ry, 1.0f, 1.0f), mat4_row(PI, 1, rx, ry, 1.0f, 1.0f),
                                    mat4_row(PI, 2, rx, ry, 1.0f, 1.0f));
                    V3 local = normalize3(target);
                    rd = mk3(mat4_row(VI, 0, local.x, local.y, local.z, 0.0f),
                             mat4_row(VI, 1, local.x, local.y, local.z, 0.0f),
                             mat4_row(VI, 2, local.x, local.y, local.z, 0.0f));
                    phase = kPhaseRay;
                    bounce = 0;
                    col = mk3(0, 0, 0);
                }
            }
        }
        if (!has) break;

        bool done = false;
        Hit h;
        if (phase == kPhaseRay) {
            if (bounce == 0) cnt.primary++;
            else cnt.secondary++;
            traverse<STATS>(e, ro, rd, 0.01f, 10000.0f, RT_RAY_FLAG_NONE, 0xFFu, 0u, h, cnt);
            col = mk3(0, 0, 0);  // payload reset (lib.rs:145-149)
            V3 nd = mk3(0, 0, 0), no = mk3(0, 0, 0);
            if (h.inst == kNoHit) {
                // primary_ray_miss (lib.rs:40-51)
                col = dot3(rd, sun_dir) > sun_c ? mk3(1.0f, 1.0f, 1.0f) : mk3(0.0f, 0.0f, 0.05f);
                done = true;
            } else {
                const InstRecord* ir = &e.insts[h.inst];
                uint32_t sbt_flags = ir->sbt_flags;
                uint32_t custom = ir->custom_mask & 0xFFFFFFu;
                const RtHitGroup* g = hit_group(e, sbt_flags, 0u);
                uint32_t prog = g ? g->closest_hit : RT_PROGRAM_NONE;
                V3 bary = mk3((1.0f - h.u) - h.v, h.u, h.v);
                TriData td;
                if (prog == RT_PROGRAM_CLOSEST_HIT_MIRROR && load_triangle(e, custom, h.geom, h.prim, &td)) {
                    // closest_hit_mirror.glsl:11-29
                    V3 ni = interp3(td.n[0], td.n[1], td.n[2], bary);
                    V3 n = normalize3(xform_normal_w2o_t(ir->w2o, ni));
                    float k = 2.0f * dot3(n, rd);
                    nd = sub3(rd, mul3s(n, k));
                    no = add3(ro, mul3s(rd, h.t));
                } else if (prog == RT_PROGRAM_CLOSEST_HIT_PORTAL) {
                    // lib.rs:300-312
                    nd = rd;
                    no = add3(add3(ro, mul3s(rd, h.t)), mk3(0.0f, 5.0f, 0.0f));
                } else if (prog == RT_PROGRAM_CLOSEST_HIT_TEXTURED && load_triangle(e, custom, h.geom, h.prim, &td)) {
                    // closest_hit_textured.glsl:174-226
                    V3 ip = interp3(td.p[0], td.p[1], td.p[2], bary);
                    V3 inrm = interp3(td.n[0], td.n[1], td.n[2], bary);
                    float iu = (td.uv[0][0] * bary.x + td.uv[1][0] * bary.y) + td.uv[2][0] * bary.z;
                    float iv = (td.uv[0][1] * bary.x + td.uv[1][1] * bary.y) + td.uv[2][1] * bary.z;
                    V3 oa = project_onto_tangent_plane(ip, td.p[0], td.n[0]);
                    V3 ob = project_onto_tangent_plane(ip, td.p[1], td.n[1]);
                    V3 oc = project_onto_tangent_plane(ip, td.p[2], td.n[2]);
                    V3 off = interp3(oa, ob, oc, bary);
                    so = xform_point(ir->o2w, add3(ip, off));
                    shade_textured(e, td, inrm, iu, iv, ir->w2o, rd, sun_dir, lambert, &NoL, &comb, &amb);
                    if (nshadow > 0) {
                        phase = kPhaseShadow;
                        shadow_i = 0;
                        lit = 0.0f;
                    } else {
                        float sf = 0.0f;
                        col = mk3((sf * NoL) * comb.x + amb.x, (sf * NoL) * comb.y + amb.y,
                                  (sf * NoL) * comb.z + amb.z);
                        done = true;
                    }
                }
                if (phase == kPhaseRay && !done) {
                    // break when new_ray_direction == 0 (lib.rs:165-171)
                    if (nd.x == 0.0f && nd.y == 0.0f && nd.z == 0.0f) {
                        done = true;
                    } else {
                        ro = no;
                        rd = nd;
                        bounce++;
                        if (bounce >= max_depth) done = true;  // colour stays reset
                    }
                }
            }
        } else {
            cnt.shadow++;
            V3 sd = shadow_direction(e, U, x, y, shadow_i, sun_dir);
            traverse<STATS>(e, so, sd, 0.001f, 10000.0f,
                            RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT | RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER, 0xFFu, 1u, h,
                            cnt);
            lit += (h.inst == kNoHit) ? 1.0f : 0.0f;  // shadow_ray_miss clears `shadowed`
            shadow_i++;
            if (shadow_i >= nshadow) {
                float sf = lit / (float)nshadow;
                col = mk3((sf * NoL) * comb.x + amb.x, (sf * NoL) * comb.y + amb.y, (sf * NoL) * comb.z + amb.z);
                done = true;
            }
        }
        if (done) {
            V3 c = col;
            if (U.show_heatmap) {
                long long dt = clock64() - t_start;
                V3 hm = heatmap_temperature((float)dt / 1000000.0f);
                c = add3(hm, mul3s(col, 0.000001f));
            }
            size_t pix = (size_t)y * W + x;
            if (rad) rad[pix] = make_float4(c.x, c.y, c.z, 1.0f);
            if (img) {
                uint32_t r = to_unorm8(linear_to_srgb(c.x)), g = to_unorm8(linear_to_srgb(c.y));
                uint32_t b = to_unorm8(linear_to_srgb(c.z));
                img[pix] = r | (g << 8) | (b << 16) | (255u << 24);
            }
            has = false;
        }
    }
    flush_counters(L.stats, cnt);
}

struct RayBufferParams {
    RayBufferLaunch L;
};

template <bool STATS>
__global__ void __launch_bounds__(128) k_trace_ray_buffer(const __grid_constant__ RayBufferParams P) {
    const RayBufferLaunch& L = P.L;
    const Env e = make_env(L.tlas, L.push, &L.sbt, L.textures, L.status);
    Counters cnt = {0, 0, 0, 0, 0, 0};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < L.count; i += gridDim.x * blockDim.x) {
        const float4* rp = reinterpret_cast<const float4*>(L.rays + i);
        float4 a = __ldg(rp), b = __ldg(rp + 1);
        Hit h;
        cnt.primary++;
        traverse<STATS>(e, mk3(a.x, a.y, a.z), mk3(b.x, b.y, b.z), a.w, b.w, L.ray_flags, L.cull_mask, L.sbt_offset,
                        h, cnt);
        RtHit o;
        if (h.inst != kNoHit) {
            const InstRecord* ir = &e.insts[h.inst];
            o.t = h.t;
            o.u = h.u;
            o.v = h.v;
            o.instance_id = h.inst_id;
            o.instance_custom_index = ir->custom_mask & 0xFFFFFFu;
            o.geometry_index = h.geom;
            o.primitive_index = h.prim;
            o.hit_kind = h.front ? 0xFEu : 0xFFu;
        } else {
            o.t = b.w;
            o.u = o.v = 0.0f;
            o.instance_id = o.instance_custom_index = o.geometry_index = o.primitive_index = 0xFFFFFFFFu;
            o.hit_kind = 0;
        }
        uint4* hp = reinterpret_cast<uint4*>(L.hits + i);
        const uint4* op = reinterpret_cast<const uint4*>(&o);
        hp[0] = op[0];
        hp[1] = op[1];
    }
    flush_counters(L.stats, cnt);
}

__global__ void k_debug_eval(uint32_t fn, const float* in, float* out, uint32_t count) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    switch (fn) {
        case RT_FN_V_SMITH_GGX_CORRELATED:
            out[i] = v_smith_ggx_correlated(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
            break;
        case RT_FN_D_GGX:
            out[i] = d_ggx(in[2 * i], in[2 * i + 1]);
            break;
        case RT_FN_LINEAR_TO_SRGB:
            out[i] = linear_to_srgb(in[i]);
            break;
        case RT_FN_HEATMAP: {
            V3 c = heatmap_temperature(in[i]);
            out[3 * i] = c.x;
            out[3 * i + 1] = c.y;
            out[3 * i + 2] = c.z;
            break;
        }
        case RT_FN_SINCOS:
            rt_sincos(in[i], &out[2 * i], &out[2 * i + 1]);
            break;
        case RT_FN_BRDF: {
            const float* p = in + 16 * (size_t)i;
            float NoL;
            V3 comb;
            brdf_parts(mk3(p[0], p[1], p[2]), mk3(p[3], p[4], p[5]), mk3(p[6], p[7], p[8]), p[9],
                       mk3(p[10], p[11], p[12]), p[13], p[15] != 0.0f, &NoL, &comb);
            float I = p[14];
            out[3 * i] = (I * NoL) * comb.x;
            out[3 * i + 1] = (I * NoL) * comb.y;
            out[3 * i + 2] = (I * NoL) * comb.z;
            break;
        }
        case RT_FN_WATERTIGHT: {
            const float* p = in + 16 * (size_t)i;
            V3 o = mk3(p[0], p[1], p[2]), d = mk3(p[3], p[4], p[5]);
            WtRay w = wt_setup(d);
            float t = 0, u = 0, v = 0;
            bool front = false;
            bool hit = tri_intersect(o, w, mk3(p[6], p[7], p[8]), mk3(p[9], p[10], p[11]), mk3(p[12], p[13], p[14]),
                                     p[15], INFINITY, &t, &u, &v, &front);
            out[4 * i] = hit ? (front ? 1.0f : -1.0f) : 0.0f;
            out[4 * i + 1] = hit ? t : 0.0f;
            out[4 * i + 2] = hit ? u : 0.0f;
            out[4 * i + 3] = hit ? v : 0.0f;
            break;
        }
        default:
            break;
    }
}

template <class K>
int persistent_blocks(K kernel, int threads, int num_sms) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, 0) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * num_sms;
}

}  // namespace

cudaError_t launch_trace_rays(const TraceLaunch& p, int num_sms, cudaStream_t stream) {
    TraceParams P;
    P.L = p;
    P.tiles_x = (p.desc.width + 7) / 8;
    uint32_t tiles_y = (p.desc.height + 3) / 4;
    P.total = P.tiles_x * tiles_y * 32u;
    P.work = p.work;
    cudaError_t err = cudaMemsetAsync(P.work, 0, sizeof(uint32_t), stream);
    if (err != cudaSuccess) return err;
    const bool stats = (p.desc.flags & RT_TRACE_FLAG_COLLECT_STATS) != 0;
    if (stats) {
        int blocks = persistent_blocks(k_trace_rays<true>, 128, num_sms);
        note_launch(), k_trace_rays<true><<<blocks, 128, 0, stream>>>(P);
    } else {
        int blocks = persistent_blocks(k_trace_rays<false>, 128, num_sms);
        note_launch(), k_trace_rays<false><<<blocks, 128, 0, stream>>>(P);
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_ray_buffer(const RayBufferLaunch& p, int num_sms, cudaStream_t stream) {
    RayBufferParams P;
    P.L = p;
    if (p.count == 0) return cudaSuccess;
    uint32_t blocks = (p.count + 127) / 128;
    if (p.collect_stats) {
        int maxb = persistent_blocks(k_trace_ray_buffer<true>, 128, num_sms);
        note_launch(), k_trace_ray_buffer<true><<<std::min<uint32_t>(blocks, (uint32_t)maxb * 8u), 128, 0, stream>>>(P);
    } else {
        int maxb = persistent_blocks(k_trace_ray_buffer<false>, 128, num_sms);
        note_launch(), k_trace_ray_buffer<false><<<std::min<uint32_t>(blocks, (uint32_t)maxb * 8u), 128, 0, stream>>>(P);
    }
    return cudaGetLastError();
}

cudaError_t launch_debug_eval(uint32_t fn, const float* in, float* out, uint32_t count, cudaStream_t stream) {
    if (count == 0) return cudaSuccess;
    note_launch(), k_debug_eval<<<(count + 127) / 128, 128, 0, stream>>>(fn, in, out, count);
    return cudaGetLastError();
}

cudaError_t upload_srgb_table() {
    float lut[256];
    for (int i = 0; i < 256; i++) {
        double c = i / 255.0;
        double l = c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
        lut[i] = (float)l;
    }
    return cudaMemcpyToSymbol(c_srgb_lut, lut, sizeof lut);
}

}  // namespace rt
