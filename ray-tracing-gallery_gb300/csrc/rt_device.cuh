// rt_device.cuh — device-side layouts and fixed-order FP32 helpers.
//
// Every translation unit that includes this header is compiled with
// -fmad=false: the geometric part of the pipeline (ray generation, instance
// transforms, the watertight triangle test, shadow / reflection ray
// construction) must round after every operation in the order written here,
// because the CPU oracle performs the same operations in the same order and
// hit IDs are compared bit for bit.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rtcore.h"

namespace rt {

// ---------------------------------------------------------------------------
// Acceleration-structure blob layout (position independent: offsets only)
// ---------------------------------------------------------------------------
constexpr uint32_t kAsMagic = 0x53415452u;  // "RTAS"
constexpr uint32_t kAsTypeBottom = 0;
constexpr uint32_t kAsTypeTop = 1;
constexpr uint32_t kHeaderBytes = 512;
constexpr uint32_t kNodeBytes = 256;
constexpr uint32_t kTriBytes = 48;
constexpr uint32_t kInstBytes = 128;
// Triangles per BLAS leaf child.  Measured on one GB300 with PLOC trees
// (Mrays/s, 1080p frame / 10.5M-triangle precision mesh FP32 / 720p default
// scene): 1 -> 967 / 2142 / 2137, 2 -> 1000 / 2223 / 2557,
// 3 -> 995 / 2182 / 2567, 4 -> 922 / 2043 / 2670, 8 -> 832 / 1748 / 2528.
constexpr uint32_t kBlasLeafMax = 2;
constexpr uint32_t kTlasLeafMax = 1;   // instances per leaf child
constexpr uint32_t kDopMaxVertices = 24;  // a 14-DOP (cube with cut corners) has at most 24
constexpr uint32_t kWide = 8;

struct AsHeader {
    uint32_t magic;
    uint32_t type;
    uint32_t build_flags;
    uint32_t status;          // RT_OK or a device-side build error
    uint32_t node_count;      // wide nodes written
    uint32_t prim_count;      // triangles or instances
    uint32_t max_nodes;       // node capacity
    uint32_t node_bytes;
    uint64_t total_size;      // bytes of the blob at capacity
    uint64_t nodes_offset;
    uint64_t prims_offset;
    uint64_t parents_offset;  // uint32 parent index per node (TLAS refit)
    float bounds_lo[3];
    float bounds_hi[3];
    uint32_t geometry_count;
    uint32_t depth;
    uint32_t leaf_max;
    uint32_t blas_kinds;      // TLAS: kBlasKind* bits of the BLASes its instances enter
    uint64_t compacted_size;
    // BLAS: a sphere holding every triangle (centre = centre of bounds_lo / hi,
    // radius rounded up); radius 0 = none.  An instance's world box is its
    // transformed bounds box cut to the transformed sphere's box.
    float sphere_center[3];
    float sphere_radius;
    // BLAS: the vertices of a 14-DOP holding every triangle (the 6 axis and
    // 8 diagonal (+-1, +-1, +-1) planes at the triangles' extreme
    // projections); 0 = none.  The instance box is also cut to the box of
    // these vertices transformed.
    uint32_t dop_count;
    uint32_t _dop_pad[3];
    float dop_vertex[kDopMaxVertices][3];
    uint8_t _pad[kHeaderBytes - 144 - 12 * kDopMaxVertices];
};
static_assert(sizeof(AsHeader) == kHeaderBytes, "header size");

// 8-wide node, SoA child boxes.  Children are packed at the front.
// child_ref is the traversal's stack entry for the child: an internal child
// is its node index (< 2^30); a leaf is kChildLeaf | (count - 1) << 28 |
// first primitive (sorted order, < 2^28); an empty slot is kChildEmpty.
// meta byte c (meta[0] holds children 0-3, meta[1] children 4-7, low byte
// first) repeats the kind for the refit: 0 = empty, kMetaInternal =
// internal, 1..8 = leaf with that many primitives.
constexpr uint32_t kMetaInternal = 0x80u;
constexpr uint32_t kChildLeaf = 0x80000000u;
constexpr uint32_t kChildEmpty = 0xFFFFFFFFu;
struct alignas(128) WideNode {
    float lox[8], hix[8], loy[8], hiy[8], loz[8], hiz[8];
    uint32_t child_ref[8];
    uint32_t meta[2];
    uint32_t _pad[6];
};
static_assert(sizeof(WideNode) == kNodeBytes, "node size");
__host__ __device__ inline uint32_t node_meta(uint32_t m0, uint32_t m1, int c) {
    return ((c < 4 ? m0 : m1) >> (8 * (c & 3))) & 0xFFu;
}

// 8-wide node with 8-bit quantised child boxes (RT_BUILD_QUANTIZED_NODES,
// BLAS only), 96 bytes.  Per axis a: quantum s_a = 2^(exp[a] - 127); child
// k's planes are origin_a + q * s_a with q = qlo / qhi bytes.  The builder
// puts origin on the quantum grid one quantum below the node's union box and
// rounds every child plane outward to the grid with at least kQuantSlack of
// a quantum to spare, so the decoded box contains the padded FP32 child box
// (the traversal's test of it is widened by a bound of its own rounding
// error, so it is never narrower than the exact test of the decoded box); an
// empty child is qlo = 255, qhi = 0 (never hit).
// child_ref is as in WideNode.
constexpr uint32_t kQNodeBytes = 96;
constexpr float kQuantSlack = 0.25f;
// Widening of the quantised slab test (rt_trace.cu, qnode_keys): each plane
// distance moves out by kQuantMargin quanta, the entry / exit distances by
// kQuantRelative of themselves (16 u, u = 2^-24).
constexpr float kQuantMargin = 0.008f;
constexpr float kQuantRelative = 9.5367431640625e-07f;
struct alignas(16) QNode {
    float origin[3];
    uint8_t exp[3];
    uint8_t _pad;
    uint32_t child_ref[8];
    uint8_t qlo_x[8], qhi_x[8], qlo_y[8], qhi_y[8], qlo_z[8], qhi_z[8];
};
static_assert(sizeof(QNode) == kQNodeBytes, "qnode size");
// InstRecord.node_count bit marking a BLAS with quantised nodes.
constexpr uint32_t kQuantizedBlasBit = 0x80000000u;
// AsHeader.blas_kinds bits of a TLAS: which node formats its instances use
// (the traversal kernels pick a loop that handles exactly those).
constexpr uint32_t kBlasKindF32 = 1u, kBlasKindQ8 = 2u;
__host__ __device__ __forceinline__ uint32_t blas_kind(uint32_t inst_node_count) {
    return (inst_node_count & kQuantizedBlasBit) ? kBlasKindQ8 : kBlasKindF32;
}

// Triangle record: v0.w = primitive index, v1.w = geometry index,
// v2.w = flags (bit 0 opaque).  Stored in leaf (sorted) order.
struct alignas(16) TriRecord {
    float4 v0, v1, v2;
};
static_assert(sizeof(TriRecord) == kTriBytes, "tri size");

// TLAS instance record, sorted order.  The last 32 bytes are read with two
// 128-bit loads when a ray enters the instance: they carry everything the
// traversal needs from the BLAS header, so the header is never read then.
struct alignas(16) InstRecord {
    float w2o[12];           // world -> object, row-major 3x4
    float o2w[12];           // object -> world (the instance transform)
    uint64_t blas;           // @96 BLAS address
    uint32_t instance_id;    // @104 index in the caller's instance array
    uint32_t custom_mask;    // @108 custom index (24) | mask (8) << 24
    uint32_t sbt_flags;      // @112 SBT offset (24) | flags (8) << 24
    uint32_t tri_count;      // @116 BLAS triangles; 0 = never hit (singular transform, null or empty BLAS)
    uint32_t node_count;     // @120 BLAS wide nodes
    uint32_t prims_off256;   // @124 BLAS triangle records offset / 256
};
static_assert(sizeof(InstRecord) == kInstBytes, "inst size");

__host__ __device__ inline uint64_t align_up(uint64_t x, uint64_t a) { return (x + a - 1) / a * a; }

// Upper bound of wide nodes for n primitives (see the collapse rule in
// rt_build.cu): non-full nodes have >= 2 leaf children (<= n/2 of them),
// full nodes absorb 7 binary nodes each (<= (n-1)/7), plus the root.
__host__ __device__ inline uint64_t max_wide_nodes(uint64_t n, uint32_t width = 8) {
    if (n <= 1) return 1;
    if (width <= 4) return n + 2;  // every wide node owns a distinct binary node
    return n / 2 + (n - 1) / 7 + 2;
}
// Children per node a build produces (RT_BUILD_EXT_NODE_WIDTH_4: 4, else 8).
__host__ __device__ inline uint32_t node_width(uint32_t build_flags) {
    return (build_flags & RT_BUILD_EXT_NODE_WIDTH_4) ? 4u : 8u;
}

// ---------------------------------------------------------------------------
// Fixed-order FP32 helpers (identical sequences exist in the oracle)
// ---------------------------------------------------------------------------
struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 mk3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 add3(V3 a, V3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 sub3(V3 a, V3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 mul3s(V3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ float dot3(V3 a, V3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
__device__ __forceinline__ V3 cross3(V3 a, V3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
// glam Vec3::normalize form: v * (1 / sqrt(dot(v, v))); sqrtf and the
// division are IEEE correctly rounded (no fast-math).
__device__ __forceinline__ V3 normalize3(V3 v) {
    float inv = 1.0f / sqrtf(dot3(v, v));
    return mul3s(v, inv);
}
__device__ __forceinline__ V3 interp3(V3 a, V3 b, V3 c, V3 w) {
    return add3(add3(mul3s(a, w.x), mul3s(b, w.y)), mul3s(c, w.z));
}
__device__ __forceinline__ float get3(V3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }
__device__ __forceinline__ float mat4_row(const float* m, int i, float x, float y, float z, float w) {
    return ((m[0 * 4 + i] * x + m[1 * 4 + i] * y) + m[2 * 4 + i] * z) + m[3 * 4 + i] * w;
}
__device__ __forceinline__ V3 xform_point(const float* m, V3 p) {
    return mk3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3], ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
               ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
__device__ __forceinline__ V3 xform_dir(const float* m, V3 d) {
    return mk3((m[0] * d.x + m[1] * d.y) + m[2] * d.z, (m[4] * d.x + m[5] * d.y) + m[6] * d.z,
               (m[8] * d.x + m[9] * d.y) + m[10] * d.z);
}
// mat3(gl_WorldToObject3x4EXT) * n
__device__ __forceinline__ V3 xform_normal_w2o_t(const float* w, V3 n) {
    return mk3((w[0] * n.x + w[4] * n.y) + w[8] * n.z, (w[1] * n.x + w[5] * n.y) + w[9] * n.z,
               (w[2] * n.x + w[6] * n.y) + w[10] * n.z);
}

// Inverse of a row-major 3x4 affine by the adjugate, fixed order.  Returns
// false for a singular (or non-finite) transform.
__host__ __device__ inline bool affine_inverse(const float* m, float* w) {
    float m00 = m[0], m01 = m[1], m02 = m[2], m10 = m[4], m11 = m[5], m12 = m[6];
    float m20 = m[8], m21 = m[9], m22 = m[10];
    float c00 = m11 * m22 - m12 * m21;
    float c01 = m12 * m20 - m10 * m22;
    float c02 = m10 * m21 - m11 * m20;
    float det = (m00 * c00 + m01 * c01) + m02 * c02;
    if (det == 0.0f || !(fabsf(det) <= 3.402823466e38f)) {
        for (int i = 0; i < 12; i++) w[i] = 0.0f;
        return false;
    }
    float id = 1.0f / det;
    w[0] = c00 * id;
    w[1] = (m02 * m21 - m01 * m22) * id;
    w[2] = (m01 * m12 - m02 * m11) * id;
    w[4] = c01 * id;
    w[5] = (m00 * m22 - m02 * m20) * id;
    w[6] = (m02 * m10 - m00 * m12) * id;
    w[8] = c02 * id;
    w[9] = (m01 * m20 - m00 * m21) * id;
    w[10] = (m00 * m11 - m01 * m10) * id;
    float tx = m[3], ty = m[7], tz = m[11];
    w[3] = -((w[0] * tx + w[1] * ty) + w[2] * tz);
    w[7] = -((w[4] * tx + w[5] * ty) + w[6] * tz);
    w[11] = -((w[8] * tx + w[9] * ty) + w[10] * tz);
    return true;
}

// sin and cos by Cody-Waite reduction (three-part pi/2, first two parts with
// 12 significant bits) and Taylor series on [-pi/4, pi/4] by Horner's rule.
// Used wherever a discrete decision (sun disc, shadow-ray direction) depends
// on the value, so the device and the oracle agree bit for bit.
__device__ __forceinline__ void rt_sincos(float x, float* s, float* c) {
    const float kTwoOverPi = 0.636619772367581343f;
    const float kC1 = 1.5703125f;
    const float kC2 = 4.83751296997070312e-04f;
    const float kC3 = 7.54978995489188216e-08f;
    float kf = floorf(x * kTwoOverPi + 0.5f);
    float r = ((x - kf * kC1) - kf * kC2) - kf * kC3;
    float r2 = r * r;
    float ps = 2.75573192e-06f;
    ps = ps * r2 + -1.98412698e-04f;
    ps = ps * r2 + 8.33333333e-03f;
    ps = ps * r2 + -1.66666667e-01f;
    ps = ps * r2;
    float sr = r + r * ps;
    float pc = -2.75573192e-07f;
    pc = pc * r2 + 2.48015873e-05f;
    pc = pc * r2 + -1.38888889e-03f;
    pc = pc * r2 + 4.16666667e-02f;
    pc = pc * r2 + -0.5f;
    float cr = 1.0f + r2 * pc;
    int k = ((int)kf) & 3;
    float so, co;
    if (k == 0) { so = sr; co = cr; }
    else if (k == 1) { so = cr; co = -sr; }
    else if (k == 2) { so = -sr; co = -cr; }
    else { so = -cr; co = sr; }
    *s = so;
    *c = co;
}

// Watertight ray setup (Woop, Benthin & Wald 2013).
struct WtRay {
    int kx, ky, kz;
    float sx, sy, sz;
};
__device__ __forceinline__ WtRay wt_setup(V3 d) {
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    if (get3(d, kz) < 0.0f) {
        int t = kx;
        kx = ky;
        ky = t;
    }
    WtRay w;
    w.kx = kx;
    w.ky = ky;
    w.kz = kz;
    float dz = get3(d, kz);
    w.sx = get3(d, kx) / dz;
    w.sy = get3(d, ky) / dz;
    w.sz = 1.0f / dz;
    return w;
}

// a*b - c*d; when the rounded difference is zero the products rounded to the
// same value and the exact difference is the difference of their rounding
// errors (exact by fmaf).  Exactly antisymmetric, so shared edges stay
// watertight without the paper's double-precision fallback.
__device__ __forceinline__ float edge_fn(float a, float b, float c, float d) {
    float p = a * b, q = c * d;
    float e = p - q;
    if (e == 0.0f) {
        float ep = fmaf(a, b, -p);
        float eq = fmaf(c, d, -q);
        e = ep - eq;
    }
    return e;
}

// Returns true for a hit with t in [tmin, tmax]; front = det < 0.
__device__ __forceinline__ bool tri_intersect(V3 o, const WtRay& w, V3 v0, V3 v1, V3 v2, float tmin, float tmax,
                                              float* t_out, float* u_out, float* v_out, bool* front) {
    V3 A = sub3(v0, o), B = sub3(v1, o), C = sub3(v2, o);
    float Akz = get3(A, w.kz), Bkz = get3(B, w.kz), Ckz = get3(C, w.kz);
    float Ax = get3(A, w.kx) - w.sx * Akz;
    float Ay = get3(A, w.ky) - w.sy * Akz;
    float Bx = get3(B, w.kx) - w.sx * Bkz;
    float By = get3(B, w.ky) - w.sy * Bkz;
    float Cx = get3(C, w.kx) - w.sx * Ckz;
    float Cy = get3(C, w.ky) - w.sy * Ckz;
    float U = edge_fn(Cx, By, Cy, Bx);
    float V = edge_fn(Ax, Cy, Ay, Cx);
    float W = edge_fn(Bx, Ay, By, Ax);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float Az = w.sz * Akz, Bz = w.sz * Bkz, Cz = w.sz * Ckz;
    float T = (U * Az + V * Bz) + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return false;
    *t_out = t;
    *u_out = V * rcp;
    *v_out = W * rcp;
    *front = det < 0.0f;
    return true;
}

// Conservative slab-test scale on the far distance (Ize 2013, 1 + 2*gamma(3)).
constexpr float kBoxFarScale = 1.0000004f;

__device__ __forceinline__ V3 safe_inv(V3 d) {
    const float e = 1e-20f;
    return mk3(1.0f / (fabsf(d.x) < e ? copysignf(e, d.x) : d.x), 1.0f / (fabsf(d.y) < e ? copysignf(e, d.y) : d.y),
               1.0f / (fabsf(d.z) < e ? copysignf(e, d.z) : d.z));
}

}  // namespace rt
