/*
 * rt_oracle.c — CPU oracle of the ray-tracing hot path (TEST INFRASTRUCTURE).
 *
 * Only the tests, the smoke check and bench.py's CPU legs load this code; the
 * product library never does.  Compiled with -ffp-contract=off so every FP32
 * operation rounds on its own: the geometric part of the pipeline (ray
 * generation, instance transforms, the triangle test, shadow and reflection
 * ray construction) follows a fixed operation order that the CUDA kernels
 * follow too, which makes hit IDs, t and the whole ray chain bit-exact.
 * Colour arithmetic (BRDF, pow, sRGB) is compared with a tolerance and can be
 * evaluated in FP64 (ORenderDesc.double_shading) to measure that error.
 *
 * Reference files restated (paths inside the reference project):
 *   shaders/ray-tracing/src/lib.rs       raygen :95-191, misses :33-51,
 *                                         linear_to_srgb :85-92, portal :300-312
 *   shaders/ray-tracing/src/heatmap.rs   heatmap_temperature :5-47
 *   shaders/ray-tracing/src/pbr.rs       V_SmithGGXCorrelated test :41-69
 *   shaders/hit_shader_common.glsl       buffers, barycentrics, load_triangle
 *   shaders/closest_hit_textured.glsl    :13-226
 *   shaders/closest_hit_mirror.glsl      :11-29
 *   shaders/any_hit_alpha_clip.glsl      :11-29
 *   shaders/pbr.glsl                     :25-103, :174-211
 *   src/main.rs:289-305                  program table (hit groups)
 *   src/gpu_structs.rs:20-58             instance record
 */
#include "rt_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdatomic.h>
#include <stdlib.h>
#include <string.h>

#define O_PI_F 3.141592653589793f
#define O_PI_D 3.141592653589793

/* ===================================================================== */
/* FP32 vector helpers (fixed operation order)                            */
/* ===================================================================== */
typedef struct { float x, y, z; } v3;
typedef struct { float x, y; } v2;

static inline v3 mk3(float x, float y, float z) { v3 r = {x, y, z}; return r; }
static inline v3 add3(v3 a, v3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub3(v3 a, v3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul3s(v3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
/* dot = (x*x' + y*y') + z*z' */
static inline float dot3(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 cross3(v3 a, v3 b) {
    return mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
/* normalize = v * (1 / sqrt(dot(v, v)))  (glam Vec3::normalize form) */
static inline v3 normalize3(v3 v) {
    float inv = 1.0f / sqrtf(dot3(v, v));
    return mul3s(v, inv);
}
/* interpolate(a, b, c, w) = (a*w.x + b*w.y) + c*w.z
 * (hit_shader_common.glsl:79-81, lib.rs:201-208) */
static inline v3 interp3(v3 a, v3 b, v3 c, v3 w) {
    return add3(add3(mul3s(a, w.x), mul3s(b, w.y)), mul3s(c, w.z));
}
static inline v2 interp2(v2 a, v2 b, v2 c, v3 w) {
    v2 r;
    r.x = (a.x * w.x + b.x * w.y) + c.x * w.z;
    r.y = (a.y * w.x + b.y * w.y) + c.y * w.z;
    return r;
}
/* column-major mat4 * vec4, component i = ((c0*x + c1*y) + c2*z) + c3*w */
static inline float mat4_row(const float* m, int i, float x, float y, float z, float w) {
    return ((m[0 * 4 + i] * x + m[1 * 4 + i] * y) + m[2 * 4 + i] * z) + m[3 * 4 + i] * w;
}
/* row-major 3x4 affine applied to a point: ((m0*x + m1*y) + m2*z) + m3 */
static inline v3 xform_point(const float* m, v3 p) {
    return mk3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3],
               ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
               ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
static inline v3 xform_dir(const float* m, v3 d) {
    return mk3((m[0] * d.x + m[1] * d.y) + m[2] * d.z, (m[4] * d.x + m[5] * d.y) + m[6] * d.z,
               (m[8] * d.x + m[9] * d.y) + m[10] * d.z);
}
/* mat3(gl_WorldToObject3x4EXT) * n: component i = (W0i*nx + W1i*ny) + W2i*nz */
static inline v3 xform_normal_w2o_t(const float* w, v3 n) {
    return mk3((w[0] * n.x + w[4] * n.y) + w[8] * n.z, (w[1] * n.x + w[5] * n.y) + w[9] * n.z,
               (w[2] * n.x + w[6] * n.y) + w[10] * n.z);
}
static inline float get3(v3 v, int i) { return i == 0 ? v.x : (i == 1 ? v.y : v.z); }

/* ===================================================================== */
/* sin/cos used where a discrete decision depends on the result           */
/* ===================================================================== */
/* Cody & Waite (1980) argument reduction by pi/2 with a three-part constant
 * whose first two parts carry 12 significant bits (so k*C1 and k*C2 are exact
 * for |k| < 2^12), followed by the Taylor series of sin and cos on
 * [-pi/4, pi/4] evaluated by Horner's rule.  Max error about 2 ulp over
 * [-1e3, 1e3].  The same operation sequence runs on the device. */
#define SC_TWO_OVER_PI 0.636619772367581343f
#define SC_C1 1.5703125f                /* pi/2 to 12 bits               */
#define SC_C2 4.83751296997070312e-04f  /* next 12 bits                  */
#define SC_C3 7.54978995489188216e-08f  /* remainder                     */
void o_sincos_f(float x, float* s, float* c) {
    float kf = floorf(x * SC_TWO_OVER_PI + 0.5f);
    float r = ((x - kf * SC_C1) - kf * SC_C2) - kf * SC_C3;
    float r2 = r * r;
    /* sin r = r*(1 + r2*(-1/6 + r2*(1/120 + r2*(-1/5040 + r2/362880)))) */
    float ps = 2.75573192e-06f;
    ps = ps * r2 + -1.98412698e-04f;
    ps = ps * r2 + 8.33333333e-03f;
    ps = ps * r2 + -1.66666667e-01f;
    ps = ps * r2;
    float sr = r + r * ps;
    /* cos r = 1 + r2*(-1/2 + r2*(1/24 + r2*(-1/720 + r2*(1/40320 - r2/3628800)))) */
    float pc = -2.75573192e-07f;
    pc = pc * r2 + 2.48015873e-05f;
    pc = pc * r2 + -1.38888889e-03f;
    pc = pc * r2 + 4.16666667e-02f;
    pc = pc * r2 + -0.5f;
    float cr = 1.0f + r2 * pc;
    int k = ((int)kf) & 3;
    switch (k) {
        case 0: *s = sr; *c = cr; break;
        case 1: *s = cr; *c = -sr; break;
        case 2: *s = -sr; *c = -cr; break;
        default: *s = -cr; *c = sr; break;
    }
}

/* ===================================================================== */
/* Instance transforms                                                    */
/* ===================================================================== */
/* world_to_object = inverse of the row-major 3x4 object_to_world, by the
 * adjugate with this exact order (the device builds the same matrix). */
int32_t o_instance_world_to_object(const float m[12], float w[12]) {
    float m00 = m[0], m01 = m[1], m02 = m[2], m10 = m[4], m11 = m[5], m12 = m[6];
    float m20 = m[8], m21 = m[9], m22 = m[10];
    float c00 = m11 * m22 - m12 * m21;
    float c01 = m12 * m20 - m10 * m22;
    float c02 = m10 * m21 - m11 * m20;
    float det = (m00 * c00 + m01 * c01) + m02 * c02;
    if (det == 0.0f || !isfinite(det)) {
        memset(w, 0, 12 * sizeof(float));
        return 0;
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
    return 1;
}

/* ===================================================================== */
/* Watertight ray/triangle test (Woop, Benthin & Wald, JCGT 2(1) 2013)     */
/* ===================================================================== */
typedef struct {
    v3 o, d;        /* ray in the current space */
    int kx, ky, kz;
    float sx, sy, sz;
    v3 inv;         /* safe reciprocal direction for box tests */
} ORay;

static void ray_setup(ORay* r, v3 o, v3 d) {
    r->o = o;
    r->d = d;
    float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
    int kz = 0;
    if (ay > ax) kz = 1;
    if (az > (kz == 0 ? ax : ay)) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (get3(d, kz) < 0.0f) { int t = kx; kx = ky; ky = t; }
    r->kx = kx; r->ky = ky; r->kz = kz;
    float dz = get3(d, kz);
    r->sx = get3(d, kx) / dz;
    r->sy = get3(d, ky) / dz;
    r->sz = 1.0f / dz;
    /* box tests only need a conservative reciprocal: clamp |d| away from 0 */
    float e = 1e-20f;
    r->inv.x = 1.0f / (fabsf(d.x) < e ? copysignf(e, d.x) : d.x);
    r->inv.y = 1.0f / (fabsf(d.y) < e ? copysignf(e, d.y) : d.y);
    r->inv.z = 1.0f / (fabsf(d.z) < e ? copysignf(e, d.z) : d.z);
}

/* a*b - c*d with an exact-sign fallback: when the rounded difference is
 * zero the two rounded products are equal and the exact difference equals
 * the difference of their rounding errors, which fmaf gives exactly.  This
 * replaces the paper's double-precision recomputation and keeps the edge
 * function exactly antisymmetric, so shared edges stay watertight. */
static inline float edge_fn(float a, float b, float c, float d) {
    float p = a * b, q = c * d;
    float e = p - q;
    if (e == 0.0f) {
        float ep = fmaf(a, b, -p);
        float eq = fmaf(c, d, -q);
        e = ep - eq;
    }
    return e;
}

/* Returns 1 on hit with t in [tmin, tmax]; front = 1 when det < 0
 * (clockwise as seen from the ray origin). */
static int tri_intersect(const ORay* r, v3 v0, v3 v1, v3 v2, float tmin, float tmax, float* t_out,
                         float* u_out, float* v_out, int* front) {
    v3 A = sub3(v0, r->o), B = sub3(v1, r->o), C = sub3(v2, r->o);
    float Akz = get3(A, r->kz), Bkz = get3(B, r->kz), Ckz = get3(C, r->kz);
    float Ax = get3(A, r->kx) - r->sx * Akz;
    float Ay = get3(A, r->ky) - r->sy * Akz;
    float Bx = get3(B, r->kx) - r->sx * Bkz;
    float By = get3(B, r->ky) - r->sy * Bkz;
    float Cx = get3(C, r->kx) - r->sx * Ckz;
    float Cy = get3(C, r->ky) - r->sy * Ckz;
    float U = edge_fn(Cx, By, Cy, Bx);
    float V = edge_fn(Ax, Cy, Ay, Cx);
    float W = edge_fn(Bx, Ay, By, Ax);
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return 0;
    float det = (U + V) + W;
    if (det == 0.0f) return 0;
    float Az = r->sz * Akz, Bz = r->sz * Bkz, Cz = r->sz * Ckz;
    float T = (U * Az + V * Bz) + W * Cz;
    float rcp = 1.0f / det;
    float t = T * rcp;
    if (!(t >= tmin && t <= tmax)) return 0;
    *t_out = t;
    *u_out = V * rcp;
    *v_out = W * rcp;
    *front = det < 0.0f;
    return 1;
}

/* Conservative slab test (Ize 2013: far distance scaled by 1 + 2*gamma(3)). */
#define O_BOX_FAR_SCALE 1.0000004f
static inline int box_hit(const ORay* r, const float* lo, const float* hi, float tmin, float tmax,
                          float* tnear_out) {
    float t0x = (lo[0] - r->o.x) * r->inv.x, t1x = (hi[0] - r->o.x) * r->inv.x;
    float t0y = (lo[1] - r->o.y) * r->inv.y, t1y = (hi[1] - r->o.y) * r->inv.y;
    float t0z = (lo[2] - r->o.z) * r->inv.z, t1z = (hi[2] - r->o.z) * r->inv.z;
    float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), tmin));
    float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tmax));
    *tnear_out = tn;
    return tn <= tf * O_BOX_FAR_SCALE;
}

/* ===================================================================== */
/* Binary binned-SAH BVH (independent of the product's LBVH)              */
/* ===================================================================== */
typedef struct {
    float lo[3], hi[3];
    uint32_t a;      /* leaf: first index into perm; inner: left child */
    uint32_t count;  /* leaf: >0 primitive count; inner: 0 (right = a+1 is NOT assumed) */
    uint32_t b;      /* inner: right child */
    uint32_t _pad;
} OBNode;

typedef struct {
    OBNode* nodes;
    uint32_t node_count, node_cap;
    uint32_t* perm;
} OBvh;

typedef struct {
    float lo[3], hi[3], c[3];
} OPrimBox;

static void box_pad(float* lo, float* hi) {
    for (int k = 0; k < 3; k++) {
        float m = fmaxf(fabsf(lo[k]), fabsf(hi[k]));
        float pad = m * 9.5367431640625e-07f /* 2^-20 */ + 1e-30f;
        lo[k] -= pad;
        hi[k] += pad;
    }
}

static uint32_t bvh_new_node(OBvh* b) {
    if (b->node_count == b->node_cap) {
        b->node_cap = b->node_cap ? b->node_cap * 2 : 64;
        b->nodes = (OBNode*)realloc(b->nodes, b->node_cap * sizeof(OBNode));
    }
    return b->node_count++;
}

#define SAH_BINS 16
#define LEAF_MAX 4
static void bvh_build_rec(OBvh* b, const OPrimBox* pb, uint32_t node, uint32_t first, uint32_t count) {
    OBNode* n = &b->nodes[node];
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    float clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (uint32_t i = first; i < first + count; i++) {
        const OPrimBox* p = &pb[b->perm[i]];
        for (int k = 0; k < 3; k++) {
            lo[k] = fminf(lo[k], p->lo[k]);
            hi[k] = fmaxf(hi[k], p->hi[k]);
            clo[k] = fminf(clo[k], p->c[k]);
            chi[k] = fmaxf(chi[k], p->c[k]);
        }
    }
    memcpy(n->lo, lo, sizeof lo);
    memcpy(n->hi, hi, sizeof hi);
    if (count <= LEAF_MAX) {
        n->a = first; n->count = count; n->b = 0;
        return;
    }
    /* binned SAH over the widest centroid axis */
    int axis = 0;
    float ext[3] = {chi[0] - clo[0], chi[1] - clo[1], chi[2] - clo[2]};
    if (ext[1] > ext[axis]) axis = 1;
    if (ext[2] > ext[axis]) axis = 2;
    uint32_t mid;
    if (!(ext[axis] > 0.0f)) {
        mid = first + count / 2; /* all centroids equal: median split */
    } else {
        uint32_t bc[SAH_BINS] = {0};
        float blo[SAH_BINS][3], bhi[SAH_BINS][3];
        for (int i = 0; i < SAH_BINS; i++)
            for (int k = 0; k < 3; k++) { blo[i][k] = INFINITY; bhi[i][k] = -INFINITY; }
        float scale = (float)SAH_BINS / ext[axis];
        for (uint32_t i = first; i < first + count; i++) {
            const OPrimBox* p = &pb[b->perm[i]];
            int bi = (int)((p->c[axis] - clo[axis]) * scale);
            if (bi >= SAH_BINS) bi = SAH_BINS - 1;
            if (bi < 0) bi = 0;
            bc[bi]++;
            for (int k = 0; k < 3; k++) {
                blo[bi][k] = fminf(blo[bi][k], p->lo[k]);
                bhi[bi][k] = fmaxf(bhi[bi][k], p->hi[k]);
            }
        }
        double best = INFINITY;
        int best_split = -1;
        for (int s = 1; s < SAH_BINS; s++) {
            float l0[3] = {INFINITY, INFINITY, INFINITY}, l1[3] = {-INFINITY, -INFINITY, -INFINITY};
            float r0[3] = {INFINITY, INFINITY, INFINITY}, r1[3] = {-INFINITY, -INFINITY, -INFINITY};
            uint32_t lc = 0, rc = 0;
            for (int i = 0; i < s; i++) {
                lc += bc[i];
                for (int k = 0; k < 3; k++) { l0[k] = fminf(l0[k], blo[i][k]); l1[k] = fmaxf(l1[k], bhi[i][k]); }
            }
            for (int i = s; i < SAH_BINS; i++) {
                rc += bc[i];
                for (int k = 0; k < 3; k++) { r0[k] = fminf(r0[k], blo[i][k]); r1[k] = fmaxf(r1[k], bhi[i][k]); }
            }
            if (lc == 0 || rc == 0) continue;
            double la = 0, ra = 0;
            {
                double dx = l1[0] - l0[0], dy = l1[1] - l0[1], dz = l1[2] - l0[2];
                la = dx * dy + dy * dz + dz * dx;
                dx = r1[0] - r0[0]; dy = r1[1] - r0[1]; dz = r1[2] - r0[2];
                ra = dx * dy + dy * dz + dz * dx;
            }
            double cost = la * lc + ra * rc;
            if (cost < best) { best = cost; best_split = s; }
        }
        if (best_split < 0) {
            mid = first + count / 2;
        } else {
            /* partition perm[first..first+count) by bin < best_split */
            uint32_t i = first, j = first + count;
            while (i < j) {
                const OPrimBox* p = &pb[b->perm[i]];
                int bi = (int)((p->c[axis] - clo[axis]) * scale);
                if (bi >= SAH_BINS) bi = SAH_BINS - 1;
                if (bi < 0) bi = 0;
                if (bi < best_split) i++;
                else { j--; uint32_t t = b->perm[i]; b->perm[i] = b->perm[j]; b->perm[j] = t; }
            }
            mid = i;
            if (mid == first || mid == first + count) mid = first + count / 2;
        }
    }
    uint32_t l = bvh_new_node(b);
    uint32_t r = bvh_new_node(b);
    n = &b->nodes[node];
    n->a = l; n->b = r; n->count = 0;
    bvh_build_rec(b, pb, l, first, mid - first);
    bvh_build_rec(b, pb, r, mid, first + count - mid);
}

static void bvh_build(OBvh* b, const OPrimBox* pb, uint32_t count) {
    free(b->nodes); free(b->perm);
    memset(b, 0, sizeof *b);
    b->perm = (uint32_t*)malloc((count ? count : 1) * sizeof(uint32_t));
    for (uint32_t i = 0; i < count; i++) b->perm[i] = i;
    uint32_t root = bvh_new_node(b);
    if (count == 0) {
        OBNode* n = &b->nodes[root];
        for (int k = 0; k < 3; k++) { n->lo[k] = INFINITY; n->hi[k] = -INFINITY; }
        n->a = 0; n->count = 0; n->b = 0;
        n->count = 0;
        return;
    }
    bvh_build_rec(b, pb, root, 0, count);
}

/* ===================================================================== */
/* Scene                                                                  */
/* ===================================================================== */
typedef struct {
    float v[3][3];
    uint32_t geom, prim, opaque;
} OTri;

typedef struct {
    OTri* tris;
    uint32_t tri_count;
    uint32_t geometry_count;
    OBvh bvh;
    float lo[3], hi[3];
    int built;
} OBlas;

typedef struct {
    float o2w[12], w2o[12];
    uint32_t custom_index, mask, sbt_offset, flags, blas;
    int valid;
} OInst;

struct OScene {
    OBlas* blas;
    uint32_t blas_count;
    OInst* inst;
    uint32_t inst_count;
    OBvh tlas;
    OModelInfo* models;
    uint32_t model_count;
    OTexture textures[RT_MAX_BOUND_IMAGES];
    int bruteforce;
};

OScene* o_scene_create(void) { return (OScene*)calloc(1, sizeof(OScene)); }

void o_scene_destroy(OScene* s) {
    if (!s) return;
    for (uint32_t i = 0; i < s->blas_count; i++) {
        free(s->blas[i].tris);
        free(s->blas[i].bvh.nodes);
        free(s->blas[i].bvh.perm);
    }
    free(s->blas);
    free(s->inst);
    free(s->tlas.nodes);
    free(s->tlas.perm);
    free(s->models);
    free(s);
}

/* Gathers the triangles of every geometry (src/util_structs.rs:151-186). */
int32_t o_scene_add_blas(OScene* s, const OGeometry* g, uint32_t count) {
    uint32_t total = 0;
    for (uint32_t i = 0; i < count; i++) total += g[i].primitive_count;
    s->blas = (OBlas*)realloc(s->blas, (s->blas_count + 1) * sizeof(OBlas));
    OBlas* b = &s->blas[s->blas_count];
    memset(b, 0, sizeof *b);
    b->tris = (OTri*)malloc((total ? total : 1) * sizeof(OTri));
    b->tri_count = total;
    b->geometry_count = count;
    uint32_t k = 0;
    for (uint32_t gi = 0; gi < count; gi++) {
        for (uint32_t p = 0; p < g[gi].primitive_count; p++, k++) {
            OTri* t = &b->tris[k];
            for (int c = 0; c < 3; c++) {
                uint32_t vi = g[gi].indices ? g[gi].indices[3 * p + c] : 3 * p + c;
                const float* src = g[gi].positions + (size_t)vi * g[gi].stride_floats;
                t->v[c][0] = src[0]; t->v[c][1] = src[1]; t->v[c][2] = src[2];
            }
            t->geom = gi;
            t->prim = p;
            t->opaque = (g[gi].flags & RT_GEOMETRY_OPAQUE) ? 1u : 0u;
        }
    }
    return (int32_t)s->blas_count++;
}

int32_t o_scene_set_instances(OScene* s, const RtAccelerationStructureInstance* in, uint32_t count) {
    free(s->inst);
    s->inst = (OInst*)calloc(count ? count : 1, sizeof(OInst));
    s->inst_count = count;
    for (uint32_t i = 0; i < count; i++) {
        OInst* o = &s->inst[i];
        memcpy(o->o2w, in[i].transform, 12 * sizeof(float));
        o->valid = o_instance_world_to_object(o->o2w, o->w2o);
        o->custom_index = in[i].instance_custom_index_and_mask & 0xFFFFFFu;
        o->mask = in[i].instance_custom_index_and_mask >> 24;
        o->sbt_offset = in[i].instance_shader_binding_table_record_offset_and_flags & 0xFFFFFFu;
        o->flags = in[i].instance_shader_binding_table_record_offset_and_flags >> 24;
        o->blas = (uint32_t)in[i].acceleration_structure_reference;
        if (o->blas >= s->blas_count) o->valid = 0;
    }
    return 0;
}

int32_t o_scene_set_models(OScene* s, const OModelInfo* m, uint32_t count) {
    free(s->models);
    s->models = (OModelInfo*)malloc((count ? count : 1) * sizeof(OModelInfo));
    memcpy(s->models, m, count * sizeof(OModelInfo));
    s->model_count = count;
    return 0;
}

int32_t o_scene_set_texture(OScene* s, uint32_t index, const OTexture* t) {
    if (index >= RT_MAX_BOUND_IMAGES) return RT_ERR_INVALID;
    s->textures[index] = *t;
    return 0;
}

void o_scene_set_bruteforce(OScene* s, int32_t on) { s->bruteforce = on; }

int32_t o_scene_build(OScene* s) {
    for (uint32_t bi = 0; bi < s->blas_count; bi++) {
        OBlas* b = &s->blas[bi];
        if (b->built) continue;
        OPrimBox* pb = (OPrimBox*)malloc((b->tri_count ? b->tri_count : 1) * sizeof(OPrimBox));
        for (int k = 0; k < 3; k++) { b->lo[k] = INFINITY; b->hi[k] = -INFINITY; }
        for (uint32_t i = 0; i < b->tri_count; i++) {
            const OTri* t = &b->tris[i];
            for (int k = 0; k < 3; k++) {
                float lo = fminf(fminf(t->v[0][k], t->v[1][k]), t->v[2][k]);
                float hi = fmaxf(fmaxf(t->v[0][k], t->v[1][k]), t->v[2][k]);
                pb[i].lo[k] = lo; pb[i].hi[k] = hi;
                pb[i].c[k] = 0.5f * (lo + hi);
                b->lo[k] = fminf(b->lo[k], lo); b->hi[k] = fmaxf(b->hi[k], hi);
            }
            box_pad(pb[i].lo, pb[i].hi);
        }
        bvh_build(&b->bvh, pb, b->tri_count);
        free(pb);
        b->built = 1;
    }
    /* TLAS over instance world boxes: the 8 transformed corners of the BLAS
     * bounds, padded (conservative for the object-space ray transform). */
    OPrimBox* pb = (OPrimBox*)malloc((s->inst_count ? s->inst_count : 1) * sizeof(OPrimBox));
    for (uint32_t i = 0; i < s->inst_count; i++) {
        const OInst* in = &s->inst[i];
        float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
        if (in->valid && s->blas[in->blas].tri_count > 0) {
            const OBlas* b = &s->blas[in->blas];
            for (int c = 0; c < 8; c++) {
                v3 p = mk3((c & 1) ? b->hi[0] : b->lo[0], (c & 2) ? b->hi[1] : b->lo[1],
                           (c & 4) ? b->hi[2] : b->lo[2]);
                v3 q = xform_point(in->o2w, p);
                for (int k = 0; k < 3; k++) {
                    lo[k] = fminf(lo[k], get3(q, k));
                    hi[k] = fmaxf(hi[k], get3(q, k));
                }
            }
            float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
            for (int k = 0; k < 3; k++) {
                float pad = (fmaxf(fabsf(lo[k]), fabsf(hi[k])) + ext) * 1e-5f + 1e-20f;
                lo[k] -= pad; hi[k] += pad;
            }
        } else {
            /* invalid / empty: a box no ray can hit */
            for (int k = 0; k < 3; k++) { lo[k] = INFINITY; hi[k] = -INFINITY; }
        }
        for (int k = 0; k < 3; k++) {
            pb[i].lo[k] = lo[k]; pb[i].hi[k] = hi[k];
            pb[i].c[k] = isfinite(lo[k]) ? 0.5f * (lo[k] + hi[k]) : 0.0f;
        }
    }
    bvh_build(&s->tlas, pb, s->inst_count);
    free(pb);
    return 0;
}

/* ===================================================================== */
/* Textures (software sampling, REPEAT addressing)                         */
/* ===================================================================== */
static float g_srgb_lut[256];
static pthread_once_t g_srgb_once = PTHREAD_ONCE_INIT;
static void srgb_init(void) {
    for (int i = 0; i < 256; i++) {
        double c = i / 255.0;
        double l = c <= 0.04045 ? c / 12.92 : pow((c + 0.055) / 1.055, 2.4);
        g_srgb_lut[i] = (float)l;
    }
}

static inline int wrap_i(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

static void texel_fetch(const OTexture* t, int x, int y, float out[4]) {
    const uint8_t* row = (const uint8_t*)t->texels + (size_t)y * t->row_pitch;
    if (t->format == RT_FORMAT_R32G32B32A32_SFLOAT) {
        memcpy(out, row + (size_t)x * 16, 16);
    } else {
        const uint8_t* p = row + (size_t)x * 4;
        if (t->format == RT_FORMAT_R8G8B8A8_SRGB) {
            out[0] = g_srgb_lut[p[0]];
            out[1] = g_srgb_lut[p[1]];
            out[2] = g_srgb_lut[p[2]];
        } else {
            out[0] = (float)p[0] / 255.0f;
            out[1] = (float)p[1] / 255.0f;
            out[2] = (float)p[2] / 255.0f;
        }
        out[3] = (float)p[3] / 255.0f;
    }
}

/* Nearest: texel floor(u*w) (mod w).  Linear: x = u*w - 0.5, weights
 * fx = x - floor(x); result = (((1-fx)(1-fy))t00 + (fx(1-fy))t10)
 * + ((1-fx)fy)t01) + (fx fy)t11, evaluated in that order. */
static void tex_sample(const OTexture* t, float u, float v, float out[4]) {
    pthread_once(&g_srgb_once, srgb_init);
    if (!t->texels || t->width == 0 || t->height == 0) {
        out[0] = out[1] = out[2] = out[3] = 0.0f;
        return;
    }
    int w = (int)t->width, h = (int)t->height;
    if (t->filter == RT_FILTER_LINEAR) {
        float x = u * (float)w - 0.5f, y = v * (float)h - 0.5f;
        float x0 = floorf(x), y0 = floorf(y);
        float fx = x - x0, fy = y - y0;
        int ix = wrap_i((int)fmaxf(fminf(x0, 2.0e9f), -2.0e9f), w);
        int iy = wrap_i((int)fmaxf(fminf(y0, 2.0e9f), -2.0e9f), h);
        int ix1 = ix + 1 == w ? 0 : ix + 1, iy1 = iy + 1 == h ? 0 : iy + 1;
        float t00[4], t10[4], t01[4], t11[4];
        texel_fetch(t, ix, iy, t00);
        texel_fetch(t, ix1, iy, t10);
        texel_fetch(t, ix, iy1, t01);
        texel_fetch(t, ix1, iy1, t11);
        float w00 = (1.0f - fx) * (1.0f - fy), w10 = fx * (1.0f - fy);
        float w01 = (1.0f - fx) * fy, w11 = fx * fy;
        for (int c = 0; c < 4; c++)
            out[c] = ((w00 * t00[c] + w10 * t10[c]) + w01 * t01[c]) + w11 * t11[c];
    } else {
        float x = floorf(u * (float)w), y = floorf(v * (float)h);
        int ix = wrap_i((int)fmaxf(fminf(x, 2.0e9f), -2.0e9f), w);
        int iy = wrap_i((int)fmaxf(fminf(y, 2.0e9f), -2.0e9f), h);
        texel_fetch(t, ix, iy, out);
    }
}

/* ===================================================================== */
/* Traversal                                                               */
/* ===================================================================== */
typedef struct {
    float t, u, v;
    uint32_t inst, geom, prim;
    int hit, front;
} OHitRec;

typedef struct {
    const OScene* s;
    const RtShaderBindingTable* sbt;
    int have_models;
    uint32_t ray_flags, cull_mask, sbt_offset;
    OStats* st;
} OTraceCtx;

/* (inst, geom, prim) lexicographically below the best hit */
static inline int id_less(uint32_t i, uint32_t g, uint32_t p, const OHitRec* b) {
    if (i != b->inst) return i < b->inst;
    if (g != b->geom) return g < b->geom;
    return p < b->prim;
}

/* any_hit_alpha_clip.glsl:11-29: alpha of the diffuse texture at the
 * interpolated uv; ignoreIntersectionEXT when alpha < 0.5. */
static int alpha_clip_accepts(const OTraceCtx* c, const OInst* in, uint32_t geom, uint32_t prim, float u,
                              float v) {
    const OScene* s = c->s;
    if (in->custom_index >= s->model_count) return 1;
    const OModelInfo* m = &s->models[in->custom_index];
    if (geom >= m->geometry_count) return 1;
    const OGeometryInfo* gi = &m->geometries[geom];
    const uint32_t* idx = gi->indices + 3 * (size_t)prim;
    v3 w = mk3((1.0f - u) - v, u, v);
    v2 a = {m->uvs[2 * idx[0]], m->uvs[2 * idx[0] + 1]};
    v2 b = {m->uvs[2 * idx[1]], m->uvs[2 * idx[1] + 1]};
    v2 cc = {m->uvs[2 * idx[2]], m->uvs[2 * idx[2] + 1]};
    v2 uv = interp2(a, b, cc, w);
    float texel[4];
    uint32_t ti = gi->diffuse_image_index;
    if (ti >= RT_MAX_BOUND_IMAGES) return 1;
    tex_sample(&s->textures[ti], uv.x, uv.y, texel);
    return !(texel[3] < 0.5f);
}

static inline const RtHitGroup* hit_group(const OTraceCtx* c, const OInst* in) {
    if (!c->sbt) return NULL;
    uint32_t gi = in->sbt_offset + c->sbt_offset;
    if (gi >= c->sbt->hit_group_count || gi >= RT_MAX_HIT_GROUPS) return NULL;
    return &c->sbt->hit_groups[gi];
}

/* Tests every triangle of one leaf / primitive list of a BLAS.  Returns 1
 * when traversal may stop (terminate-on-first-hit accepted a hit). */
static int test_tri(const OTraceCtx* c, const ORay* r, const OInst* in, uint32_t inst_id, const OTri* tri,
                    float tmin, OHitRec* best) {
    uint32_t rf = c->ray_flags;
    if (c->st) c->st->triangles_tested++;
    int opaque = (int)tri->opaque;
    if (in->flags & RT_INSTANCE_FORCE_OPAQUE) opaque = 1;
    if (in->flags & RT_INSTANCE_FORCE_NO_OPAQUE) opaque = 0;
    if (rf & RT_RAY_FLAG_OPAQUE) opaque = 1;
    if (rf & RT_RAY_FLAG_NO_OPAQUE) opaque = 0;
    if ((rf & RT_RAY_FLAG_CULL_OPAQUE) && opaque) return 0;
    if ((rf & RT_RAY_FLAG_CULL_NO_OPAQUE) && !opaque) return 0;
    float t, u, v;
    int front;
    v3 v0 = mk3(tri->v[0][0], tri->v[0][1], tri->v[0][2]);
    v3 v1 = mk3(tri->v[1][0], tri->v[1][1], tri->v[1][2]);
    v3 v2v = mk3(tri->v[2][0], tri->v[2][1], tri->v[2][2]);
    if (!tri_intersect(r, v0, v1, v2v, tmin, best->t, &t, &u, &v, &front)) return 0;
    if (in->flags & RT_INSTANCE_TRIANGLE_FLIP_FACING) front = !front;
    if (!(in->flags & RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE)) {
        if ((rf & RT_RAY_FLAG_CULL_BACK_FACING) && !front) return 0;
        if ((rf & RT_RAY_FLAG_CULL_FRONT_FACING) && front) return 0;
    }
    if (t == best->t && best->hit && !id_less(inst_id, tri->geom, tri->prim, best)) return 0;
    if (!opaque) {
        const RtHitGroup* g = hit_group(c, in);
        if (g && g->any_hit == RT_PROGRAM_ANY_HIT_ALPHA_CLIP && c->have_models) {
            if (!alpha_clip_accepts(c, in, tri->geom, tri->prim, u, v)) return 0;
        }
    }
    best->t = t; best->u = u; best->v = v;
    best->inst = inst_id; best->geom = tri->geom; best->prim = tri->prim;
    best->hit = 1; best->front = front;
    return (rf & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT) ? 1 : 0;
}

static int trace_blas(const OTraceCtx* c, const ORay* r, const OInst* in, uint32_t inst_id, float tmin,
                      OHitRec* best) {
    const OBlas* b = &c->s->blas[in->blas];
    if (c->s->bruteforce) {
        for (uint32_t i = 0; i < b->tri_count; i++)
            if (test_tri(c, r, in, inst_id, &b->tris[i], tmin, best)) return 1;
        return 0;
    }
    if (b->tri_count == 0) return 0;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const OBNode* n = &b->bvh.nodes[stack[--sp]];
        float tn;
        if (c->st) c->st->nodes_visited++;
        if (!box_hit(r, n->lo, n->hi, tmin, best->t, &tn)) continue;
        if (n->count > 0) {
            for (uint32_t i = 0; i < n->count; i++)
                if (test_tri(c, r, in, inst_id, &b->tris[b->bvh.perm[n->a + i]], tmin, best)) return 1;
        } else {
            if (sp + 2 > 128) abort();
            stack[sp++] = n->b;
            stack[sp++] = n->a;
        }
    }
    return 0;
}

static int trace_instance(const OTraceCtx* c, const ORay* wr, uint32_t inst_id, float tmin, OHitRec* best) {
    const OInst* in = &c->s->inst[inst_id];
    if (!in->valid) return 0;
    if ((in->mask & c->cull_mask) == 0) return 0;
    if (c->st) c->st->instances_visited++;
    ORay orr;
    ray_setup(&orr, xform_point(in->w2o, wr->o), xform_dir(in->w2o, wr->d));
    return trace_blas(c, &orr, in, inst_id, tmin, best);
}

/* One traceRayEXT: closest hit (or first accepted hit) in [tmin, tmax]. */
static void trace_one(const OTraceCtx* c, v3 o, v3 d, float tmin, float tmax, OHitRec* best) {
    memset(best, 0, sizeof *best);
    best->t = tmax;
    best->hit = 0;
    best->inst = best->geom = best->prim = 0xFFFFFFFFu;
    if (c->st) c->st->traversals++;
    ORay wr;
    ray_setup(&wr, o, d);
    const OScene* s = c->s;
    if (s->bruteforce) {
        for (uint32_t i = 0; i < s->inst_count; i++)
            if (trace_instance(c, &wr, i, tmin, best)) return;
        return;
    }
    if (s->inst_count == 0) return;
    uint32_t stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp > 0) {
        const OBNode* n = &s->tlas.nodes[stack[--sp]];
        float tn;
        if (c->st) c->st->nodes_visited++;
        if (!box_hit(&wr, n->lo, n->hi, tmin, best->t, &tn)) continue;
        if (n->count > 0) {
            for (uint32_t i = 0; i < n->count; i++)
                if (trace_instance(c, &wr, s->tlas.perm[n->a + i], tmin, best)) return;
        } else {
            if (sp + 2 > 128) abort();
            stack[sp++] = n->b;
            stack[sp++] = n->a;
        }
    }
}

/* ===================================================================== */
/* Thread pool helper                                                      */
/* ===================================================================== */
typedef struct {
    atomic_uint_fast64_t next;
    uint64_t total, chunk;
    void (*fn)(void* arg, uint64_t begin, uint64_t end, OStats* st);
    void* arg;
    OStats* stats;      /* per thread */
} OPool;

typedef struct { OPool* p; int id; } OWorker;

static void* pool_main(void* a) {
    OWorker* w = (OWorker*)a;
    OPool* p = w->p;
    for (;;) {
        uint64_t b = atomic_fetch_add(&p->next, p->chunk);
        if (b >= p->total) break;
        uint64_t e = b + p->chunk < p->total ? b + p->chunk : p->total;
        p->fn(p->arg, b, e, &p->stats[w->id]);
    }
    return NULL;
}

static void pool_run(int threads, uint64_t total, uint64_t chunk,
                     void (*fn)(void*, uint64_t, uint64_t, OStats*), void* arg, OStats* out) {
    if (threads < 1) threads = 1;
    OPool p;
    atomic_init(&p.next, 0);
    p.total = total;
    p.chunk = chunk ? chunk : 1;
    p.fn = fn;
    p.arg = arg;
    p.stats = (OStats*)calloc((size_t)threads, sizeof(OStats));
    OWorker* ws = (OWorker*)calloc((size_t)threads, sizeof(OWorker));
    pthread_t* th = (pthread_t*)calloc((size_t)threads, sizeof(pthread_t));
    for (int i = 0; i < threads; i++) {
        ws[i].p = &p;
        ws[i].id = i;
        if (i > 0) pthread_create(&th[i], NULL, pool_main, &ws[i]);
    }
    pool_main(&ws[0]);
    for (int i = 1; i < threads; i++) pthread_join(th[i], NULL);
    if (out) {
        for (int i = 0; i < threads; i++) {
            out->traversals += p.stats[i].traversals;
            out->primary_rays += p.stats[i].primary_rays;
            out->secondary_rays += p.stats[i].secondary_rays;
            out->shadow_rays += p.stats[i].shadow_rays;
            out->nodes_visited += p.stats[i].nodes_visited;
            out->triangles_tested += p.stats[i].triangles_tested;
            out->instances_visited += p.stats[i].instances_visited;
        }
    }
    free(p.stats);
    free(ws);
    free(th);
}

/* ===================================================================== */
/* Ray-buffer query                                                        */
/* ===================================================================== */
typedef struct {
    OScene* s;
    const RtShaderBindingTable* sbt;
    int have_models;
    uint32_t ray_flags, cull_mask, sbt_offset;
    const RtRay* rays;
    RtHit* hits;
} ORBArgs;

static void rb_chunk(void* a, uint64_t b, uint64_t e, OStats* st) {
    ORBArgs* A = (ORBArgs*)a;
    OTraceCtx c = {A->s, A->sbt, A->have_models, A->ray_flags, A->cull_mask, A->sbt_offset, st};
    for (uint64_t i = b; i < e; i++) {
        const RtRay* r = &A->rays[i];
        OHitRec h;
        trace_one(&c, mk3(r->origin[0], r->origin[1], r->origin[2]),
                  mk3(r->direction[0], r->direction[1], r->direction[2]), r->tmin, r->tmax, &h);
        RtHit* o = &A->hits[i];
        if (h.hit) {
            o->t = h.t; o->u = h.u; o->v = h.v;
            o->instance_id = h.inst;
            o->instance_custom_index = A->s->inst[h.inst].custom_index;
            o->geometry_index = h.geom;
            o->primitive_index = h.prim;
            o->hit_kind = h.front ? 0xFEu : 0xFFu;
        } else {
            o->t = r->tmax; o->u = 0.0f; o->v = 0.0f;
            o->instance_id = 0xFFFFFFFFu;
            o->instance_custom_index = 0xFFFFFFFFu;
            o->geometry_index = 0xFFFFFFFFu;
            o->primitive_index = 0xFFFFFFFFu;
            o->hit_kind = 0;
        }
    }
}

int32_t o_trace_ray_buffer(OScene* s, const RtShaderBindingTable* sbt, int32_t have_models, uint32_t ray_flags,
                           uint32_t cull_mask, uint32_t sbt_offset, const RtRay* rays, uint32_t count, RtHit* hits,
                           int32_t threads, OStats* stats) {
    ORBArgs a = {s, sbt, have_models, ray_flags, cull_mask, sbt_offset, rays, hits};
    pool_run(threads, count, 1024, rb_chunk, &a, stats);
    return 0;
}

/* ===================================================================== */
/* Shading arithmetic, FP32 and FP64 (colour only)                         */
/* ===================================================================== */
#define REAL float
#define RSFX(n) n##_f
#define RCONST(x) x##f
#define RSQRT sqrtf
#define RPOW powf
#define RFLOOR floorf
#define RFMIN fminf
#define RFMAX fmaxf
#include "rt_oracle_shade.inc"
#undef REAL
#undef RSFX
#undef RCONST
#undef RSQRT
#undef RPOW
#undef RFLOOR
#undef RFMIN
#undef RFMAX

#define REAL double
#define RSFX(n) n##_d
#define RCONST(x) x
#define RSQRT sqrt
#define RPOW pow
#define RFLOOR floor
#define RFMIN fmin
#define RFMAX fmax
#include "rt_oracle_shade.inc"
#undef REAL
#undef RSFX
#undef RCONST
#undef RSQRT
#undef RPOW
#undef RFLOOR
#undef RFMIN
#undef RFMAX

/* ===================================================================== */
/* The pipeline: ray_generation + programs                                 */
/* ===================================================================== */
typedef struct {
    OScene* s;
    const RtUniforms* u;
    const RtShaderBindingTable* sbt;
    const ORenderDesc* d;
    uint8_t* image;
    float* radiance;
} ORenderArgs;

/* Loads the hit triangle from the model buffers (hit_shader_common.glsl:
 * read_indices :83-87, load_triangle :144-154). */
typedef struct {
    v3 p[3], n[3];
    v2 uv[3];
    const OGeometryInfo* gi;
} OTriData;

static int load_triangle(const OScene* s, const OInst* in, uint32_t geom, uint32_t prim, OTriData* td) {
    if (in->custom_index >= s->model_count) return 0;
    const OModelInfo* m = &s->models[in->custom_index];
    if (geom >= m->geometry_count) return 0;
    td->gi = &m->geometries[geom];
    const uint32_t* idx = td->gi->indices + 3 * (size_t)prim;
    for (int k = 0; k < 3; k++) {
        uint32_t i = idx[k];
        td->p[k] = mk3(m->positions[3 * i], m->positions[3 * i + 1], m->positions[3 * i + 2]);
        td->n[k] = mk3(m->normals[3 * i], m->normals[3 * i + 1], m->normals[3 * i + 2]);
        td->uv[k].x = m->uvs[2 * i];
        td->uv[k].y = m->uvs[2 * i + 1];
    }
    return 1;
}

/* closest_hit_textured.glsl:13-19 */
static v3 project_onto_tangent_plane(v3 point, v3 vp, v3 vn) {
    v3 vtp = sub3(point, vp);
    float dp = fminf(0.0f, dot3(vtp, vn));
    return sub3(vtp, mul3s(vn, dp));
}

/* closest_hit_textured.glsl:25-39 (Ray Tracing Gems II ch. 4.3) */
static v3 shadow_terminator_origin(const OTriData* td, v3 p, v3 bary, const float* o2w) {
    v3 oa = project_onto_tangent_plane(p, td->p[0], td->n[0]);
    v3 ob = project_onto_tangent_plane(p, td->p[1], td->n[1]);
    v3 oc = project_onto_tangent_plane(p, td->p[2], td->n[2]);
    v3 off = interp3(oa, ob, oc, bary);
    return xform_point(o2w, add3(p, off));
}

/* closest_hit_textured.glsl:99-111 */
static v2 sample_blue_noise(const OScene* s, uint32_t tex, uint32_t x, uint32_t y, uint32_t i) {
    uint32_t f0x = i * 2u * 13u, f0y = i * 2u * 41u;
    uint32_t f1x = (i * 2u + 1u) * 13u, f1y = (i * 2u + 1u) * 41u;
    float a[4], b[4];
    const OTexture* t = tex < RT_MAX_BOUND_IMAGES ? &s->textures[tex] : NULL;
    v2 r = {0.0f, 0.0f};
    if (!t) return r;
    tex_sample(t, (float)(x + f0x) / 64.0f, (float)(y + f0y) / 64.0f, a);
    tex_sample(t, (float)(x + f1x) / 64.0f, (float)(y + f1y) / 64.0f, b);
    r.x = a[0];
    r.y = b[0];
    return r;
}

/* closest_hit_textured.glsl:116-120 */
static v2 animated_blue_noise(v2 bn, uint32_t frame) {
    float g = (float)(frame % 32u) * 0.618033988749f;
    float sx = bn.x + g, sy = bn.y + g;
    v2 r = {sx - floorf(sx), sy - floorf(sy)};
    return r;
}

/* closest_hit_textured.glsl:77-94 */
static v3 sample_directional_light(v2 rng, v3 center, float radius) {
    float rad = sqrtf(rng.x);
    float ang = (rng.y * 2.0f) * O_PI_F;
    float sn, cs;
    o_sincos_f(ang, &sn, &cs);
    float px = (rad * cs) * radius, py = (rad * sn) * radius;
    v3 tangent = normalize3(cross3(center, mk3(0.0f, 1.0f, 0.0f)));
    v3 bitangent = normalize3(cross3(tangent, center));
    return normalize3(add3(add3(center, mul3s(tangent, px)), mul3s(bitangent, py)));
}

static inline uint8_t to_unorm8(float x) {
    float c = fminf(fmaxf(x, 0.0f), 1.0f);
    return (uint8_t)(uint32_t)(c * 255.0f + 0.5f);
}

static void render_chunk(void* a, uint64_t b, uint64_t e, OStats* st) {
    ORenderArgs* A = (ORenderArgs*)a;
    const OScene* s = A->s;
    const RtUniforms* U = A->u;
    const ORenderDesc* D = A->d;
    OTraceCtx prim_ctx = {A->s, A->sbt, 1, RT_RAY_FLAG_NONE, 0xFFu, 0u, st};
    OTraceCtx shadow_ctx = {A->s, A->sbt, 1,
                            RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT | RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER, 0xFFu, 1u,
                            st};
    v3 sun_dir = mk3(U->sun_dir[0], U->sun_dir[1], U->sun_dir[2]);
    float sun_s, sun_c;
    o_sincos_f(U->sun_radius, &sun_s, &sun_c);
    const int dbl = D->double_shading != 0;
    for (uint64_t pi = b; pi < e; pi++) {
        uint32_t x = (uint32_t)(pi % D->width);
        uint32_t y = (uint32_t)(pi / D->width) + D->row_begin;
        /* lib.rs:126-142 */
        float pcx = (float)x + 0.5f, pcy = (float)y + 0.5f;
        float tcx = pcx / (float)D->width, tcy = pcy / (float)D->height;
        float rx = tcx * 2.0f - 1.0f, ry = tcy * 2.0f - 1.0f;
        const float* VI = U->view_inverse;
        const float* PI = U->proj_inverse;
        v3 origin = mk3(mat4_row(VI, 0, 0.0f, 0.0f, 0.0f, 1.0f), mat4_row(VI, 1, 0.0f, 0.0f, 0.0f, 1.0f),
                        mat4_row(VI, 2, 0.0f, 0.0f, 0.0f, 1.0f));
        v3 target = mk3(mat4_row(PI, 0, rx, ry, 1.0f, 1.0f), mat4_row(PI, 1, rx, ry, 1.0f, 1.0f),
                        mat4_row(PI, 2, rx, ry, 1.0f, 1.0f));
        v3 local = normalize3(target);
        v3 dir = mk3(mat4_row(VI, 0, local.x, local.y, local.z, 0.0f),
                     mat4_row(VI, 1, local.x, local.y, local.z, 0.0f),
                     mat4_row(VI, 2, local.x, local.y, local.z, 0.0f));
        double col[3] = {0.0, 0.0, 0.0};
        for (uint32_t bounce = 0; bounce < D->max_trace_depth; bounce++) {
            /* payload reset (lib.rs:145-149) */
            col[0] = col[1] = col[2] = 0.0;
            v3 new_o = mk3(0.0f, 0.0f, 0.0f), new_d = mk3(0.0f, 0.0f, 0.0f);
            OHitRec h;
            if (st) { if (bounce == 0) st->primary_rays++; else st->secondary_rays++; }
            trace_one(&prim_ctx, origin, dir, 0.01f, 10000.0f, &h);
            if (!h.hit) {
                /* primary_ray_miss (lib.rs:40-51) */
                if (dot3(dir, sun_dir) > sun_c) { col[0] = col[1] = col[2] = 1.0; }
                else { col[0] = 0.0; col[1] = 0.0; col[2] = dbl ? 0.05 : (double)0.05f; }
            } else {
                const OInst* in = &s->inst[h.inst];
                const RtHitGroup* g = hit_group(&prim_ctx, in);
                uint32_t prog = g ? g->closest_hit : RT_PROGRAM_NONE;
                OTriData td;
                v3 bary = mk3((1.0f - h.u) - h.v, h.u, h.v);
                if (prog == RT_PROGRAM_CLOSEST_HIT_MIRROR && load_triangle(s, in, h.geom, h.prim, &td)) {
                    /* closest_hit_mirror.glsl:11-29 */
                    v3 ni = interp3(td.n[0], td.n[1], td.n[2], bary);
                    v3 n = normalize3(xform_normal_w2o_t(in->w2o, ni));
                    float k = 2.0f * dot3(n, dir);
                    new_d = sub3(dir, mul3s(n, k));
                    new_o = add3(origin, mul3s(dir, h.t));
                } else if (prog == RT_PROGRAM_CLOSEST_HIT_PORTAL) {
                    /* lib.rs:300-312 */
                    new_d = dir;
                    new_o = add3(add3(origin, mul3s(dir, h.t)), mk3(0.0f, 5.0f, 0.0f));
                } else if (prog == RT_PROGRAM_CLOSEST_HIT_TEXTURED && load_triangle(s, in, h.geom, h.prim, &td)) {
                    /* closest_hit_textured.glsl:174-226 */
                    v3 ip = interp3(td.p[0], td.p[1], td.p[2], bary);
                    v3 inrm = interp3(td.n[0], td.n[1], td.n[2], bary);
                    v2 iuv = interp2(td.uv[0], td.uv[1], td.uv[2], bary);
                    v3 so = shadow_terminator_origin(&td, ip, bary, in->o2w);
                    float lit = 0.0f;
                    for (uint32_t i = 0; i < D->shadow_ray_count; i++) {
                        v2 bn = animated_blue_noise(sample_blue_noise(s, U->blue_noise_texture_index, x, y, i),
                                                    U->frame_index);
                        v3 sd = sample_directional_light(bn, sun_dir, U->sun_radius);
                        OHitRec sh;
                        if (st) st->shadow_rays++;
                        trace_one(&shadow_ctx, so, sd, 0.001f, 10000.0f, &sh);
                        /* shadow_ray_miss sets shadowed = 0; a hit leaves 1 */
                        lit += sh.hit ? 0.0f : 1.0f;
                    }
                    float sun_factor = lit / (float)(D->shadow_ray_count ? D->shadow_ray_count : 1);
                    OShadeIn si;
                    si.uv[0] = iuv.x; si.uv[1] = iuv.y;
                    si.interp_normal[0] = inrm.x; si.interp_normal[1] = inrm.y; si.interp_normal[2] = inrm.z;
                    for (int k = 0; k < 3; k++) {
                        si.p[k][0] = td.p[k].x; si.p[k][1] = td.p[k].y; si.p[k][2] = td.p[k].z;
                        si.tuv[k][0] = td.uv[k].x; si.tuv[k][1] = td.uv[k].y;
                    }
                    memcpy(si.w2o, in->w2o, sizeof si.w2o);
                    si.view_dir[0] = dir.x; si.view_dir[1] = dir.y; si.view_dir[2] = dir.z;
                    si.sun_dir[0] = sun_dir.x; si.sun_dir[1] = sun_dir.y; si.sun_dir[2] = sun_dir.z;
                    si.sun_factor = sun_factor;
                    si.lambert = (D->flags & RT_TRACE_FLAG_LAMBERT_DIFFUSE) != 0;
                    si.gi = td.gi;
                    si.textures = s->textures;
                    if (dbl) shade_textured_d(&si, col);
                    else shade_textured_f(&si, col);
                }
            }
            if (new_d.x == 0.0f && new_d.y == 0.0f && new_d.z == 0.0f) break;
            origin = new_o;
            dir = new_d;
        }
        size_t o = ((size_t)y * D->width + x);
        if (A->radiance) {
            A->radiance[4 * o + 0] = (float)col[0];
            A->radiance[4 * o + 1] = (float)col[1];
            A->radiance[4 * o + 2] = (float)col[2];
            A->radiance[4 * o + 3] = 1.0f;
        }
        if (A->image) {
            for (int k = 0; k < 3; k++) {
                double sv = dbl ? linear_to_srgb_d(col[k]) : (double)linear_to_srgb_f((float)col[k]);
                A->image[4 * o + k] = to_unorm8((float)sv);
            }
            A->image[4 * o + 3] = 255;
        }
    }
}

int32_t o_render(OScene* s, const RtUniforms* u, const RtShaderBindingTable* sbt, const ORenderDesc* d,
                 uint8_t* image, float* radiance, int32_t threads, OStats* stats) {
    if (!s || !u || !d || d->width == 0 || d->height == 0) return RT_ERR_INVALID;
    RtShaderBindingTable def;
    if (!sbt) {
        memset(&def, 0, sizeof def);
        def.hit_group_count = 3;
        def.hit_groups[0].closest_hit = RT_PROGRAM_CLOSEST_HIT_TEXTURED;
        def.hit_groups[1].closest_hit = RT_PROGRAM_CLOSEST_HIT_MIRROR;
        def.hit_groups[2].closest_hit = RT_PROGRAM_CLOSEST_HIT_PORTAL;
        for (int i = 0; i < 3; i++) def.hit_groups[i].any_hit = RT_PROGRAM_ANY_HIT_ALPHA_CLIP;
        sbt = &def;
    }
    uint32_t r0 = d->row_begin, r1 = d->row_end ? d->row_end : d->height;
    if (r1 > d->height || r0 >= r1) return RT_ERR_INVALID;
    ORenderDesc dd = *d;
    dd.row_begin = r0;
    dd.row_end = r1;
    ORenderArgs a = {s, u, sbt, &dd, image, radiance};
    pool_run(threads, (uint64_t)(r1 - r0) * d->width, 4096, render_chunk, &a, stats);
    return 0;
}

/* ===================================================================== */
/* Element-wise function evaluation                                        */
/* ===================================================================== */
int32_t o_debug_eval(uint32_t fn, const float* in, float* out, uint32_t count, int32_t dbl) {
    for (uint32_t i = 0; i < count; i++) {
        switch (fn) {
            case RT_FN_V_SMITH_GGX_CORRELATED:
                out[i] = dbl ? (float)v_smith_ggx_correlated_d(in[3 * i], in[3 * i + 1], in[3 * i + 2])
                             : v_smith_ggx_correlated_f(in[3 * i], in[3 * i + 1], in[3 * i + 2]);
                break;
            case RT_FN_D_GGX:
                out[i] = dbl ? (float)d_ggx_d(in[2 * i], in[2 * i + 1]) : d_ggx_f(in[2 * i], in[2 * i + 1]);
                break;
            case RT_FN_LINEAR_TO_SRGB:
                out[i] = dbl ? (float)linear_to_srgb_d(in[i]) : linear_to_srgb_f(in[i]);
                break;
            case RT_FN_HEATMAP: {
                float rgb[3];
                heatmap_temperature_f(in[i], rgb);
                out[3 * i] = rgb[0]; out[3 * i + 1] = rgb[1]; out[3 * i + 2] = rgb[2];
                break;
            }
            case RT_FN_SINCOS: {
                if (dbl) { out[2 * i] = (float)sin((double)in[i]); out[2 * i + 1] = (float)cos((double)in[i]); }
                else o_sincos_f(in[i], &out[2 * i], &out[2 * i + 1]);
                break;
            }
            case RT_FN_BRDF: {
                /* in: normal3, view3, light3, perceptual_roughness, base3, metallic, intensity, lambert */
                const float* p = in + 16 * (size_t)i;
                double rgb[3];
                if (dbl) brdf_d(p, rgb); else brdf_f(p, rgb);
                out[3 * i] = (float)rgb[0]; out[3 * i + 1] = (float)rgb[1]; out[3 * i + 2] = (float)rgb[2];
                break;
            }
            case RT_FN_WATERTIGHT: {
                /* in: o3, d3, v0 3, v1 3, v2 3, tmin -> out: hit, t, u, v */
                const float* p = in + 16 * (size_t)i;
                ORay r;
                ray_setup(&r, mk3(p[0], p[1], p[2]), mk3(p[3], p[4], p[5]));
                float t = 0, u = 0, v = 0;
                int front = 0;
                int h = tri_intersect(&r, mk3(p[6], p[7], p[8]), mk3(p[9], p[10], p[11]),
                                      mk3(p[12], p[13], p[14]), p[15], INFINITY, &t, &u, &v, &front);
                out[4 * i] = h ? (front ? 1.0f : -1.0f) : 0.0f;
                out[4 * i + 1] = h ? t : 0.0f;
                out[4 * i + 2] = h ? u : 0.0f;
                out[4 * i + 3] = h ? v : 0.0f;
                break;
            }
            default:
                return RT_ERR_INVALID;
        }
    }
    return 0;
}
