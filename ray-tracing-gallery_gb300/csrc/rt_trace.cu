// rt_trace.cu — traversal, and the reference's pipeline as wavefronts.
//
// Traversal (replaces the driver's traceRayEXT, called at
// shaders/ray-tracing/src/lib.rs:67-82,151-163 and
// shaders/closest_hit_textured.glsl:159-172) runs in persistent kernels: a
// lane holds one ray, advances it by exactly one step per loop iteration
// (one 8-wide node, one leaf, or a return from an instance), and as soon as
// its ray finishes it takes the next one from a warp-aggregated atomic
// counter — so lanes never wait for the slowest ray of their warp.  A node
// step reads the 256-byte node with 128-bit loads, runs the eight slab tests
// and orders the hit children front to back with a 19-comparator sorting
// network on (tnear bits | slot) keys.  Leaves run the watertight FP32
// triangle test; non-opaque candidates run the alpha-clip any-hit inline.
// The closest hit is the minimum under (t, instance index, geometry index,
// primitive index), so the result does not depend on the BVH or visit order.
// Coherent wavefront lists (camera rays in 8x4 pixel tiles) can instead be
// traversed as warp packets (k_trace_packet): one node sequence for the
// union of 32 neighbouring rays, the same hits.
//
// Pipeline (replaces cmd_trace_rays, src/command_buffer_recording.rs:116-126,
// with the programs of src/main.rs:289-305), one frame:
//   setup -> raygen -> trace closest (every mirror / portal bounce followed
//   in the traversal) -> shade -> trace shadow rays (any hit, terminate on
//   first) -> resolve -> output
// `shade` runs the closest-hit / miss programs for the last ray of every
// slot: misses and terminal hits write the pixel's colour; textured hits
// store their BRDF terms and shadow origin and append the pixel's shadow
// rays.  Appends are warp-aggregated (one atomic per list per warp), which
// compacts the wavefronts.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "rt_internal.h"
#include "rt_shade.cuh"

namespace rt {

namespace {

// Stack entries: internal node index (bit 31 clear, < 2^30); leaf =
// bit 31 | (count - 1) << 28 | first primitive; kMarker = return to the
// TLAS.  kNoEntry would be a leaf of 8 primitives starting at 2^28 - 1,
// which no structure can hold (primitive counts are < 2^28), so it is free
// to mean "done".
constexpr uint32_t kStackSize = 64;
constexpr uint32_t kMarker = 0x7FFFFFFFu;
constexpr uint32_t kLeafEntry = 0x80000000u;
constexpr uint32_t kNoEntry = 0xFFFFFFFFu;
constexpr uint32_t kNoPixel = 0xFFFFFFFFu;
constexpr uint32_t kNoItem = 0xFFFFFFFFu;
// Upper bound of traversal steps of one ray; reaching it means a malformed
// structure: the ray stops and RT_ERR_TIMEOUT is recorded.
constexpr uint32_t kMaxTraversalSteps = 1u << 22;
constexpr int kTraceThreads = 128;
constexpr int kMaxDepth = 64;
// Warp phase scheduling.  Each iteration of the traversal loop runs either
// node steps (lanes whose next entry is an internal node) or the other steps
// (leaves, instance entries, TLAS returns), so a warp never pays for both
// branch bodies in one iteration.  Lanes wait for their phase: the warp
// switches to the leaf phase once leaf_wait/32 of its active lanes wait on
// one (or no lane has a node).  The default; the wavefront launches take it
// from the context's traversal configuration.
#ifndef RT_TRACE_LEAF_WAIT
#define RT_TRACE_LEAF_WAIT 20
#endif
// Resident warps per SM every trace kernel variant is compiled for (at most
// 80 registers a thread); block size x blocks per SM = 24 warps.
constexpr int kTraceWarpsPerSM = 24;
// Kernels that decode only quantised BLAS nodes hold fewer node registers.
// The ray-buffer query runs them at 32 warps per SM (at most 64 registers a
// thread: random rays over a hierarchy larger than L2 want the most rays in
// flight); the wavefront launches at 24 (80 registers, fewer spills: the
// 64-scene batch's shadow launch 12.5 -> 12.1 ms; 20 and 28 warps were
// slower).
#ifndef RT_Q8_TRACE_WARPS
#define RT_Q8_TRACE_WARPS 24
#endif
#ifndef RT_Q8_RAYBUF_WARPS
#define RT_Q8_RAYBUF_WARPS 32
#endif
constexpr int trace_warps_per_sm(uint32_t kinds) { return kinds == kBlasKindQ8 ? RT_Q8_TRACE_WARPS : kTraceWarpsPerSM; }
constexpr int raybuf_warps_per_sm(uint32_t kinds) {
    return kinds == kBlasKindQ8 ? RT_Q8_RAYBUF_WARPS : kTraceWarpsPerSM;
}

constexpr int kModeBounce = 0;   // closest hit of a bounce list -> hit records
constexpr int kModeShadow = 1;   // any hit of generated shadow rays -> lit counters

// Work counters of one lane (RT_TRACE_FLAG_COLLECT_STATS launches only).
struct Counters {
    uint32_t nodes, tris, insts, qnodes;  // qnodes: of `nodes`, the quantised ones
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Index for this lane in a warp-aggregated append (one atomic per warp).
// Every converged lane must call it; `pred` selects the appending lanes.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool pred) {
    unsigned m = __activemask();
    unsigned b = __ballot_sync(m, pred);
    uint32_t base = 0;
    if (b) {
        int leader = __ffs(b) - 1;
        if ((int)(threadIdx.x & 31u) == leader) base = atomicAdd(counter, (uint32_t)__popc(b));
        base = __shfl_sync(m, base, leader);
    }
    return base + __popc(b & lanemask_lt());
}

// Three-input min / max (one instruction on sm_100 and later).  Like fminf
// / fmaxf they return the non-NaN operand; the box test never produces NaN.
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Float4 offsets (within a node) of the near-plane box arrays for each axis,
// from the signs of the reciprocal direction: x at 0 (lox) or 2 (hix), y at
// 4 or 6, z at 8 or 10; the far plane is at offset ^ 2.
__device__ __forceinline__ uint32_t octant_offsets(V3 inv) {
    return (inv.x < 0.0f ? 2u : 0u) | ((inv.y < 0.0f ? 6u : 4u) << 8) | ((inv.z < 0.0f ? 10u : 8u) << 16);
}

__device__ __forceinline__ uint32_t pick8(const uint32_t v[8], uint32_t s) {
    uint32_t r = v[0];
#pragma unroll
    for (int j = 1; j < 8; j++) r = (s == (uint32_t)j) ? v[j] : r;
    return r;
}

#define RT_CSWAP(a, b)                  \
    {                                   \
        uint32_t lo_ = min(k[a], k[b]); \
        uint32_t hi_ = max(k[a], k[b]); \
        k[a] = lo_;                     \
        k[b] = hi_;                     \
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

// ---------------------------------------------------------------------------
// Traversal state of one ray (one lane)
// ---------------------------------------------------------------------------
struct Trav {
    V3 wo, wd;                 // world ray
    V3 o, d, inv;              // ray in the current space (world or object)
    uint32_t oct;              // octant_offsets(inv)
    WtRay wt;                  // watertight shear of the object-space ray
    float tmin;
    float t, u, v;             // best hit so far (t = tmax before any hit)
    uint32_t hit_inst;         // sorted TLAS index of the best hit, kNoHit if none
    uint32_t hit_geom, hit_prim;
    bool front, in_blas;
    bool quant;                // current nodes are QNodes (a quantised BLAS)
    uint32_t entry;            // what the next step processes
    int sp;
    const WideNode* nodes;
    const TriRecord* tris;
    uint32_t node_count, tri_count;
    uint32_t c_inst, c_sbt_flags;  // the instance being traversed
    uint32_t steps;
    uint32_t scene;            // the ray's scene in a batched launch
};

__device__ __forceinline__ void trav_begin(Trav& s, const Env& e, V3 o, V3 d, float tmin, float tmax) {
    s.wo = o;
    s.wd = d;
    s.o = o;
    s.d = d;
    s.inv = safe_inv(d);
    s.oct = octant_offsets(s.inv);
    s.wt.kx = s.wt.ky = s.wt.kz = 0;
    s.wt.sx = s.wt.sy = s.wt.sz = 0.0f;
    s.tmin = tmin;
    s.t = tmax;
    s.u = s.v = 0.0f;
    s.hit_inst = kNoHit;
    s.hit_geom = s.hit_prim = kNoHit;
    s.front = false;
    s.in_blas = false;
    s.sp = 0;
    s.nodes = e.tnodes;
    s.tris = nullptr;
    s.node_count = e.tnode_count;
    s.quant = false;
    s.tri_count = 0;
    s.c_inst = 0;
    s.c_sbt_flags = 0;
    s.steps = 0;
    s.entry = (e.tnode_count == 0 || !(tmin <= tmax)) ? kNoEntry : 0u;  // 0 = TLAS root
}

// The traversal stack of one lane: kStackSize entries (node/leaf entry,
// tnear bits).  The first SD live in shared memory (a column per thread,
// stride BLOCK, so a warp's accesses are conflict-free), the rest in local
// memory; SD = 0 keeps all of it local.  The split only moves entries, so
// every depth gives the same hits; the autotuner picks SD by speed.
template <int SD, int BLOCK>
struct TravStack {
    uint2* sh;                                  // this thread's column in dynamic shared memory
    uint2 lo[kStackSize - SD];
    __device__ __forceinline__ void put(int i, uint2 v) {
        if (SD > 0 && i < SD) sh[i * BLOCK] = v;
        else lo[i - SD] = v;
    }
    __device__ __forceinline__ uint2 get(int i) const { return (SD > 0 && i < SD) ? sh[i * BLOCK] : lo[i - SD]; }
};

template <class STK>
__device__ __forceinline__ void trav_pop(Trav& s, const STK& stack) {
    const float cull = s.t * kBoxFarScale;
    while (s.sp > 0) {
        uint2 en = stack.get(--s.sp);
        if (en.x != kMarker && __uint_as_float(en.y) > cull) continue;
        s.entry = en.x;
        return;
    }
    s.entry = kNoEntry;
}

__device__ __forceinline__ void trav_restore_world(Trav& s, const Env& e) {
    s.in_blas = false;
    s.nodes = e.tnodes;
    s.node_count = e.tnode_count;
    s.quant = false;
    s.o = s.wo;
    s.d = s.wd;
    s.inv = safe_inv(s.wd);
    s.oct = octant_offsets(s.inv);
}

// Sort key of a child: tnear bits rounded down to 8 ulps | slot (ascending =
// near first); 0xFFFFFFFF when the child is missed or empty.
__device__ __forceinline__ uint32_t child_key(float tn, float tf, uint32_t ref, int k) {
    bool hit = (ref != kChildEmpty) && (tn <= tf * kBoxFarScale);
    return hit ? ((__float_as_uint(fmaxf(tn, 0.0f)) & ~7u) | (uint32_t)k) : 0xFFFFFFFFu;
}

// Slab tests of four children (base 0 or 4) of an FP32 node from their
// near / far plane float4s.
__device__ __forceinline__ void fnode_keys4(const Trav& s, float4 nx, float4 fx, float4 ny, float4 fy, float4 nz,
                                            float4 fz, uint4 r, int base, uint32_t keys[8], uint32_t refs[8]) {
    const float a_nx[4] = {nx.x, nx.y, nx.z, nx.w}, a_fx[4] = {fx.x, fx.y, fx.z, fx.w};
    const float a_ny[4] = {ny.x, ny.y, ny.z, ny.w}, a_fy[4] = {fy.x, fy.y, fy.z, fy.w};
    const float a_nz[4] = {nz.x, nz.y, nz.z, nz.w}, a_fz[4] = {fz.x, fz.y, fz.z, fz.w};
    const uint32_t a_r[4] = {r.x, r.y, r.z, r.w};
    const float tcap = s.t;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        float tnx = (a_nx[j] - s.o.x) * s.inv.x, tfx = (a_fx[j] - s.o.x) * s.inv.x;
        float tny = (a_ny[j] - s.o.y) * s.inv.y, tfy = (a_fy[j] - s.o.y) * s.inv.y;
        float tnz = (a_nz[j] - s.o.z) * s.inv.z, tfz = (a_fz[j] - s.o.z) * s.inv.z;
        refs[base + j] = a_r[j];
        keys[base + j] =
            child_key(fmax3(fmaxf(tnx, s.tmin), tny, tnz), fmin3(fminf(tfx, tcap), tfy, tfz), a_r[j], base + j);
    }
}

// Slab tests of an FP32 node.  Near / far planes were chosen per ray by the
// direction signs (s.oct): the loads fetch them directly, so each child needs
// one subtract and one multiply per plane and no per-axis min/max.  All eight
// slots are tested (empty ones never hit): skipping children 4-7 of nodes
// with at most four children measured slower than the branch saves, 4-wide
// builds included.
// Node loads: read-only global loads, or plain loads of a copy the warp
// staged in shared memory (packet traversal, RT_PACKET_STAGE).
template <bool GLOBAL, class T>
__device__ __forceinline__ T ldn(const T* p) {
    if constexpr (GLOBAL) return __ldg(p);
    else return *p;
}

template <bool GLOBAL = true>
__device__ __forceinline__ void fnode_keys_at(const Trav& s, const float4* np, uint32_t keys[8], uint32_t refs[8]) {
    const uint32_t ox = s.oct & 0xFFu, oy = (s.oct >> 8) & 0xFFu, oz = s.oct >> 16;
    const uint4 r0 = ldn<GLOBAL>(reinterpret_cast<const uint4*>(np + 12));
    const uint4 r1 = ldn<GLOBAL>(reinterpret_cast<const uint4*>(np + 13));
    const float4 nx0 = ldn<GLOBAL>(np + ox), fx0 = ldn<GLOBAL>(np + (ox ^ 2u)), ny0 = ldn<GLOBAL>(np + oy);
    const float4 fy0 = ldn<GLOBAL>(np + (oy ^ 2u)), nz0 = ldn<GLOBAL>(np + oz), fz0 = ldn<GLOBAL>(np + (oz ^ 2u));
    const float4 nx1 = ldn<GLOBAL>(np + ox + 1), fx1 = ldn<GLOBAL>(np + (ox ^ 2u) + 1), ny1 = ldn<GLOBAL>(np + oy + 1);
    const float4 fy1 = ldn<GLOBAL>(np + (oy ^ 2u) + 1), nz1 = ldn<GLOBAL>(np + oz + 1);
    const float4 fz1 = ldn<GLOBAL>(np + (oz ^ 2u) + 1);
    fnode_keys4(s, nx0, fx0, ny0, fy0, nz0, fz0, r0, 0, keys, refs);
    fnode_keys4(s, nx1, fx1, ny1, fy1, nz1, fz1, r1, 4, keys, refs);
}
__device__ __forceinline__ void fnode_keys(const Trav& s, uint32_t entry, uint32_t keys[8], uint32_t refs[8]) {
    fnode_keys_at<true>(s, reinterpret_cast<const float4*>(s.nodes + entry), keys, refs);
}

// Byte j of w as the float 1 + q 2^-15: q lands in mantissa bits 8..15 of
// 1.0f (one PRMT).  The constant offset 2^15 quanta is folded into the
// per-node term below, where it costs 2^-9 of a quantum at most.
__device__ __forceinline__ float qbyte(uint32_t w, int j) {
    return __int_as_float((int)__byte_perm(w, 0x3F800000u, 0x7604u | ((uint32_t)j << 4)));
}

// Exact decode (plane = origin + q s is an exact float by construction; then
// the FP32 node's arithmetic, which is conservative for those planes).  Only
// used when a node's scale times the ray's inverse direction is outside
// [2^-100, 2^100], where the fast form's products could underflow or
// overflow.
struct Keys8 {
    uint32_t k[8];
};
__device__ __noinline__ Keys8 qnode_keys_exact(const uint8_t* node, float ox, float oy, float oz, float ix, float iy,
                                               float iz, float tmin, float tmax) {
    const QNode* q = reinterpret_cast<const QNode*>(node);
    const float o[3] = {ox, oy, oz}, inv[3] = {ix, iy, iz};
    const uint8_t* qlo[3] = {q->qlo_x, q->qlo_y, q->qlo_z};
    const uint8_t* qhi[3] = {q->qhi_x, q->qhi_y, q->qhi_z};
    Keys8 out;
    for (int k = 0; k < 8; k++) {
        float tn = tmin, tf = tmax;
        for (int a = 0; a < 3; a++) {
            const float sc = __uint_as_float((uint32_t)q->exp[a] << 23);
            const bool pos = inv[a] >= 0.0f;
            float pn = fmaf((float)(pos ? qlo[a][k] : qhi[a][k]), sc, q->origin[a]);
            float pf = fmaf((float)(pos ? qhi[a][k] : qlo[a][k]), sc, q->origin[a]);
            tn = fmaxf(tn, (pn - o[a]) * inv[a]);
            tf = fminf(tf, (pf - o[a]) * inv[a]);
        }
        out.k[k] = child_key(tn, tf, q->child_ref[k], k);
    }
    return out;
}

// Slab tests of a quantised node, conservative by an error bound.  Per axis,
// with quantum s, A = s inv and B = (origin - o) inv, the plane of byte q is
// at t = q A + B = (1 + q 2^-15) (2^15 A) + (B - 2^15 A): one PRMT (the byte
// as the float 1 + q 2^-15) and one FMA per plane; the near / far byte words
// are fetched by the ray's octant (s.oct) like the FP32 node's planes.
// Against the exact slab distance (plane - o) / d, the computed t errs by at
// most about 6u|t| + 0.004|A| (u = 2^-24: the reciprocal, the two roundings
// of B, the rounding of B - 2^15 A and the final FMA, with |B - 2^15 A| <=
// |t| + 33023|A|).  Each near plane is therefore lowered and each far plane
// raised by 0.008|A| (folded into the constant term), and the combined entry
// / exit distances are moved out by 16u of themselves before tmin / the
// current hit distance bound them.  The test is thus never narrower than the
// exact test of the quantised box, which contains the padded FP32 child box
// (the builder rounds every plane outward): every child an FP32 traversal
// would need is visited, so the hits are identical, whatever the distance
// between the ray origin and the node.
template <bool GLOBAL = true>
__device__ __forceinline__ void qnode_keys_at(const Trav& s, const uint8_t* node, uint32_t keys[8],
                                              uint32_t refs[8]) {
    const uint4* qp = reinterpret_cast<const uint4*>(node);
    const uint2* q2 = reinterpret_cast<const uint2*>(node);
    uint4 h = ldn<GLOBAL>(qp), r0 = ldn<GLOBAL>(qp + 1), r1 = ldn<GLOBAL>(qp + 2);
    // uint2 index of the near-plane words: qlo at 6 + 2a, qhi at 7 + 2a
    const uint32_t ix = 6u + ((s.oct & 0xFFu) >> 1), iy = 6u + (((s.oct >> 8) & 0xFFu) >> 1),
                   iz = 6u + ((s.oct >> 16) >> 1);
    uint2 nx = ldn<GLOBAL>(q2 + ix), fx = ldn<GLOBAL>(q2 + (ix ^ 1u));
    uint2 ny = ldn<GLOBAL>(q2 + iy), fy = ldn<GLOBAL>(q2 + (iy ^ 1u));
    uint2 nz = ldn<GLOBAL>(q2 + iz), fz = ldn<GLOBAL>(q2 + (iz ^ 1u));
    refs[0] = r0.x; refs[1] = r0.y; refs[2] = r0.z; refs[3] = r0.w;
    refs[4] = r1.x; refs[5] = r1.y; refs[6] = r1.z; refs[7] = r1.w;
    const float Ax = __uint_as_float((h.w & 0xFFu) << 23) * s.inv.x;
    const float Ay = __uint_as_float(((h.w >> 8) & 0xFFu) << 23) * s.inv.y;
    const float Az = __uint_as_float(((h.w >> 16) & 0xFFu) << 23) * s.inv.z;
    const float ax = fabsf(Ax), ay = fabsf(Ay), az = fabsf(Az);
    if (!(fmin3(ax, ay, az) >= 7.88860905e-31f && fmax3(ax, ay, az) <= 1.26765060e30f)) {  // 2^-100, 2^100
        Keys8 kk = qnode_keys_exact(node, s.o.x, s.o.y, s.o.z, s.inv.x, s.inv.y, s.inv.z, s.tmin, s.t);
#pragma unroll
        for (int k = 0; k < 8; k++) keys[k] = kk.k[k];
        return;
    }
    const float Bx = (__uint_as_float(h.x) - s.o.x) * s.inv.x;
    const float By = (__uint_as_float(h.y) - s.o.y) * s.inv.y;
    const float Bz = (__uint_as_float(h.z) - s.o.z) * s.inv.z;
    const float Sx = Ax * 32768.0f, Sy = Ay * 32768.0f, Sz = Az * 32768.0f;
    const float Cx = fmaf(-32768.0f, Ax, Bx), Cy = fmaf(-32768.0f, Ay, By), Cz = fmaf(-32768.0f, Az, Bz);
    const float Nx = fmaf(-kQuantMargin, ax, Cx), Ny = fmaf(-kQuantMargin, ay, Cy), Nz = fmaf(-kQuantMargin, az, Cz);
    const float Fx = fmaf(kQuantMargin, ax, Cx), Fy = fmaf(kQuantMargin, ay, Cy), Fz = fmaf(kQuantMargin, az, Cz);
    const float tcap = s.t, tlo = s.tmin;
#pragma unroll
    for (int k = 0; k < 8; k++) {
        const int j = k & 3;
        const uint32_t wnx = k < 4 ? nx.x : nx.y, wfx = k < 4 ? fx.x : fx.y;
        const uint32_t wny = k < 4 ? ny.x : ny.y, wfy = k < 4 ? fy.x : fy.y;
        const uint32_t wnz = k < 4 ? nz.x : nz.y, wfz = k < 4 ? fz.x : fz.y;
        const float tn = fmax3(fmaf(qbyte(wnx, j), Sx, Nx), fmaf(qbyte(wny, j), Sy, Ny), fmaf(qbyte(wnz, j), Sz, Nz));
        const float tf = fmin3(fmaf(qbyte(wfx, j), Sx, Fx), fmaf(qbyte(wfy, j), Sy, Fy), fmaf(qbyte(wfz, j), Sz, Fz));
        keys[k] = child_key(fmaxf(fmaf(-kQuantRelative, fabsf(tn), tn), tlo),
                            fminf(fmaf(kQuantRelative, fabsf(tf), tf), tcap), refs[k], k);
    }
}
__device__ __forceinline__ void qnode_keys(const Trav& s, uint32_t entry, uint32_t keys[8], uint32_t refs[8]) {
    qnode_keys_at<true>(s, reinterpret_cast<const uint8_t*>(s.nodes) + (size_t)entry * kQNodeBytes, keys, refs);
}

// (inst, geom, prim) below the best hit's, comparing caller instance indices
// (only reached on an exact tie in t).
__device__ __noinline__ bool ids_below_best(const InstRecord* insts, uint32_t c_inst, uint32_t hit_inst,
                                            uint32_t geom, uint32_t prim, uint32_t hit_geom, uint32_t hit_prim) {
    uint32_t ci = insts[c_inst].instance_id, bi = insts[hit_inst].instance_id;
    if (ci != bi) return ci < bi;
    if (geom != hit_geom) return geom < hit_geom;
    return prim < hit_prim;
}

// Moves the lane's ray into the object space of TLAS instance `first` (its
// record's BLAS fields q0 = blas lo, blas hi, instance_id, custom_mask and
// q1 = sbt_flags, tri_count, node_count, prims_off256).
__device__ __forceinline__ void enter_instance(Trav& s, const InstRecord* ir, uint4 q0, uint4 q1, uint32_t first) {
    const float4* wp = reinterpret_cast<const float4*>(ir->w2o);
    float4 w0 = __ldg(wp), w1 = __ldg(wp + 1), w2 = __ldg(wp + 2);
    const float w[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
    s.o = xform_point(w, s.wo);
    s.d = xform_dir(w, s.wd);
    s.inv = safe_inv(s.d);
    s.oct = octant_offsets(s.inv);
    s.wt = wt_setup(s.d);
    const uint8_t* blas = reinterpret_cast<const uint8_t*>(((uint64_t)q0.y << 32) | q0.x);
    s.nodes = reinterpret_cast<const WideNode*>(blas + kHeaderBytes);
    s.tris = reinterpret_cast<const TriRecord*>(blas + (uint64_t)q1.w * 256u);
    s.node_count = q1.z & ~kQuantizedBlasBit;
    s.quant = (q1.z & kQuantizedBlasBit) != 0u;
    s.tri_count = q1.y;
    s.c_inst = first;
    s.c_sbt_flags = q1.x;
    s.in_blas = true;
}

// Triangle `idx` of the current BLAS against the lane's ray: the opacity and
// facing flags of the ray and the instance, the watertight test, the
// total-order tie break and the alpha-clip any-hit.  An accepted triangle
// becomes the best hit and the call returns true.
template <bool STATS, class SV>
__device__ __forceinline__ bool try_triangle(Trav& s, const SV& sv, const RtShaderBindingTable* sbt,
                                             uint32_t ray_flags, uint32_t ray_sbt_offset, uint32_t idx,
                                             Counters& cnt) {
    const uint32_t iflags = s.c_sbt_flags >> 24;
    if (STATS) cnt.tris++;
    const float4* tp = reinterpret_cast<const float4*>(s.tris + idx);
    float4 p0 = __ldg(tp), p1 = __ldg(tp + 1), p2 = __ldg(tp + 2);
    uint32_t prim = __float_as_uint(p0.w), geom = __float_as_uint(p1.w), tfl = __float_as_uint(p2.w);
    bool opaque = (tfl & 1u) != 0u;
    if (iflags & RT_INSTANCE_FORCE_OPAQUE) opaque = true;
    if (iflags & RT_INSTANCE_FORCE_NO_OPAQUE) opaque = false;
    if (ray_flags & RT_RAY_FLAG_OPAQUE) opaque = true;
    if (ray_flags & RT_RAY_FLAG_NO_OPAQUE) opaque = false;
    if ((ray_flags & RT_RAY_FLAG_CULL_OPAQUE) && opaque) return false;
    if ((ray_flags & RT_RAY_FLAG_CULL_NO_OPAQUE) && !opaque) return false;
    float t, u, v;
    bool front;
    if (!tri_intersect(s.o, s.wt, mk3(p0.x, p0.y, p0.z), mk3(p1.x, p1.y, p1.z), mk3(p2.x, p2.y, p2.z), s.tmin, s.t,
                       &t, &u, &v, &front))
        return false;
    if (iflags & RT_INSTANCE_TRIANGLE_FLIP_FACING) front = !front;
    if (!(iflags & RT_INSTANCE_TRIANGLE_FACING_CULL_DISABLE)) {
        if ((ray_flags & RT_RAY_FLAG_CULL_BACK_FACING) && !front) return false;
        if ((ray_flags & RT_RAY_FLAG_CULL_FRONT_FACING) && front) return false;
    }
    if (t == s.t && s.hit_inst != kNoHit &&
        !ids_below_best(sv(s.scene).insts, s.c_inst, s.hit_inst, geom, prim, s.hit_geom, s.hit_prim))
        return false;
    if (!opaque) {
        const Env e = sv(s.scene);
        const RtHitGroup* g = e.models ? hit_group(sbt, s.c_sbt_flags, ray_sbt_offset) : nullptr;
        if (g && g->any_hit == RT_PROGRAM_ANY_HIT_ALPHA_CLIP &&
            !alpha_clip_accepts(e.models, e.textures, e.texture_count, e.insts[s.c_inst].custom_mask & 0xFFFFFFu,
                                geom, prim, u, v))
            return false;
    }
    s.t = t;
    s.u = u;
    s.v = v;
    s.hit_inst = s.c_inst;
    s.hit_geom = geom;
    s.hit_prim = prim;
    s.front = front;
    return true;
}

// One traversal step.  Returns true when the ray is finished (s.t/hit_* hold
// the result; with terminate-on-first-hit, any accepted hit finishes it).
// KINDS (kBlasKind* bits) are the BLAS node formats this instantiation
// decodes: a loop for FP32-only or quantised-only scenes carries no code for
// the other format, so neither pays the other's registers.  An instance of a
// format outside KINDS is reported (RT_ERR_BAD_AS) and skipped.
__device__ __forceinline__ bool is_node_entry(uint32_t entry) {
    return entry != kMarker && (entry & kLeafEntry) == 0u;  // kNoEntry has the leaf bit
}

// The phase of this iteration for the calling (converged) lanes: leaves once
// leaf_wait/32 of them wait on a non-node step (or none has a node).
__device__ __forceinline__ bool node_phase(uint32_t entry, uint32_t leaf_wait) {
    const unsigned act = __activemask();
    const unsigned nm = __ballot_sync(act, is_node_entry(entry));
    if (nm == 0u) return false;
    if (nm == act) return true;
    return (uint32_t)__popc(act & ~nm) * 32u < leaf_wait * (uint32_t)__popc(act);
}

// `phase`: 1 = node steps only, 0 = non-node steps only, -1 = any step.
// One scene of a wavefront launch, in device memory (written by k_setup).
struct alignas(128) SceneRec {
    Env env;
    const RtUniforms* uniforms;
    uint32_t* image;           // RGBA8, may be null
    float4* radiance;          // may be null
    uint32_t width, height, max_depth, shadow_count;
    uint32_t flags;            // RT_TRACE_FLAG_* of this scene
    uint32_t tiles_x;          // 8x4 tiles per row
    uint32_t tile_begin;       // first tile of the batch's tile list
    uint32_t pixel_begin;      // first pixel of the batch's pixel list
};
static_assert(sizeof(SceneRec) == 128, "scene record size");

struct OneScene {
    Env e;
    __device__ __forceinline__ const Env& operator()(uint32_t) const { return e; }
};
struct SceneTable {
    const SceneRec* recs;
    __device__ __forceinline__ Env operator()(uint32_t i) const { return recs[i].env; }
};

// SV maps the ray's scene index to its Env: OneScene (the ray-buffer query,
// registers) or SceneTable (the wavefront pipeline, one device record per
// scene; loaded only on instance entry / exit and in leaves).
template <bool STATS, uint32_t KINDS, class SV, class STK>
__device__ __forceinline__ bool trav_step(Trav& s, STK& stack, const SV& sv, const RtShaderBindingTable* sbt,
                                          uint32_t* status, uint32_t ray_flags, uint32_t cull_mask,
                                          uint32_t ray_sbt_offset, Counters& cnt, int phase) {
    const uint32_t entry = s.entry;
    if (entry == kNoEntry) return true;
    if (phase >= 0 && is_node_entry(entry) != (phase == 1)) return false;  // waits for its phase
    if (++s.steps > kMaxTraversalSteps) {
        atomicOr(status, 1u << RT_ERR_TIMEOUT);
        return true;
    }
    if (entry == kMarker) {
        trav_restore_world(s, sv(s.scene));
    } else if ((entry & kLeafEntry) == 0) {
        if (entry >= s.node_count) {
            atomicOr(status, 1u << RT_ERR_BAD_AS);  // malformed reference: skip it
        } else {
            if (STATS) cnt.nodes++;
            uint32_t keys[8], refs[8];
            // TLAS nodes are always FP32
            if ((KINDS & kBlasKindQ8) && s.in_blas && (KINDS == kBlasKindQ8 || s.quant)) {
                if (STATS) cnt.qnodes++;
                qnode_keys(s, entry, keys, refs);
            } else {
                fnode_keys(s, entry, keys, refs);
            }
            if (ray_flags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT) {
                // Any accepted hit ends the ray and t never shrinks before
                // that, so neither the visit order nor the stored tnear
                // matters: the hit children go on the stack unsorted.
                uint32_t mask = 0;
#pragma unroll
                for (int k = 0; k < 8; k++) mask |= (keys[k] != 0xFFFFFFFFu ? 1u : 0u) << k;
                if (mask) {
                    s.entry = pick8(refs, (uint32_t)(__ffs(mask) - 1));
                    mask &= mask - 1u;
                    while (mask) {
                        const uint32_t k = (uint32_t)(__ffs(mask) - 1);
                        mask &= mask - 1u;
                        if (s.sp < (int)kStackSize) stack.put(s.sp++, make_uint2(pick8(refs, k), 0u));
                        else atomicOr(status, 1u << RT_ERR_STACK_OVERFLOW);
                    }
                    return false;
                }
            } else {
                sort8(keys);
                if (keys[0] != 0xFFFFFFFFu) {
                    // push the other hit children farthest first; the nearest
                    // is next.  The stored tnear is rounded down: culling stays
                    // conservative.
#pragma unroll
                    for (int q = 7; q >= 1; q--) {
                        uint32_t key = keys[q];
                        if (key == 0xFFFFFFFFu) continue;
                        const uint32_t ref = pick8(refs, key & 7u);
                        if (s.sp < (int)kStackSize) stack.put(s.sp++, make_uint2(ref, key & ~7u));
                        else atomicOr(status, 1u << RT_ERR_STACK_OVERFLOW);
                    }
                    s.entry = pick8(refs, keys[0] & 7u);
                    return false;
                }
            }
        }
    } else {
        const uint32_t first = entry & 0x0FFFFFFFu;
        const uint32_t count = ((entry >> 28) & 7u) + 1u;
        if (first + count > (s.in_blas ? s.tri_count : sv(s.scene).inst_count)) {
            atomicOr(status, 1u << RT_ERR_BAD_AS);  // malformed leaf: skip it
        } else if (!s.in_blas) {
            // instance leaf: the record's last 32 bytes hold the BLAS fields
            const InstRecord* ir = &sv(s.scene).insts[first];
            const uint4* tail = reinterpret_cast<const uint4*>(&ir->blas);
            uint4 q0 = __ldg(tail), q1 = __ldg(tail + 1);
            // q0 = blas lo, blas hi, instance_id, custom_mask; q1 = sbt_flags, tri_count, node_count, prims_off256
            bool enter = q1.y != 0u && ((q0.w >> 24) & cull_mask) != 0u;
            if (enter && (blas_kind(q1.z) & KINDS) == 0u) {
                atomicOr(status, 1u << RT_ERR_BAD_AS);  // the TLAS header does not list this format
                enter = false;
            }
            if (enter) {
                if (STATS) cnt.insts++;
                enter_instance(s, ir, q0, q1, first);
                if (s.sp < (int)kStackSize) {
                    stack.put(s.sp++, make_uint2(kMarker, 0u));
                    s.entry = 0;  // BLAS root
                    return false;
                }
                atomicOr(status, 1u << RT_ERR_STACK_OVERFLOW);
                trav_restore_world(s, sv(s.scene));
            }
        } else {
            for (uint32_t q = 0; q < count; q++) {
                if (try_triangle<STATS>(s, sv, sbt, ray_flags, ray_sbt_offset, first + q, cnt) &&
                    (ray_flags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT)) {
                    s.entry = kNoEntry;
                    return true;
                }
            }
        }
    }
    trav_pop(s, stack);
    return s.entry == kNoEntry;
}

__device__ __forceinline__ void flush_counters(RtStats* st, const Counters& c) {
    if (c.nodes | c.tris | c.insts) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->nodes_visited), (unsigned long long)c.nodes);
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->triangles_tested), (unsigned long long)c.tris);
        atomicAdd(reinterpret_cast<unsigned long long*>(&st->instances_visited), (unsigned long long)c.insts);
        if (c.qnodes)
            atomicAdd(reinterpret_cast<unsigned long long*>(&st->quantized_nodes_visited),
                      (unsigned long long)c.qnodes);
    }
}

// Rays are counted without per-ray atomics, so the traversal loops carry no
// counters: primary rays once per scene (k_setup), the shadow and bounce
// rays k_shade appended from the list totals (k_output, one thread), mirror /
// portal continuations in the traversal.  (Same-address atomics serialise in
// L2: counting per warp in the ray generation kernel took most of its time.)
__device__ __forceinline__ void count_list_rays(RtStats* st, uint32_t shadow, uint32_t bounce) {
    if (!st || !(shadow | bounce)) return;
    atomicAdd(reinterpret_cast<unsigned long long*>(&st->traversals), (unsigned long long)shadow + bounce);
    if (shadow) atomicAdd(reinterpret_cast<unsigned long long*>(&st->shadow_rays), (unsigned long long)shadow);
    if (bounce) atomicAdd(reinterpret_cast<unsigned long long*>(&st->secondary_rays), (unsigned long long)bounce);
}

// ---------------------------------------------------------------------------
// Wavefront buffers (the per-stream workspace of the context).  A launch
// traces a batch of scenes: their 8x4 pixel tiles and their pixels are
// concatenated into one list each, and every ray carries its scene index,
// so one persistent launch per wavefront serves all scenes.
// ---------------------------------------------------------------------------
struct WfCounters {
    uint32_t ray_count[kMaxDepth + 1];  // rays of each bounce list
    uint32_t shade_count;               // pixels with a textured hit
    uint32_t shadow_count;              // shadow rays
    uint32_t work[kMaxDepth + 2];       // fetch counters of the persistent trace launches
    uint32_t kinds;                     // union of the scenes' TLAS kinds (k_setup)
};

struct WfBuffers {
    float4* rays[2];           // per ray: (origin, tmin), (direction, tmax)
    uint32_t* ray_pixel[2];    // batch pixel of each ray, kNoPixel for padding
    uint32_t* ray_scene[2];    // scene of each ray
    uint4* hits;               // per ray: (t, u, v, inst), (geom, prim, front, 0)
    float4* colour;            // per batch pixel, linear
    float4* shade;             // per pixel: (so.xyz, NoL), (comb.xyz, amb.x), (amb.yz, 0, 0)
    uint32_t* lit;             // per pixel: shadow rays that missed
    uint32_t* shade_list;      // pixels with a textured hit
    float4* shadow_rays;       // per shadow ray: (origin, tmin), (direction, tmax)
    uint32_t* shadow_pixel;    // per shadow ray: its pixel
    uint32_t* shadow_scene;    // per shadow ray: its scene
    unsigned long long* heat;  // per pixel traversal clock cycles (heatmap)
    WfCounters* ctr;
    SceneRec* scenes;
    RtTextureDesc* ctx_textures;  // the context's texture table, copied by k_setup
};

struct WfParams {
    WfBuffers B;
    RtShaderBindingTable sbt;
    RtStats* stats;
    uint32_t* status;
    uint32_t scene_count;
    uint32_t total_slots;      // ray slots of the primary list (tiles * 32)
    uint32_t total_pixels;
    uint32_t bounce;
    uint32_t kinds_built;
    uint32_t leaf_wait;        // phase threshold (node_phase)
};

// Scene of batch tile / pixel v: the last scene whose first tile / pixel is <= v.
template <bool PIXEL>
__device__ __forceinline__ uint32_t scene_of(const WfParams& P, uint32_t v) {
    uint32_t lo = 0, hi = P.scene_count;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        const uint32_t first = PIXEL ? P.B.scenes[mid].pixel_begin : P.B.scenes[mid].tile_begin;
        if (first <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Rays of a persistent shadow-ray launch: a warp takes a chunk of
// consecutive list entries at a time from the launch's counter and its lanes
// take their next rays from that chunk, so the rays one warp works on stay
// neighbours in the list (the shadow rays of neighbouring pixels, which meet
// the same instances).  The chunk is RT_FETCH_CHUNK entries, less for short
// lists (at least 32, and about 8 chunks per resident warp), so a small frame
// still spreads over every warp.  Measured on the 64-scene batch: shadow
// launch 11.65 -> 10.38 ms with chunks of 128 (512: 10.85); the closest-hit
// lists keep the whole-list counter (chunks made them 6 % slower).
#ifndef RT_FETCH_CHUNK
#define RT_FETCH_CHUNK 128
#endif
// Packet traversal: each node is staged through shared memory by the
// sub-packet (1) or read by every lane from global memory (0).
#ifndef RT_PACKET_STAGE
#define RT_PACKET_STAGE 0
#endif

struct WarpChunk {
    uint32_t next = 0, end = 0;  // the same in every lane of the warp
    uint32_t size = 32;
    bool exhausted = false;
    __device__ explicit WarpChunk(uint32_t total) {
        const uint32_t warps = gridDim.x * (blockDim.x >> 5);
        size = min((uint32_t)RT_FETCH_CHUNK, max(32u, total / (8u * warps)));
    }
};
// All 32 lanes call it, converged.  Returns the list entry of a lane that
// wants one, kNoItem if it gets none this time.
__device__ __forceinline__ uint32_t chunk_fetch(WarpChunk& c, uint32_t* work, uint32_t total, bool want) {
    const unsigned need = __ballot_sync(0xFFFFFFFFu, want);
    if (need && c.next >= c.end && !c.exhausted) {
        uint32_t base = 0;
        if ((threadIdx.x & 31u) == 0u) base = atomicAdd(work, c.size);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= total) {
            c.exhausted = true;
        } else {
            c.next = base;
            c.end = min(base + c.size, total);
        }
    }
    uint32_t it = kNoItem;
    if (need && c.next < c.end) {
        const uint32_t r = (uint32_t)__popc(need & lanemask_lt());
        if (want && c.next + r < c.end) it = c.next + r;
        c.next = min(c.next + (uint32_t)__popc(need), c.end);
    }
    return it;
}

// Warp-aggregated append of n items per lane; all 32 lanes must call it.
__device__ __forceinline__ uint32_t warp_append_n(uint32_t* counter, uint32_t n) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t x = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, x, 31);
    uint32_t base = 0;
    if (lane == 31u && total) base = atomicAdd(counter, total);
    base = __shfl_sync(0xFFFFFFFFu, base, 31);
    return base + x - n;
}

constexpr uint32_t kSetupChunk = 64;
struct SceneLayout {
    uint32_t tiles_x, tile_begin, pixel_begin;
};
struct SetupParams {
    TraceScene d[kSetupChunk];
    SceneLayout lay[kSetupChunk];
    RtTextureDesc textures[RT_MAX_BOUND_IMAGES];  // the context's table
    WfBuffers B;
    RtStats* stats;
    uint32_t* status;
    uint32_t first, count;
    uint32_t copy_textures;
};

// Scene records of one chunk of the batch (TLAS header -> Env).
__global__ void k_setup(const __grid_constant__ SetupParams P) {
    const uint32_t t = threadIdx.x;
    if (P.copy_textures)
        for (uint32_t i = t; i < RT_MAX_BOUND_IMAGES; i += blockDim.x) P.B.ctx_textures[i] = P.textures[i];
    if (t >= P.count) return;
    const TraceScene& d = P.d[t];
    SceneRec r;
    const bool own = d.textures != nullptr;
    r.env = make_env(d.push.acceleration_structure, d.push.model_info, own ? d.textures : P.B.ctx_textures,
                     own ? d.texture_count : RT_MAX_BOUND_IMAGES, P.status);
    r.uniforms = reinterpret_cast<const RtUniforms*>(d.push.uniforms);
    r.image = reinterpret_cast<uint32_t*>(d.desc.image_address);
    r.radiance = reinterpret_cast<float4*>(d.desc.radiance_address);
    r.width = d.desc.width;
    r.height = d.desc.height;
    r.max_depth = d.desc.max_trace_depth;
    r.shadow_count = d.desc.shadow_ray_count;
    r.flags = d.desc.flags;
    r.tiles_x = P.lay[t].tiles_x;
    r.tile_begin = P.lay[t].tile_begin;
    r.pixel_begin = P.lay[t].pixel_begin;
    P.B.scenes[P.first + t] = r;
    atomicOr(&P.B.ctr->kinds, r.env.blas_kinds ? r.env.blas_kinds : kBlasKindF32);
    // every pixel traces one primary ray: counted here, once per scene
    const unsigned long long px = (unsigned long long)r.width * r.height;
    if (px && P.stats) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->traversals), px);
        atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->primary_rays), px);
    }
}

// ray_generation, lib.rs:126-142 (camera ray, fixed operation order)
__global__ void k_raygen(const __grid_constant__ WfParams P) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.total_slots) return;
    const uint32_t tile = i >> 5, l = i & 31u;
    const uint32_t sc = scene_of<false>(P, tile);
    const SceneRec& S = P.B.scenes[sc];
    const uint32_t lt = tile - S.tile_begin, W = S.width, H = S.height;
    const uint32_t x = (lt % S.tiles_x) * 8u + (l & 7u), y = (lt / S.tiles_x) * 4u + (l >> 3);
    float4* R = P.B.rays[0];
    if (x < W && y < H) {
        const RtUniforms& U = *S.uniforms;
        float pcx = (float)x + 0.5f, pcy = (float)y + 0.5f;
        float tcx = pcx / (float)W, tcy = pcy / (float)H;
        float rx = tcx * 2.0f - 1.0f, ry = tcy * 2.0f - 1.0f;
        const float* VI = U.view_inverse;
        const float* PI = U.proj_inverse;
        V3 ro = mk3(mat4_row(VI, 0, 0.0f, 0.0f, 0.0f, 1.0f), mat4_row(VI, 1, 0.0f, 0.0f, 0.0f, 1.0f),
                    mat4_row(VI, 2, 0.0f, 0.0f, 0.0f, 1.0f));
        V3 target = mk3(mat4_row(PI, 0, rx, ry, 1.0f, 1.0f), mat4_row(PI, 1, rx, ry, 1.0f, 1.0f),
                        mat4_row(PI, 2, rx, ry, 1.0f, 1.0f));
        V3 local = normalize3(target);
        V3 rd = mk3(mat4_row(VI, 0, local.x, local.y, local.z, 0.0f), mat4_row(VI, 1, local.x, local.y, local.z, 0.0f),
                    mat4_row(VI, 2, local.x, local.y, local.z, 0.0f));
        R[2 * (size_t)i] = make_float4(ro.x, ro.y, ro.z, 0.01f);
        R[2 * (size_t)i + 1] = make_float4(rd.x, rd.y, rd.z, 10000.0f);
        P.B.ray_pixel[0][i] = S.pixel_begin + y * W + x;
    } else {
        R[2 * (size_t)i] = make_float4(0.0f, 0.0f, 0.0f, 1.0f);  // tmin > tmax: never traversed
        R[2 * (size_t)i + 1] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
        P.B.ray_pixel[0][i] = kNoPixel;
    }
    P.B.ray_scene[0][i] = sc;
    if (i == 0) P.B.ctr->ray_count[0] = P.total_slots;
}

// The next bounce ray of a mirror hit (closest_hit_mirror.glsl:11-29:
// reflect about the interpolated world normal) or a portal hit
// (lib.rs:300-312: same direction, origin lifted by (0, 5, 0)); a zero
// direction for any other program or a mirror without model data, which
// ends the reference's bounce loop (lib.rs:165-171).
struct NextRay {
    V3 o, d;
};
__device__ __forceinline__ NextRay next_bounce_ray(const Env& e, const RtShaderBindingTable* sbt, uint32_t inst,
                                                uint32_t geom, uint32_t prim, float t, float hu, float hv, V3 ro,
                                                V3 rd) {
    NextRay r;
    r.o = mk3(0.0f, 0.0f, 0.0f);
    r.d = mk3(0.0f, 0.0f, 0.0f);
    const InstRecord* ir = &e.insts[inst];
    const RtHitGroup* g = hit_group(sbt, ir->sbt_flags, 0u);
    const uint32_t prog = g ? g->closest_hit : RT_PROGRAM_NONE;
    TriData td;
    if (prog == RT_PROGRAM_CLOSEST_HIT_MIRROR && load_triangle(e, ir->custom_mask & 0xFFFFFFu, geom, prim, &td)) {
        const V3 bary = mk3((1.0f - hu) - hv, hu, hv);
        V3 ni = interp3(td.n[0], td.n[1], td.n[2], bary);
        V3 n = normalize3(xform_normal_w2o_t(ir->w2o, ni));
        float k = 2.0f * dot3(n, rd);
        r.d = sub3(rd, mul3s(n, k));
        r.o = add3(ro, mul3s(rd, t));
    } else if (prog == RT_PROGRAM_CLOSEST_HIT_PORTAL) {
        r.d = rd;
        r.o = add3(add3(ro, mul3s(rd, t)), mk3(0.0f, 5.0f, 0.0f));
    }
    return r;
}

// Ray-list scene words carry the ray's bounce depth in their top byte.
constexpr uint32_t kSceneBits = 24;
constexpr uint32_t kSceneMask = (1u << kSceneBits) - 1u;

// Persistent trace loop with per-lane ray replacement.  Bounce lists:
// when a ray's closest hit is a mirror or a portal and the scene's depth
// allows another bounce, the same lane traces the next ray at once (the
// closest-hit program's arithmetic, bit for bit), so every bounce of a pixel
// runs in one launch; the list slot then holds the last ray, its hit and its
// depth for the shading kernel.
template <int MODE, bool STATS, uint32_t KINDS, int SD, int BLOCK>
__device__ __forceinline__ void trace_wavefront(const WfParams& P) {
    const SceneTable sv{P.B.scenes};
    const uint32_t b = P.bounce;
    uint32_t total;
    uint32_t* work;
    if (MODE == kModeBounce) {
        total = P.B.ctr->ray_count[b];
        work = &P.B.ctr->work[b];
    } else {
        total = P.B.ctr->shadow_count;
        work = &P.B.ctr->work[kMaxDepth + 1];
    }
    const uint32_t ray_flags = MODE == kModeShadow
                                   ? (RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT | RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER)
                                   : RT_RAY_FLAG_NONE;
    const uint32_t sbt_offset = MODE == kModeShadow ? 1u : 0u;

    Counters cnt = {0, 0, 0, 0};
    TravStack<SD, BLOCK> stack;
    if (SD > 0) {
        extern __shared__ uint2 stack_smem[];
        stack.sh = stack_smem + threadIdx.x;
    }
    Trav s;
    uint32_t item = kNoItem;
    bool heat = false;
    uint32_t t0 = 0;  // clock() at the ray's start (heatmap only)
    uint32_t depth = 0;  // bits 0-7: depth of the ray being traced; 8-15: depth the slot started at
    WarpChunk chunk(total);
    for (;;) {
        uint32_t my;
        if (MODE == kModeShadow && RT_FETCH_CHUNK) {
            const bool want = item == kNoItem;
            if (__all_sync(0xFFFFFFFFu, want) && chunk.exhausted) break;
            my = chunk_fetch(chunk, work, total, want);
            if (want && my == kNoItem) continue;  // idle until the warp has a ray for it (or is done)
        } else {
            my = warp_append(work, item == kNoItem);
        }
        if (item == kNoItem) {
            if (my >= total) break;
            item = my;
            uint32_t sc, pix;
            if (MODE == kModeBounce) {
                float4 a = P.B.rays[b & 1][2 * (size_t)item], c = P.B.rays[b & 1][2 * (size_t)item + 1];
                pix = P.B.ray_pixel[b & 1][item];
                const uint32_t rs = P.B.ray_scene[b & 1][item];
                sc = rs & kSceneMask;
                depth = (rs >> kSceneBits) * 0x101u;
                trav_begin(s, sv(sc), mk3(a.x, a.y, a.z), mk3(c.x, c.y, c.z), a.w, c.w);
            } else {
                float4 a = P.B.shadow_rays[2 * (size_t)item], c = P.B.shadow_rays[2 * (size_t)item + 1];
                pix = P.B.shadow_pixel[item];
                sc = P.B.shadow_scene[item];
                trav_begin(s, sv(sc), mk3(a.x, a.y, a.z), mk3(c.x, c.y, c.z), a.w, c.w);
            }
            s.scene = sc;
            heat = pix != kNoPixel && P.B.scenes[sc].uniforms->show_heatmap != 0;
            if (heat) t0 = (uint32_t)clock();
        }
        const int phase = node_phase(s.entry, P.leaf_wait) ? 1 : 0;
        if (!trav_step<STATS, KINDS>(s, stack, sv, &P.sbt, P.status, ray_flags, 0xFFu, sbt_offset, cnt, phase))
            continue;
        // the ray is finished
        if (MODE == kModeBounce) {
            if (s.hit_inst != kNoHit && (depth & 0xFFu) + 1 < P.B.scenes[s.scene].max_depth) {
                const NextRay nr =
                    next_bounce_ray(P.B.scenes[s.scene].env, &P.sbt, s.hit_inst, s.hit_geom, s.hit_prim, s.t, s.u,
                                    s.v, s.wo, s.wd);
                if (nr.d.x != 0.0f || nr.d.y != 0.0f || nr.d.z != 0.0f) {
                    trav_begin(s, sv(s.scene), nr.o, nr.d, 0.01f, 10000.0f);
                    depth++;
                    atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->traversals), 1ull);
                    atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->secondary_rays), 1ull);
                    continue;
                }
            }
            P.B.hits[2 * (size_t)item] = make_uint4(__float_as_uint(s.t), __float_as_uint(s.u), __float_as_uint(s.v),
                                                    s.hit_inst);
            P.B.hits[2 * (size_t)item + 1] = make_uint4(s.hit_geom, s.hit_prim, s.front ? 1u : 0u, 0u);
            if ((depth & 0xFFu) != (depth >> 8)) {  // the slot's ray, for the shading kernel, is the last one traced
                P.B.rays[b & 1][2 * (size_t)item] = make_float4(s.wo.x, s.wo.y, s.wo.z, 0.01f);
                P.B.rays[b & 1][2 * (size_t)item + 1] = make_float4(s.wd.x, s.wd.y, s.wd.z, 10000.0f);
                P.B.ray_scene[b & 1][item] = s.scene | ((depth & 0xFFu) << kSceneBits);
            }
        } else if (s.hit_inst == kNoHit) {
            atomicAdd(&P.B.lit[P.B.shadow_pixel[item]], 1u);  // shadow_ray_miss clears `shadowed`
        }
        if (heat) {
            const uint32_t pix = MODE == kModeBounce ? P.B.ray_pixel[b & 1][item] : P.B.shadow_pixel[item];
            atomicAdd(&P.B.heat[pix], (unsigned long long)((uint32_t)clock() - t0));
        }
        item = kNoItem;
    }
    flush_counters(P.stats, cnt);
}

// One traversal kernel per BLAS node-format set KINDS, each with its own
// register allocation (one kernel holding all three loops spills far more).
// The host launches the variant for the formats this process has built; when
// it has built both, it launches all three and each runs only if the
// scenes' TLAS headers name exactly its set.
__device__ __forceinline__ bool kinds_selected(uint32_t kinds_built, uint32_t tlas_kinds, uint32_t kinds) {
    if (kinds_built != (kBlasKindF32 | kBlasKindQ8)) return true;  // the only launch
    return (tlas_kinds ? tlas_kinds : kBlasKindF32) == kinds;
}

template <int MODE, bool STATS, uint32_t KINDS, int SD, int BLOCK>
__global__ void __launch_bounds__(BLOCK, trace_warps_per_sm(KINDS) * 32 / BLOCK)
    k_trace(const __grid_constant__ WfParams P) {
    if (kinds_selected(P.kinds_built, P.B.ctr->kinds, KINDS)) trace_wavefront<MODE, STATS, KINDS, SD, BLOCK>(P);
}

// ---------------------------------------------------------------------------
// Packet traversal of the wavefront lists.  Neighbouring entries of a list
// are neighbouring rays: the primary list holds the 32 rays of one 8x4 pixel
// tile per warp-sized chunk, and a shading warp appends the shadow rays of
// its pixels contiguously.  A warp takes a chunk of 32 entries and walks one
// node sequence for its rays of one scene (a sub-packet): every lane tests
// the node's eight children against its own ray, each child's key is reduced
// to its minimum over the lanes (REDUX), and the union of the hit children,
// ordered by those keys, goes on one stack per warp in shared memory.
// Leaves and instance entries run once for the sub-packet, each lane testing
// its own ray.  A lane tests every triangle of every box its ray hits (and
// some more), so the closest hit under the total order is the per-lane
// traversal's, bit for bit; every lane runs the same steps, so the SIMD
// lanes stay full while the rays agree.
// ---------------------------------------------------------------------------

// Traverses the sub-packet `act` (the calling lanes, converged, one scene,
// each at the TLAS root).  ws: the warp's stack (kStackSize entries).
template <bool STATS, uint32_t KINDS>
__device__ __forceinline__ void packet_traverse(Trav& s, uint2* ws, float4* nb, const unsigned act,
                                                const SceneTable& sv, const RtShaderBindingTable* sbt,
                                                uint32_t* status, uint32_t ray_flags, uint32_t ray_sbt_offset,
                                                Counters& cnt) {
    const bool any_hit = (ray_flags & RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT) != 0u;
    const bool leader = (threadIdx.x & 31u) == (uint32_t)(__ffs(act) - 1);
    bool done = false;  // any-hit rays: an accepted hit ends the lane's part
    uint32_t entry = s.entry;
    int sp = 0;
    uint32_t steps = 0;
    while (entry != kNoEntry) {
        if (++steps > kMaxTraversalSteps) {
            if (leader) atomicOr(status, 1u << RT_ERR_TIMEOUT);
            break;
        }
        bool pop = true;
        if (entry == kMarker) {
            trav_restore_world(s, sv(s.scene));
        } else if ((entry & kLeafEntry) == 0u) {
            if (entry >= s.node_count) {
                if (leader) atomicOr(status, 1u << RT_ERR_BAD_AS);
            } else {
                if (STATS) cnt.nodes++;
                uint32_t keys[8], refs[8];
                const bool qn = (KINDS & kBlasKindQ8) && s.in_blas && (KINDS == kBlasKindQ8 || s.quant);
                if (RT_PACKET_STAGE) {
                    // the sub-packet's lanes copy the node into the warp's buffer with one
                    // 16-byte load each, then every lane reads its planes from there
                    const float4* src = qn ? reinterpret_cast<const float4*>(reinterpret_cast<const uint8_t*>(s.nodes) +
                                                                             (size_t)entry * kQNodeBytes)
                                           : reinterpret_cast<const float4*>(s.nodes + entry);
                    const uint32_t n16 = qn ? kQNodeBytes / 16u : kNodeBytes / 16u;
                    const uint32_t r = (uint32_t)__popc(act & lanemask_lt()), na = (uint32_t)__popc(act);
                    __syncwarp(act);  // every lane has read the previous node
                    for (uint32_t q = r; q < n16; q += na) nb[q] = __ldg(src + q);
                    __syncwarp(act);
                    if (qn) {
                        if (STATS) cnt.qnodes++;
                        qnode_keys_at<false>(s, reinterpret_cast<const uint8_t*>(nb), keys, refs);
                    } else {
                        fnode_keys_at<false>(s, nb, keys, refs);
                    }
                } else if (qn) {
                    if (STATS) cnt.qnodes++;
                    qnode_keys(s, entry, keys, refs);
                } else {
                    fnode_keys(s, entry, keys, refs);
                }
                // the nearest lane's key of each child; every lane has read its
                // last popped entry before this point, so the pushes below
                // cannot overwrite an entry a lane has yet to read
#pragma unroll
                for (int k = 0; k < 8; k++) keys[k] = __reduce_min_sync(act, done ? 0xFFFFFFFFu : keys[k]);
                if (any_hit) {
                    uint32_t mask = 0;
#pragma unroll
                    for (int k = 0; k < 8; k++) mask |= (keys[k] != 0xFFFFFFFFu ? 1u : 0u) << k;
                    if (mask) {
                        entry = pick8(refs, (uint32_t)(__ffs(mask) - 1));
                        mask &= mask - 1u;
                        while (mask) {
                            const uint32_t k = (uint32_t)(__ffs(mask) - 1);
                            mask &= mask - 1u;
                            if (sp < (int)kStackSize) ws[sp++] = make_uint2(pick8(refs, k), 0u);
                            else if (leader) atomicOr(status, 1u << RT_ERR_STACK_OVERFLOW);
                        }
                        pop = false;
                    }
                } else {
                    sort8(keys);
                    if (keys[0] != 0xFFFFFFFFu) {
#pragma unroll
                        for (int q = 7; q >= 1; q--) {
                            const uint32_t key = keys[q];
                            if (key == 0xFFFFFFFFu) continue;
                            if (sp < (int)kStackSize) ws[sp++] = make_uint2(pick8(refs, key & 7u), key & ~7u);
                            else if (leader) atomicOr(status, 1u << RT_ERR_STACK_OVERFLOW);
                        }
                        entry = pick8(refs, keys[0] & 7u);
                        pop = false;
                    }
                }
            }
        } else {
            const uint32_t first = entry & 0x0FFFFFFFu;
            const uint32_t count = ((entry >> 28) & 7u) + 1u;
            if (first + count > (s.in_blas ? s.tri_count : sv(s.scene).inst_count)) {
                if (leader) atomicOr(status, 1u << RT_ERR_BAD_AS);
            } else if (!s.in_blas) {
                const InstRecord* ir = &sv(s.scene).insts[first];
                const uint4* tail = reinterpret_cast<const uint4*>(&ir->blas);
                const uint4 q0 = __ldg(tail), q1 = __ldg(tail + 1);
                bool enter = q1.y != 0u && (q0.w >> 24) != 0u;  // cull mask 0xFF
                if (enter && (blas_kind(q1.z) & KINDS) == 0u) {
                    if (leader) atomicOr(status, 1u << RT_ERR_BAD_AS);
                    enter = false;
                }
                if (enter) {
                    if (sp < (int)kStackSize) {
                        if (STATS) cnt.insts++;
                        enter_instance(s, ir, q0, q1, first);
                        __syncwarp(act);  // every lane has read the entry this push replaces
                        ws[sp++] = make_uint2(kMarker, 0u);
                        entry = 0;  // BLAS root
                        pop = false;
                    } else if (leader) {
                        atomicOr(status, 1u << RT_ERR_STACK_OVERFLOW);
                    }
                }
            } else {
                if (!done) {
                    for (uint32_t q = 0; q < count; q++) {
                        if (try_triangle<STATS>(s, sv, sbt, ray_flags, ray_sbt_offset, first + q, cnt) && any_hit) {
                            done = true;
                            break;
                        }
                    }
                }
                if (any_hit && __all_sync(act, done)) break;
            }
        }
        if (pop) {
            // the next entry some lane still needs (markers always)
            entry = kNoEntry;
            const float cull = s.t * kBoxFarScale;
            while (sp > 0) {
                const uint2 en = ws[--sp];
                if (en.x == kMarker) {
                    entry = kMarker;
                    break;
                }
                if (__any_sync(act, !done && !(__uint_as_float(en.y) > cull))) {
                    entry = en.x;
                    break;
                }
            }
        }
    }
}

// LANE_BOUNCES: mirror / portal continuations traced one per lane inside the
// launch (RT_TRAVERSAL_PACKET_LANE_BOUNCES), else as further sub-packets.
template <int MODE, bool STATS, uint32_t KINDS, int BLOCK, bool LANE_BOUNCES>
__device__ __forceinline__ void trace_packets(const WfParams& P) {
    __shared__ uint2 stacks[BLOCK / 32][kStackSize];
    __shared__ float4 nbuf[BLOCK / 32][RT_PACKET_STAGE ? kNodeBytes / 16 : 1];  // staged node per warp
    uint2* ws = stacks[threadIdx.x >> 5];
    const SceneTable sv{P.B.scenes};
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t b = P.bounce;
    uint32_t total;
    uint32_t* work;
    if (MODE == kModeBounce) {
        total = P.B.ctr->ray_count[b];
        work = &P.B.ctr->work[b];
    } else {
        total = P.B.ctr->shadow_count;
        work = &P.B.ctr->work[kMaxDepth + 1];
    }
    const uint32_t ray_flags = MODE == kModeShadow
                                   ? (RT_RAY_FLAG_TERMINATE_ON_FIRST_HIT | RT_RAY_FLAG_SKIP_CLOSEST_HIT_SHADER)
                                   : RT_RAY_FLAG_NONE;
    const uint32_t sbt_offset = MODE == kModeShadow ? 1u : 0u;
    Counters cnt = {0, 0, 0, 0};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= total) break;
        const uint32_t item = base + lane;
        const bool valid = item < total;
        Trav s;
        s.scene = 0;
        s.entry = kNoEntry;
        uint32_t depth = 0, depth0 = 0, pix = kNoPixel;  // depth of the ray traced / of the slot's ray
        if (valid) {
            uint32_t sc;
            if (MODE == kModeBounce) {
                const float4 a = P.B.rays[b & 1][2 * (size_t)item], c = P.B.rays[b & 1][2 * (size_t)item + 1];
                pix = P.B.ray_pixel[b & 1][item];
                const uint32_t rs = P.B.ray_scene[b & 1][item];
                sc = rs & kSceneMask;
                depth = depth0 = rs >> kSceneBits;
                trav_begin(s, sv(sc), mk3(a.x, a.y, a.z), mk3(c.x, c.y, c.z), a.w, c.w);
            } else {
                const float4 a = P.B.shadow_rays[2 * (size_t)item], c = P.B.shadow_rays[2 * (size_t)item + 1];
                pix = P.B.shadow_pixel[item];
                sc = P.B.shadow_scene[item];
                trav_begin(s, sv(sc), mk3(a.x, a.y, a.z), mk3(c.x, c.y, c.z), a.w, c.w);
            }
            s.scene = sc;
        }
        const bool heat = pix != kNoPixel && P.B.scenes[s.scene].uniforms->show_heatmap != 0;
        const uint32_t t0 = heat ? (uint32_t)clock() : 0u;
        unsigned pending = __ballot_sync(0xFFFFFFFFu, s.entry != kNoEntry);
        while (pending) {
            const uint32_t lead = (uint32_t)(__ffs(pending) - 1);
            const uint32_t sc = __shfl_sync(0xFFFFFFFFu, s.scene, lead);
            const unsigned act = __ballot_sync(0xFFFFFFFFu, ((pending >> lane) & 1u) != 0u && s.scene == sc);
            pending &= ~act;
            bool cont = false;
            if ((act >> lane) & 1u) {
                packet_traverse<STATS, KINDS>(s, ws, nbuf[threadIdx.x >> 5], act, sv, &P.sbt, P.status, ray_flags,
                                              sbt_offset, cnt);
                if (MODE == kModeBounce && LANE_BOUNCES) {
                    // every further bounce of the lane's ray, traced by the lane
                    // alone (the closest-hit program's arithmetic, bit for bit)
                    TravStack<0, BLOCK> stk;
                    while (s.hit_inst != kNoHit && depth + 1 < P.B.scenes[s.scene].max_depth) {
                        const NextRay nr = next_bounce_ray(P.B.scenes[s.scene].env, &P.sbt, s.hit_inst, s.hit_geom,
                                                           s.hit_prim, s.t, s.u, s.v, s.wo, s.wd);
                        if (nr.d.x == 0.0f && nr.d.y == 0.0f && nr.d.z == 0.0f) break;
                        trav_begin(s, sv(s.scene), nr.o, nr.d, 0.01f, 10000.0f);
                        depth++;
                        atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->traversals), 1ull);
                        atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->secondary_rays), 1ull);
                        while (!trav_step<STATS, KINDS>(s, stk, sv, &P.sbt, P.status, ray_flags, 0xFFu, sbt_offset,
                                                        cnt, -1)) {
                        }
                    }
                } else if (MODE == kModeBounce && s.hit_inst != kNoHit &&
                           depth + 1 < P.B.scenes[s.scene].max_depth) {
                    // a mirror / portal hit with depth left: the lane's next ray
                    // joins the chunk's next sub-packet
                    const NextRay nr = next_bounce_ray(P.B.scenes[s.scene].env, &P.sbt, s.hit_inst, s.hit_geom,
                                                       s.hit_prim, s.t, s.u, s.v, s.wo, s.wd);
                    if (nr.d.x != 0.0f || nr.d.y != 0.0f || nr.d.z != 0.0f) {
                        trav_begin(s, sv(s.scene), nr.o, nr.d, 0.01f, 10000.0f);
                        depth++;
                        atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->traversals), 1ull);
                        atomicAdd(reinterpret_cast<unsigned long long*>(&P.stats->secondary_rays), 1ull);
                        cont = s.entry != kNoEntry;
                    }
                }
            }
            __syncwarp();
            pending |= __ballot_sync(0xFFFFFFFFu, cont);
        }
        if (valid) {
            if (MODE == kModeBounce) {
                P.B.hits[2 * (size_t)item] = make_uint4(__float_as_uint(s.t), __float_as_uint(s.u),
                                                        __float_as_uint(s.v), s.hit_inst);
                P.B.hits[2 * (size_t)item + 1] = make_uint4(s.hit_geom, s.hit_prim, s.front ? 1u : 0u, 0u);
                if (depth != depth0) {  // the slot's ray, for the shading kernel, is the last one traced
                    P.B.rays[b & 1][2 * (size_t)item] = make_float4(s.wo.x, s.wo.y, s.wo.z, 0.01f);
                    P.B.rays[b & 1][2 * (size_t)item + 1] = make_float4(s.wd.x, s.wd.y, s.wd.z, 10000.0f);
                    P.B.ray_scene[b & 1][item] = s.scene | (depth << kSceneBits);
                }
            } else if (s.hit_inst == kNoHit) {
                atomicAdd(&P.B.lit[pix], 1u);
            }
        }
        if (heat) atomicAdd(&P.B.heat[pix], (unsigned long long)((uint32_t)clock() - t0));
    }
    flush_counters(P.stats, cnt);
}

// Packets hold the per-lane keys, the reduced keys and the child references
// at once: the FP32 kernels run at 20 warps per SM (96 registers, 68-byte
// spills instead of 288 at 80 registers; 1080p frame +0.8 %, 16 warps -1 %).
// A 256-thread block cannot make 20 warps and keeps 24.  The quantised-only
// packet kernels run at 32 warps (64 registers): 28, 24 and 20 warps made the
// 64-scene batch's camera-ray launch slower (11.9 -> 12.3 / 12.6 / 12.7 ms).
#ifndef RT_Q8_PACKET_WARPS
#define RT_Q8_PACKET_WARPS 32
#endif
constexpr int packet_warps_per_sm(uint32_t kinds, int block) {
    return kinds == kBlasKindQ8 ? (block == 256 && RT_Q8_PACKET_WARPS < 24 ? 24 : RT_Q8_PACKET_WARPS)
                                : (block == 256 ? 24 : 20);
}

template <int MODE, bool STATS, uint32_t KINDS, int BLOCK, bool LANE_BOUNCES>
__global__ void __launch_bounds__(BLOCK, packet_warps_per_sm(KINDS, BLOCK) * 32 / BLOCK)
    k_trace_packet(const __grid_constant__ WfParams P) {
    if (kinds_selected(P.kinds_built, P.B.ctr->kinds, KINDS))
        trace_packets<MODE, STATS, KINDS, BLOCK, LANE_BOUNCES>(P);
}

// The closest-hit and miss programs for the last ray of every slot of bounce
// list b (its depth is in the slot's scene word).  Mirror and portal hits
// that reach it end their pixel's bounce loop (no depth left, or a zero
// direction): the traversal already followed every other one.  The append
// of a further bounce ray is kept for lists traced without that.  Every lane
// of the (full) warps reaches the appends at the end.
// 8 blocks of 128 per SM (<= 64 registers): the shading is latency-bound on
// dependent loads (instance -> model -> indices -> vertices -> textures);
// 1080p frame 199 -> 170 us against the unconstrained 90 registers.
__global__ void __launch_bounds__(128, 8) k_shade(const __grid_constant__ WfParams P) {
    const uint32_t b = P.bounce;
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t p = kNoPixel, sc = 0, depth = 0, nshadow = 0;
    bool emit_ray = false, write_colour = false;
    V3 col = mk3(0.0f, 0.0f, 0.0f), nd = mk3(0, 0, 0), no = mk3(0, 0, 0);
    if (i < P.B.ctr->ray_count[b]) p = P.B.ray_pixel[b & 1][i];
    if (p != kNoPixel) {
        const uint32_t rs = P.B.ray_scene[b & 1][i];
        sc = rs & kSceneMask;
        depth = rs >> kSceneBits;
        const SceneRec& S = P.B.scenes[sc];
        const Env& e = S.env;
        const RtUniforms& U = *S.uniforms;
        const V3 sun_dir = mk3(U.sun_dir[0], U.sun_dir[1], U.sun_dir[2]);
        float4 ra = P.B.rays[b & 1][2 * (size_t)i], rb = P.B.rays[b & 1][2 * (size_t)i + 1];
        V3 ro = mk3(ra.x, ra.y, ra.z), rd = mk3(rb.x, rb.y, rb.z);
        uint4 h0 = P.B.hits[2 * (size_t)i], h1 = P.B.hits[2 * (size_t)i + 1];
        const float t = __uint_as_float(h0.x), hu = __uint_as_float(h0.y), hv = __uint_as_float(h0.z);
        const uint32_t inst = h0.w;
        if (inst == kNoHit) {
            // primary_ray_miss (lib.rs:40-51)
            float sun_s, sun_c;
            rt_sincos(U.sun_radius, &sun_s, &sun_c);
            col = dot3(rd, sun_dir) > sun_c ? mk3(1.0f, 1.0f, 1.0f) : mk3(0.0f, 0.0f, 0.05f);
            write_colour = true;
        } else {
            const InstRecord* ir = &e.insts[inst];
            const uint32_t sbt_flags = ir->sbt_flags, custom = ir->custom_mask & 0xFFFFFFu;
            const RtHitGroup* g = hit_group(&P.sbt, sbt_flags, 0u);
            const uint32_t prog = g ? g->closest_hit : RT_PROGRAM_NONE;
            const V3 bary = mk3((1.0f - hu) - hv, hu, hv);
            TriData td;
            if (prog == RT_PROGRAM_CLOSEST_HIT_MIRROR || prog == RT_PROGRAM_CLOSEST_HIT_PORTAL) {
                const NextRay nr = next_bounce_ray(e, &P.sbt, inst, h1.x, h1.y, t, hu, hv, ro, rd);
                no = nr.o;
                nd = nr.d;
            } else if (prog == RT_PROGRAM_CLOSEST_HIT_TEXTURED && load_triangle(e, custom, h1.x, h1.y, &td)) {
                // closest_hit_textured.glsl:174-226
                V3 ip = interp3(td.p[0], td.p[1], td.p[2], bary);
                V3 inrm = interp3(td.n[0], td.n[1], td.n[2], bary);
                float iu = (td.uv[0][0] * bary.x + td.uv[1][0] * bary.y) + td.uv[2][0] * bary.z;
                float iv = (td.uv[0][1] * bary.x + td.uv[1][1] * bary.y) + td.uv[2][1] * bary.z;
                V3 oa = project_onto_tangent_plane(ip, td.p[0], td.n[0]);
                V3 ob = project_onto_tangent_plane(ip, td.p[1], td.n[1]);
                V3 oc = project_onto_tangent_plane(ip, td.p[2], td.n[2]);
                V3 off = interp3(oa, ob, oc, bary);
                V3 so = xform_point(ir->o2w, add3(ip, off));
                float NoL;
                V3 comb, amb;
                const bool lambert = (S.flags & RT_TRACE_FLAG_LAMBERT_DIFFUSE) != 0;
                shade_textured(e, td, inrm, iu, iv, ir->w2o, rd, sun_dir, lambert, &NoL, &comb, &amb);
                if (S.shadow_count > 0) {
                    float4* sh = P.B.shade + 3 * (size_t)p;
                    sh[0] = make_float4(so.x, so.y, so.z, NoL);
                    sh[1] = make_float4(comb.x, comb.y, comb.z, amb.x);
                    sh[2] = make_float4(amb.y, amb.z, 0.0f, 0.0f);
                    nshadow = S.shadow_count;
                } else {
                    float sf = 0.0f;
                    col = mk3((sf * NoL) * comb.x + amb.x, (sf * NoL) * comb.y + amb.y, (sf * NoL) * comb.z + amb.z);
                    write_colour = true;
                }
            }
            if (nshadow == 0 && !write_colour) {
                // payload: break when new_ray_direction == 0 (lib.rs:165-171),
                // and after the last iteration the colour stays reset (black)
                if ((nd.x == 0.0f && nd.y == 0.0f && nd.z == 0.0f) || depth + 1 >= S.max_depth) {
                    col = mk3(0.0f, 0.0f, 0.0f);
                    write_colour = true;
                } else {
                    emit_ray = true;
                }
            }
        }
    }
    if (write_colour) P.B.colour[p] = make_float4(col.x, col.y, col.z, 1.0f);
    const uint32_t si = warp_append(&P.B.ctr->shade_count, nshadow > 0);
    if (nshadow > 0) P.B.shade_list[si] = p;
    const uint32_t first = warp_append_n(&P.B.ctr->shadow_count, nshadow);
    const uint32_t ri = warp_append(&P.B.ctr->ray_count[b + 1], emit_ray);
    if (nshadow > 0) {
        // the textured hit's shadow rays (closest_hit_textured.glsl:159-172)
        const SceneRec& S = P.B.scenes[sc];
        const RtUniforms& U = *S.uniforms;
        const V3 sun_dir = mk3(U.sun_dir[0], U.sun_dir[1], U.sun_dir[2]);
        const uint32_t lp = p - S.pixel_begin, x = lp % S.width, y = lp / S.width;
        const float4 so = P.B.shade[3 * (size_t)p];
        for (uint32_t k = 0; k < nshadow; k++) {
            const V3 sd = shadow_direction(S.env, U, x, y, k, sun_dir);
            float4* R = P.B.shadow_rays + 2 * (size_t)(first + k);
            R[0] = make_float4(so.x, so.y, so.z, 0.001f);
            R[1] = make_float4(sd.x, sd.y, sd.z, 10000.0f);
            P.B.shadow_pixel[first + k] = p;
            P.B.shadow_scene[first + k] = sc;
        }
    }
    if (emit_ray) {
        float4* R = P.B.rays[(b + 1) & 1];
        R[2 * (size_t)ri] = make_float4(no.x, no.y, no.z, 0.01f);
        R[2 * (size_t)ri + 1] = make_float4(nd.x, nd.y, nd.z, 10000.0f);
        P.B.ray_pixel[(b + 1) & 1][ri] = p;
        P.B.ray_scene[(b + 1) & 1][ri] = sc | ((depth + 1) << kSceneBits);
    }
}

// sun_factor = lit / N; colour = brdf * sun_factor + ambient.
__global__ void k_resolve(const __grid_constant__ WfParams P) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= P.B.ctr->shade_count) return;
    const uint32_t p = P.B.shade_list[k];
    const SceneRec& S = P.B.scenes[scene_of<true>(P, p)];
    const float4* sh = P.B.shade + 3 * (size_t)p;
    float4 s0 = sh[0], s1 = sh[1], s2 = sh[2];
    float sf = (float)P.B.lit[p] / (float)S.shadow_count;
    float NoL = s0.w;
    P.B.colour[p] = make_float4((sf * NoL) * s1.x + s1.w, (sf * NoL) * s1.y + s2.x, (sf * NoL) * s1.z + s2.y, 1.0f);
}

// Heatmap (lib.rs:174-186), linear_to_srgb and the RGBA8 image write.
__global__ void k_output(const __grid_constant__ WfParams P) {
    const uint32_t gp = blockIdx.x * blockDim.x + threadIdx.x;
    if (gp >= P.total_pixels) return;
    if (gp == 0) {  // the shadow and bounce rays the shading launch appended
        uint32_t bounce = 0;
        for (uint32_t d = 1; d <= kMaxDepth; d++) bounce += P.B.ctr->ray_count[d];
        count_list_rays(P.stats, P.B.ctr->shadow_count, bounce);
    }
    const SceneRec& S = P.B.scenes[scene_of<true>(P, gp)];
    const uint32_t p = gp - S.pixel_begin;
    float4 c4 = P.B.colour[gp];
    V3 c = mk3(c4.x, c4.y, c4.z);
    if (S.uniforms->show_heatmap) {
        V3 hm = heatmap_temperature((float)P.B.heat[gp] / 1000000.0f);
        c = add3(hm, mul3s(c, 0.000001f));
    }
    if (S.radiance) S.radiance[p] = make_float4(c.x, c.y, c.z, 1.0f);
    if (S.image) {
        uint32_t r = to_unorm8(linear_to_srgb(c.x)), g = to_unorm8(linear_to_srgb(c.y));
        uint32_t bl = to_unorm8(linear_to_srgb(c.z));
        S.image[p] = r | (g << 8) | (bl << 16) | (255u << 24);
    }
}

struct RayBufferParams {
    RayBufferLaunch L;
};

template <bool STATS, uint32_t KINDS>
__device__ __forceinline__ void trace_ray_buffer(const RayBufferParams& P, const Env& e) {
    const RayBufferLaunch& L = P.L;
    const OneScene sv{e};
    Counters cnt = {0, 0, 0, 0};
    TravStack<0, kTraceThreads> stack;
    Trav s;
    uint32_t item = kNoItem;
    if (blockIdx.x == 0 && threadIdx.x == 0 && L.count) {
        atomicAdd(reinterpret_cast<unsigned long long*>(&L.stats->traversals), (unsigned long long)L.count);
        atomicAdd(reinterpret_cast<unsigned long long*>(&L.stats->primary_rays), (unsigned long long)L.count);
    }
    for (;;) {
        uint32_t my = warp_append(L.work, item == kNoItem);
        if (item == kNoItem) {
            if (my >= L.count) break;
            item = my;
            const float4* rp = reinterpret_cast<const float4*>(L.rays + item);
            float4 a = __ldg(rp), c = __ldg(rp + 1);
            trav_begin(s, e, mk3(a.x, a.y, a.z), mk3(c.x, c.y, c.z), a.w, c.w);
            s.scene = 0;
        }
        const int phase = node_phase(s.entry, RT_TRACE_LEAF_WAIT) ? 1 : 0;
        if (!trav_step<STATS, KINDS>(s, stack, sv, &L.sbt, L.status, L.ray_flags, L.cull_mask, L.sbt_offset, cnt,
                                     phase))
            continue;
        RtHit o;
        if (s.hit_inst != kNoHit) {
            const InstRecord* ir = &e.insts[s.hit_inst];
            o.t = s.t;
            o.u = s.u;
            o.v = s.v;
            o.instance_id = ir->instance_id;
            o.instance_custom_index = ir->custom_mask & 0xFFFFFFu;
            o.geometry_index = s.hit_geom;
            o.primitive_index = s.hit_prim;
            o.hit_kind = s.front ? 0xFEu : 0xFFu;
        } else {
            o.t = s.t;
            o.u = o.v = 0.0f;
            o.instance_id = o.instance_custom_index = o.geometry_index = o.primitive_index = 0xFFFFFFFFu;
            o.hit_kind = 0;
        }
        uint4* hp = reinterpret_cast<uint4*>(L.hits + item);
        const uint4* op = reinterpret_cast<const uint4*>(&o);
        hp[0] = op[0];
        hp[1] = op[1];
        item = kNoItem;
    }
    flush_counters(L.stats, cnt);
}

template <bool STATS, uint32_t KINDS>
__global__ void __launch_bounds__(kTraceThreads, raybuf_warps_per_sm(KINDS) * 32 / kTraceThreads)
    k_trace_ray_buffer(const __grid_constant__ RayBufferParams P) {
    const Env e = make_env(P.L.tlas, P.L.push.model_info, P.L.textures, RT_MAX_BOUND_IMAGES, P.L.status);
    if (kinds_selected(P.L.kinds_built, e.blas_kinds, KINDS)) trace_ray_buffer<STATS, KINDS>(P, e);
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
int persistent_blocks(K kernel, int threads, int num_sms, size_t smem = 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1)
        per_sm = 1;
    return per_sm * num_sms;
}

// Calls f(std::integral_constant<uint32_t, KINDS>) for each traversal
// variant to launch, given the BLAS formats built so far (kinds_selected).
template <class F>
void for_each_variant(uint32_t kinds_built, F&& f) {
    using F32 = std::integral_constant<uint32_t, kBlasKindF32>;
    using Q8 = std::integral_constant<uint32_t, kBlasKindQ8>;
    using Both = std::integral_constant<uint32_t, kBlasKindF32 | kBlasKindQ8>;
    if (kinds_built == (kBlasKindF32 | kBlasKindQ8)) {
        f(F32{});
        f(Q8{});
        f(Both{});
    } else if (kinds_built == kBlasKindQ8) {
        f(Q8{});
    } else {
        f(F32{});
    }
}

template <int MODE, bool STATS, uint32_t KINDS, int SD, int BLOCK>
void launch_trace_kernel(const WfParams& P, int num_sms, cudaStream_t stream) {
    const auto kern = k_trace<MODE, STATS, KINDS, SD, BLOCK>;
    constexpr size_t smem = (size_t)SD * BLOCK * sizeof(uint2);
    static int blocks = 0;
    if (!blocks) {
        if (smem > 48 * 1024) cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        blocks = persistent_blocks(kern, BLOCK, num_sms, smem);
    }
    note_launch(), kern<<<blocks, BLOCK, smem, stream>>>(P);
}

template <int MODE, bool STATS, uint32_t KINDS, int BLOCK, bool LANE_BOUNCES = false>
void launch_packet_kernel(const WfParams& P, int num_sms, cudaStream_t stream) {
    const auto kern = k_trace_packet<MODE, STATS, KINDS, BLOCK, LANE_BOUNCES>;
    static int blocks = 0;
    if (!blocks) blocks = persistent_blocks(kern, BLOCK, num_sms);
    note_launch(), kern<<<blocks, BLOCK, 0, stream>>>(P);
}

// The traversal variants the autotuner chooses among: block size x depth of
// the shared-memory part of the stack (kTraversalConfigs in the same order).
#define RT_FOR_EACH_TRAVERSAL_VARIANT(X) \
    X(64, 0) X(64, 16) X(64, 24) X(64, 32) X(128, 0) X(128, 16) X(128, 24) X(128, 32) \
    X(256, 0) X(256, 16) X(256, 24) X(256, 32)

template <int MODE, uint32_t K>
void launch_trace_config(const WfParams& P, const RtTraversalConfig& c, bool stats, int num_sms,
                         cudaStream_t stream) {
    if (stats) {  // statistics runs use the default per-lane variant: work counted per ray
        launch_trace_kernel<MODE, true, K, 0, kTraceThreads>(P, num_sms, stream);
        return;
    }
    if (c.packet_lists & (MODE == kModeBounce ? RT_TRAVERSAL_PACKET_PRIMARY : RT_TRAVERSAL_PACKET_SHADOW)) {
        if constexpr (MODE == kModeBounce) {
            if (c.packet_lists & RT_TRAVERSAL_PACKET_LANE_BOUNCES) {
                if (c.block_size == 64) launch_packet_kernel<MODE, false, K, 64, true>(P, num_sms, stream);
                else if (c.block_size == 256) launch_packet_kernel<MODE, false, K, 256, true>(P, num_sms, stream);
                else launch_packet_kernel<MODE, false, K, 128, true>(P, num_sms, stream);
                return;
            }
        }
        if (c.block_size == 64) {
            launch_packet_kernel<MODE, false, K, 64>(P, num_sms, stream);
        } else if (c.block_size == 256) {
            launch_packet_kernel<MODE, false, K, 256>(P, num_sms, stream);
        } else {
            launch_packet_kernel<MODE, false, K, 128>(P, num_sms, stream);
        }
        return;
    }
#define RT_TRACE_CASE(B, D)                                                  \
    if (c.block_size == B && c.shared_stack_depth == D) {                   \
        launch_trace_kernel<MODE, false, K, D, B>(P, num_sms, stream);     \
        return;                                                             \
    }
    RT_FOR_EACH_TRAVERSAL_VARIANT(RT_TRACE_CASE)
#undef RT_TRACE_CASE
    launch_trace_kernel<MODE, false, K, 0, kTraceThreads>(P, num_sms, stream);
}

template <int MODE>
void launch_trace_mode(const WfParams& P, const RtTraversalConfig& c, bool stats, int num_sms, cudaStream_t stream) {
    for_each_variant(P.kinds_built, [&](auto k) {
        constexpr uint32_t K = decltype(k)::value;
        launch_trace_config<MODE, K>(P, c, stats, num_sms, stream);
    });
}

template <bool STATS, uint32_t KINDS>
void launch_ray_buffer_kernel(const RayBufferParams& P, int num_sms, cudaStream_t stream) {
    static int blocks = 0;
    if (!blocks) blocks = persistent_blocks(k_trace_ray_buffer<STATS, KINDS>, kTraceThreads, num_sms);
    note_launch(), k_trace_ray_buffer<STATS, KINDS><<<blocks, kTraceThreads, 0, stream>>>(P);
}

}  // namespace

namespace {

// Host-side layout of a batch: tiles and pixels concatenated scene by scene,
// and the workspace regions.
struct BatchLayout {
    std::vector<SceneLayout> lay;
    uint64_t slots = 0, pixels = 0, shadow_rays = 0;
    uint32_t max_depth = 0;
    bool any_shadow = false;
    uint64_t off_ctr, off_scenes, off_tex, off_rays0, off_rays1, off_pix0, off_pix1, off_sc0, off_sc1, off_hits,
        off_colour, off_shade, off_lit, off_shade_list, off_shadow_rays, off_shadow_pix, off_shadow_scene, off_heat,
        total;

    explicit BatchLayout(const TraceScene* sc, uint32_t n) : lay(n) {
        for (uint32_t i = 0; i < n; i++) {
            const uint32_t W = sc[i].desc.width, H = sc[i].desc.height;
            const uint32_t tx = (W + 7) / 8, ty = (H + 3) / 4;
            lay[i] = {tx, (uint32_t)(slots / 32), (uint32_t)pixels};
            slots += (uint64_t)tx * ty * 32;
            pixels += (uint64_t)W * H;
            shadow_rays += (uint64_t)W * H * sc[i].desc.shadow_ray_count;
            max_depth = std::max(max_depth, sc[i].desc.max_trace_depth);
            any_shadow = any_shadow || sc[i].desc.shadow_ray_count > 0;
        }
        place(n);
    }
    // A layout for batch totals alone (no per-scene records): the workspace
    // of any batch of at most n scenes, `slots` ray slots (pixels padded to
    // 8x4 tiles), `pixels` pixels and `shadow` shadow rays fits in it.
    BatchLayout(uint32_t n, uint64_t slots_, uint64_t pixels_, uint64_t shadow) {
        slots = slots_;
        pixels = pixels_;
        shadow_rays = shadow;
        place(n);
    }
    void place(uint32_t n) {
        uint64_t b = 0;
        auto take = [&](uint64_t bytes) {
            uint64_t r = b;
            b = align_up(b + bytes, 256);
            return r;
        };
        off_ctr = take(sizeof(WfCounters));
        off_scenes = take((uint64_t)n * sizeof(SceneRec));
        off_tex = take(RT_MAX_BOUND_IMAGES * sizeof(RtTextureDesc));
        off_rays0 = take(slots * 32);
        off_rays1 = take(slots * 32);
        off_pix0 = take(slots * 4);
        off_pix1 = take(slots * 4);
        off_sc0 = take(slots * 4);
        off_sc1 = take(slots * 4);
        off_hits = take(slots * 32);
        off_colour = take(pixels * 16);
        off_shade = take(pixels * 48);
        off_lit = take(pixels * 4);
        off_shade_list = take(pixels * 4);
        off_shadow_rays = take(shadow_rays * 32);
        off_shadow_pix = take(shadow_rays * 4);
        off_shadow_scene = take(shadow_rays * 4);
        off_heat = take(pixels * 8);
        total = b;
    }
};

}  // namespace

bool traversal_config_supported(const RtTraversalConfig& c) {
    if (c.leaf_wait > 32) return false;
    if (c.packet_lists &
        ~(RT_TRAVERSAL_PACKET_PRIMARY | RT_TRAVERSAL_PACKET_SHADOW | RT_TRAVERSAL_PACKET_LANE_BOUNCES))
        return false;
#define RT_TRACE_SUPPORTED(B, D) \
    if (c.block_size == B && c.shared_stack_depth == D) return true;
    RT_FOR_EACH_TRAVERSAL_VARIANT(RT_TRACE_SUPPORTED)
#undef RT_TRACE_SUPPORTED
    return false;
}

uint64_t trace_workspace_bytes(const TraceScene* scenes, uint32_t count) {
    return BatchLayout(scenes, count).total;
}

uint64_t trace_workspace_bound(uint32_t count, uint64_t slots, uint64_t pixels, uint64_t shadow_rays) {
    return BatchLayout(count, slots, pixels, shadow_rays).total;
}

cudaError_t launch_trace_batch(const TraceBatch& tb, uint8_t* ws, int num_sms, cudaStream_t stream,
                               KernelTimer* timer) {
    auto mark = [&](uint8_t kind) {
        if (timer && timer->n < KernelTimer::kMax) {
            timer->kind[timer->n] = kind;
            cudaEventRecord(timer->ev[timer->n++], stream);
        }
    };
    if (timer) timer->n = 0;
    mark(kKernStart);
    const BatchLayout L(tb.scenes, tb.count);
    WfParams P;
    P.B.ctr = reinterpret_cast<WfCounters*>(ws + L.off_ctr);
    P.B.scenes = reinterpret_cast<SceneRec*>(ws + L.off_scenes);
    P.B.ctx_textures = reinterpret_cast<RtTextureDesc*>(ws + L.off_tex);
    P.B.rays[0] = reinterpret_cast<float4*>(ws + L.off_rays0);
    P.B.rays[1] = reinterpret_cast<float4*>(ws + L.off_rays1);
    P.B.ray_pixel[0] = reinterpret_cast<uint32_t*>(ws + L.off_pix0);
    P.B.ray_pixel[1] = reinterpret_cast<uint32_t*>(ws + L.off_pix1);
    P.B.ray_scene[0] = reinterpret_cast<uint32_t*>(ws + L.off_sc0);
    P.B.ray_scene[1] = reinterpret_cast<uint32_t*>(ws + L.off_sc1);
    P.B.hits = reinterpret_cast<uint4*>(ws + L.off_hits);
    P.B.colour = reinterpret_cast<float4*>(ws + L.off_colour);
    P.B.shade = reinterpret_cast<float4*>(ws + L.off_shade);
    P.B.lit = reinterpret_cast<uint32_t*>(ws + L.off_lit);
    P.B.shade_list = reinterpret_cast<uint32_t*>(ws + L.off_shade_list);
    P.B.shadow_rays = reinterpret_cast<float4*>(ws + L.off_shadow_rays);
    P.B.shadow_pixel = reinterpret_cast<uint32_t*>(ws + L.off_shadow_pix);
    P.B.shadow_scene = reinterpret_cast<uint32_t*>(ws + L.off_shadow_scene);
    P.B.heat = reinterpret_cast<unsigned long long*>(ws + L.off_heat);
    P.sbt = tb.sbt;
    P.stats = tb.stats_dev;
    P.status = tb.status;
    P.scene_count = tb.count;
    P.total_slots = (uint32_t)L.slots;
    P.total_pixels = (uint32_t)L.pixels;
    P.bounce = 0;
    P.kinds_built = tb.kinds_built;
    P.leaf_wait = tb.config.leaf_wait;
    cudaError_t err = cudaMemsetAsync(P.B.ctr, 0, sizeof(WfCounters), stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(P.B.lit, 0, L.pixels * 4, stream);
    if (err == cudaSuccess) err = cudaMemsetAsync(P.B.heat, 0, L.pixels * 8, stream);
    if (err != cudaSuccess) return err;
    // scene records, kSetupChunk scenes per launch (their descriptions travel as kernel parameters)
    static SetupParams sp;  // 10 KB: kept off the stack; launches copy it
    static std::mutex sp_mu;
    {
        std::lock_guard<std::mutex> lk(sp_mu);
        for (uint32_t first = 0; first < tb.count; first += kSetupChunk) {
            const uint32_t n = std::min(kSetupChunk, tb.count - first);
            for (uint32_t i = 0; i < n; i++) {
                sp.d[i] = tb.scenes[first + i];
                sp.lay[i] = L.lay[first + i];
            }
            sp.copy_textures = first == 0;
            if (first == 0) memcpy(sp.textures, tb.ctx_textures, sizeof sp.textures);
            sp.B = P.B;
            sp.stats = P.stats;
            sp.status = tb.status;
            sp.first = first;
            sp.count = n;
            note_launch(), k_setup<<<1, 128, 0, stream>>>(sp);
        }
    }
    const bool stats = tb.stats != 0;
    note_launch(), k_raygen<<<(uint32_t)((L.slots + 255) / 256), 256, 0, stream>>>(P);
    mark(kKernOther);
    // the traversal follows every mirror / portal bounce itself, so one closest-hit launch and one
    // shading launch cover all bounces
    P.bounce = 0;
    launch_trace_mode<kModeBounce>(P, tb.config, stats, num_sms, stream);
    mark(kKernClosest);
    note_launch(), k_shade<<<(uint32_t)((L.slots + 127) / 128), 128, 0, stream>>>(P);
    mark(kKernShade);
    if (L.any_shadow) {
        launch_trace_mode<kModeShadow>(P, tb.config, stats, num_sms, stream);
        mark(kKernShadow);
        note_launch(), k_resolve<<<(uint32_t)((L.pixels + 255) / 256), 256, 0, stream>>>(P);
        mark(kKernOther);
    }
    note_launch(), k_output<<<(uint32_t)((L.pixels + 255) / 256), 256, 0, stream>>>(P);
    mark(kKernOther);
    return cudaGetLastError();
}

cudaError_t launch_trace_ray_buffer(const RayBufferLaunch& p, int num_sms, cudaStream_t stream) {
    RayBufferParams P;
    P.L = p;
    if (p.count == 0) return cudaSuccess;
    cudaError_t err = cudaMemsetAsync(p.work, 0, sizeof(uint32_t), stream);
    if (err != cudaSuccess) return err;
    for_each_variant(p.kinds_built, [&](auto k) {
        constexpr uint32_t K = decltype(k)::value;
        if (p.collect_stats) launch_ray_buffer_kernel<true, K>(P, num_sms, stream);
        else launch_ray_buffer_kernel<false, K>(P, num_sms, stream);
    });
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
