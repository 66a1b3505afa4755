// rt_build.cu — BLAS / TLAS construction, TLAS refit and AS copies.
//
// Build = a binary hierarchy over Morton-ordered primitives, collapsed to
// 8-wide nodes:
//   1. primitive boxes (triangles, or instance world boxes) + centroid bounds
//   2. 30-bit Morton codes of the centroids
//   3. stable LSD radix sort, 8-bit digits, 4 passes: one block for up to
//      kSortTile keys, else onesweep (one upfront histogram of all digits,
//      then one kernel per digit with decoupled look-back across partitions)
//   4. the binary hierarchy: PLOC clustering (RT_BUILD_PREFER_FAST_TRACE;
//      boxes and subtree sizes come with each merge), or the Karras LBVH
//      (index-augmented for ties) with bottom-up boxes from one arrival
//      counter per internal node
//   5. collapse to 8-wide nodes: a node takes its binary children and
//      repeatedly opens the child of largest surface area until it has 8
//      children or none can open; a subtree of <= leaf_max primitives is a
//      leaf.  Each task carries the first position of its primitives in the
//      final order; its children's primitives follow each other in slot
//      order, and a leaf child writes its primitives' positions (perm).
//      Levels run breadth-first, one launch each: a task is stashed in its
//      own (not yet written) wide-node slot, and the nodes one launch
//      allocates are the next launch's tasks.  The levels past the launched
//      ones run as one depth-first task per thread.
//   6. primitive records written in that final order.
// Everything runs on the caller's stream; no host synchronisation.
//
// Replaces vkCmdBuildAccelerationStructuresKHR as called by
// AccelerationStructure::build_blas / new (src/util_structs.rs:140-283),
// build_tlas (src/util_functions.rs:453-510) and update_tlas
// (src/util_structs.rs:285-357), and vkCmdCopyAccelerationStructureKHR CLONE
// (src/util_structs.rs:359-405).
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "rt_internal.h"

namespace rt {

namespace {

constexpr uint32_t kNone = 0xFFFFFFFFu;
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kMinLevels = 6;   // wide levels built breadth-first (more for large n: collapse_levels)
constexpr int kMaxLevels = 24;
constexpr uint32_t kCollapseBlocks = 2432;  // 152 SMs x 16 blocks of 128 threads
constexpr int kTailStack = 192;
constexpr int kSortThreads = 256;
constexpr int kDopThreads = 128;
constexpr int kDopTriples = 14 * 13 * 12 / 6;  // 364 plane triples of the 14-DOP
constexpr int kDopBlocks = (kDopTriples + kDopThreads - 1) / kDopThreads;
constexpr int kDopPer = (kDopTriples + kDopThreads - 1) / kDopThreads;  // triples per thread when merging
constexpr int kSortItems = 8;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;

struct BuildState {
    uint32_t cb[6];   // centroid bounds, ordered-uint encoding: min xyz, max xyz
    uint32_t bb[6];   // primitive box bounds
    uint32_t node_counter;
    uint32_t level_lo, level_hi;  // wide-node slots holding the current collapse level's tasks
    uint32_t level_blocks_done;   // blocks of the current collapse launch that have finished
    uint32_t error;
    uint32_t depth;
    uint32_t blas_kinds;  // TLAS: kBlasKind* bits of the BLASes its instances enter
    uint32_t ploc_count[2];  // PLOC clusters entering the round (double-buffered by round parity)
    uint32_t merge_counter;  // PLOC merges so far (internal node ids count down from n - 2)
    uint32_t ploc_blocks_done;  // blocks of the current merge launch that have finished
    uint32_t radius_bits;    // BLAS: largest vertex distance from the bounds centre (float bits, rounded up)
    uint32_t dop_hi[7], dop_lo[7];  // BLAS: largest / smallest vertex projection on each 14-DOP axis (ordered uint)
    uint32_t dop_blocks_done;       // blocks of k_dop_vertices that have finished
    uint32_t dop_state[kDopTriples];  // 1: the triple's planes meet in a point of the 14-DOP
    double dop_cand[kDopTriples][3];  // that point
};

// The seven 14-DOP axes (unnormalised): x, y, z and the four diagonals.
__device__ __constant__ const int8_t kDopAxis[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 1},
                                                       {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}};

__device__ __forceinline__ uint32_t f2o(float f) {
    uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(uint32_t u) {
    return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// Centre of the primitive bounds, computed the same way wherever it is used.
__device__ __forceinline__ float bounds_center(const BuildState* st, int k) {
    return 0.5f * (o2f(st->bb[k]) + o2f(st->bb[3 + k]));
}

// Distance of v from c, rounded up (every operation rounds towards +inf).
__device__ __forceinline__ float distance_ru(const float v[3], const float c[3]) {
    float s = 0.0f;
    for (int k = 0; k < 3; k++) {
        float d = fmaxf(__fsub_ru(v[k], c[k]), __fsub_ru(c[k], v[k]));
        s = __fadd_ru(s, __fmul_ru(d, d));
    }
    return __fsqrt_ru(s);
}

__device__ __forceinline__ void pad_box(float lo[3], float hi[3]) {
    for (int k = 0; k < 3; k++) {
        float m = fmaxf(fabsf(lo[k]), fabsf(hi[k]));
        float pad = m * 9.5367431640625e-07f + 1e-30f;  // 2^-20 relative
        lo[k] -= pad;
        hi[k] += pad;
    }
}

__device__ __forceinline__ bool finite3(const float v[3]) {
    return fabsf(v[0]) <= FLT_MAX && fabsf(v[1]) <= FLT_MAX && fabsf(v[2]) <= FLT_MAX;
}

// Block-wide min/max reduction of 12 ordered-uint values, then atomics.
__device__ void reduce_bounds(BuildState* st, const float cmin[3], const float cmax[3], const float bmin[3],
                              const float bmax[3]) {
    uint32_t v[12];
    for (int k = 0; k < 3; k++) {
        v[k] = f2o(cmin[k]);
        v[3 + k] = f2o(cmax[k]);
        v[6 + k] = f2o(bmin[k]);
        v[9 + k] = f2o(bmax[k]);
    }
    for (int off = 16; off > 0; off >>= 1) {
        for (int k = 0; k < 12; k++) {
            uint32_t o = __shfl_xor_sync(0xFFFFFFFFu, v[k], off);
            bool is_min = (k < 3) || (k >= 6 && k < 9);
            v[k] = is_min ? min(v[k], o) : max(v[k], o);
        }
    }
    // then over the block's warps, so that each block makes one atomic per
    // bound (one per warp serialised ~82k same-address atomics per bound on a
    // 2.6M-triangle build); every thread of the block must call this
    __shared__ uint32_t s[32][12];
    const uint32_t w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 12; k++) s[w][k] = v[k];
    __syncthreads();
    if (threadIdx.x < 12) {
        const int k = threadIdx.x;
        const bool is_min = (k < 3) || (k >= 6 && k < 9);
        uint32_t r = s[0][k];
        for (uint32_t j = 1; j < nw; j++) r = is_min ? min(r, s[j][k]) : max(r, s[j][k]);
        uint32_t* dst = k < 6 ? &st->cb[k] : &st->bb[k - 6];
        if (is_min) atomicMin(dst, r);
        else atomicMax(dst, r);
    }
}

__global__ void k_init_state(BuildState* st) {
    if (threadIdx.x == 0) {
        for (int k = 0; k < 3; k++) {
            st->cb[k] = 0xFFFFFFFFu;
            st->cb[3 + k] = 0u;
            st->bb[k] = 0xFFFFFFFFu;
            st->bb[3 + k] = 0u;
        }
        st->node_counter = 1;
        st->level_lo = st->level_hi = 0;
        st->level_blocks_done = 0;
        st->error = 0;
        st->depth = 1;
        st->blas_kinds = 0;
        st->ploc_count[0] = st->ploc_count[1] = 0;
        st->merge_counter = 0;
        st->ploc_blocks_done = 0;
        st->dop_blocks_done = 0;
        st->radius_bits = 0;
        for (int k = 0; k < 7; k++) {
            st->dop_hi[k] = 0u;
            st->dop_lo[k] = 0xFFFFFFFFu;
        }
    }
}

__device__ __forceinline__ int find_geometry(const BlasInput& in, uint32_t i) {
    int lo = 0, hi = (int)in.geometry_count - 1;
    while (lo < hi) {
        int mid = (lo + hi + 1) >> 1;
        if (in.g[mid].prefix <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// Fetches triangle i's vertices; false for an invalid index or an inactive
// (NaN) triangle.
__device__ bool fetch_triangle(const BlasInput& in, uint32_t i, int* geom, uint32_t* prim, float v[3][3]) {
    int g = find_geometry(in, i);
    const BuildGeom& G = in.g[g];
    uint32_t p = i - G.prefix;
    *geom = g;
    *prim = p;
    uint32_t vi[3];
    if (G.idx) {
        vi[0] = G.idx[3 * (size_t)p];
        vi[1] = G.idx[3 * (size_t)p + 1];
        vi[2] = G.idx[3 * (size_t)p + 2];
    } else {
        vi[0] = 3 * p;
        vi[1] = 3 * p + 1;
        vi[2] = 3 * p + 2;
    }
    bool ok = true;
    for (int c = 0; c < 3; c++) {
        if (vi[c] > G.max_vertex) {
            ok = false;
            v[c][0] = v[c][1] = v[c][2] = __int_as_float(0x7FC00000);
            continue;
        }
        const float* src = G.pos + (size_t)vi[c] * G.stride_floats;
        v[c][0] = src[0];
        v[c][1] = src[1];
        v[c][2] = src[2];
        if (!finite3(v[c])) ok = false;
    }
    return ok;
}

__global__ void k_blas_prims(const __grid_constant__ BlasInput in, float4* boxes, BuildState* st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float bmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    if (i < in.n) {
        int g;
        uint32_t p;
        float v[3][3];
        float lo[3], hi[3];
        bool ok = fetch_triangle(in, i, &g, &p, v);
        if (ok) {
            for (int k = 0; k < 3; k++) {
                lo[k] = fminf(fminf(v[0][k], v[1][k]), v[2][k]);
                hi[k] = fmaxf(fmaxf(v[0][k], v[1][k]), v[2][k]);
            }
            pad_box(lo, hi);
            for (int k = 0; k < 3; k++) {
                float c = 0.5f * (lo[k] + hi[k]);
                cmin[k] = c;
                cmax[k] = c;
                bmin[k] = lo[k];
                bmax[k] = hi[k];
            }
        } else {
            for (int k = 0; k < 3; k++) {
                lo[k] = INFINITY;
                hi[k] = -INFINITY;
            }
            bool bad_index = false;
            const BuildGeom& G = in.g[g];
            if (G.idx) {
                for (int c = 0; c < 3; c++) bad_index |= G.idx[3 * (size_t)p + c] > G.max_vertex;
            } else {
                bad_index = 3 * p + 2 > G.max_vertex;
            }
            if (bad_index) atomicOr(&st->error, 1u << RT_ERR_INVALID);
        }
        boxes[2 * (size_t)i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        boxes[2 * (size_t)i + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    }
    reduce_bounds(st, cmin, cmax, bmin, bmax);
}

// Fills a TLAS instance record from the caller's instance `r` (index id):
// world-to-object inverse, BLAS fields for the traversal, and the world box
// = the 8 transformed corners of the BLAS bounds, padded so the box stays
// conservative for the rounded object-space ray.  Returns false (empty box,
// tri_count 0) for a singular transform or a null / empty BLAS.
__device__ bool fill_instance(const RtAccelerationStructureInstance& r, uint32_t id, InstRecord* rec, float lo[3],
                              float hi[3], uint32_t* err) {
    const float* m = &r.transform[0][0];
    for (int k = 0; k < 12; k++) rec->o2w[k] = m[k];
    bool valid = affine_inverse(m, rec->w2o);
    rec->blas = r.acceleration_structure_reference;
    rec->instance_id = id;
    rec->custom_mask = r.instance_custom_index_and_mask;
    rec->sbt_flags = r.instance_shader_binding_table_record_offset_and_flags;
    rec->tri_count = 0;
    rec->node_count = 0;
    rec->prims_off256 = 0;
    for (int k = 0; k < 3; k++) {
        lo[k] = INFINITY;
        hi[k] = -INFINITY;
    }
    if (rec->blas == 0) valid = false;
    if (valid) {
        const AsHeader* bh = reinterpret_cast<const AsHeader*>(rec->blas);
        if (bh->magic != kAsMagic || bh->type != kAsTypeBottom) {
            valid = false;
            atomicOr(err, 1u << RT_ERR_BAD_AS);
        } else if (bh->prim_count == 0) {
            valid = false;
        } else {
            float blo[3] = {bh->bounds_lo[0], bh->bounds_lo[1], bh->bounds_lo[2]};
            float bhi[3] = {bh->bounds_hi[0], bh->bounds_hi[1], bh->bounds_hi[2]};
            for (int c = 0; c < 8; c++) {
                V3 p = mk3((c & 1) ? bhi[0] : blo[0], (c & 2) ? bhi[1] : blo[1], (c & 4) ? bhi[2] : blo[2]);
                V3 q = xform_point(rec->o2w, p);
                lo[0] = fminf(lo[0], q.x);
                lo[1] = fminf(lo[1], q.y);
                lo[2] = fminf(lo[2], q.z);
                hi[0] = fmaxf(hi[0], q.x);
                hi[1] = fmaxf(hi[1], q.y);
                hi[2] = fmaxf(hi[2], q.z);
            }
            // Cut to the box of the transformed bounding sphere: the ellipsoid
            // M S + t has half-extent r |row_k(M)| along world axis k.  The
            // transformed centre is widened by its rounding error (a few ulps
            // of |M c| + |t|); the padding below adds more.
            const float rad = bh->sphere_radius;
            if (rad > 0.0f && rad <= FLT_MAX) {
                const float* M = rec->o2w;
                V3 cw = xform_point(M, mk3(bh->sphere_center[0], bh->sphere_center[1], bh->sphere_center[2]));
                const float cwv[3] = {cw.x, cw.y, cw.z};
                for (int k = 0; k < 3; k++) {
                    const float a = M[4 * k], b = M[4 * k + 1], d = M[4 * k + 2];
                    const float row = __fsqrt_ru(__fadd_ru(__fadd_ru(__fmul_ru(a, a), __fmul_ru(b, b)), __fmul_ru(d, d)));
                    const float mc = __fadd_ru(__fadd_ru(__fmul_ru(fabsf(a), fabsf(bh->sphere_center[0])),
                                                         __fmul_ru(fabsf(b), fabsf(bh->sphere_center[1]))),
                                               __fadd_ru(__fmul_ru(fabsf(d), fabsf(bh->sphere_center[2])),
                                                         fabsf(M[4 * k + 3])));
                    const float e = __fadd_ru(__fmul_ru(rad, row), __fmul_ru(mc, 4.8e-7f));  // + 4 ulps of |M c| + |t|
                    lo[k] = fmaxf(lo[k], __fsub_rd(cwv[k], e));
                    hi[k] = fminf(hi[k], __fadd_ru(cwv[k], e));
                }
            }
            // and to the box of the transformed 14-DOP vertices
            const uint32_t nd = bh->dop_count;
            if (nd >= 4u && nd <= kDopMaxVertices) {
                float dlo[3] = {INFINITY, INFINITY, INFINITY}, dhi[3] = {-INFINITY, -INFINITY, -INFINITY};
                for (uint32_t v = 0; v < nd; v++) {
                    const V3 q = xform_point(rec->o2w, mk3(bh->dop_vertex[v][0], bh->dop_vertex[v][1],
                                                          bh->dop_vertex[v][2]));
                    dlo[0] = fminf(dlo[0], q.x); dlo[1] = fminf(dlo[1], q.y); dlo[2] = fminf(dlo[2], q.z);
                    dhi[0] = fmaxf(dhi[0], q.x); dhi[1] = fmaxf(dhi[1], q.y); dhi[2] = fmaxf(dhi[2], q.z);
                }
                for (int k = 0; k < 3; k++) {
                    lo[k] = fmaxf(lo[k], dlo[k]);
                    hi[k] = fminf(hi[k], dhi[k]);
                }
            }
            float ext = fmaxf(fmaxf(hi[0] - lo[0], hi[1] - lo[1]), hi[2] - lo[2]);
            for (int k = 0; k < 3; k++) {
                float pad = (fmaxf(fabsf(lo[k]), fabsf(hi[k])) + ext) * 1e-5f + 1e-20f;
                lo[k] -= pad;
                hi[k] += pad;
            }
            if (!finite3(lo) || !finite3(hi)) valid = false;
            if (valid) {
                rec->tri_count = bh->prim_count;
                rec->node_count = bh->node_count | (bh->node_bytes == kQNodeBytes ? kQuantizedBlasBit : 0u);
                rec->prims_off256 = (uint32_t)(bh->prims_offset / 256);
            }
        }
    }
    if (!valid) {
        rec->tri_count = 0;
        for (int k = 0; k < 3; k++) {
            lo[k] = INFINITY;
            hi[k] = -INFINITY;
        }
    }
    return valid;
}

__global__ void k_tlas_prims(const RtAccelerationStructureInstance* inst, uint32_t n, float4* boxes,
                             InstRecord* temp, BuildState* st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    float bmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    uint32_t kinds = 0;
    if (i < n) {
        RtAccelerationStructureInstance r = inst[i];
        InstRecord rec;
        float lo[3], hi[3];
        if (fill_instance(r, i, &rec, lo, hi, &st->error)) {
            for (int k = 0; k < 3; k++) {
                float c = 0.5f * (lo[k] + hi[k]);
                cmin[k] = cmax[k] = c;
                bmin[k] = lo[k];
                bmax[k] = hi[k];
            }
            kinds = blas_kind(rec.node_count);
        }
        temp[i] = rec;
        boxes[2 * (size_t)i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        boxes[2 * (size_t)i + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
    }
    kinds = __reduce_or_sync(0xFFFFFFFFu, kinds);
    if ((threadIdx.x & 31u) == 0 && kinds) atomicOr(&st->blas_kinds, kinds);
    reduce_bounds(st, cmin, cmax, bmin, bmax);
}

__device__ __forceinline__ uint32_t expand_bits10(uint32_t x) {
    x = (x * 0x00010001u) & 0xFF0000FFu;
    x = (x * 0x00000101u) & 0x0F00F00Fu;
    x = (x * 0x00000011u) & 0xC30C30C3u;
    x = (x * 0x00000005u) & 0x49249249u;
    return x;
}

__global__ void k_morton(const float4* boxes, uint32_t n, const BuildState* st, uint32_t* keys, uint32_t* vals) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float4 lo = boxes[2 * (size_t)i], hi = boxes[2 * (size_t)i + 1];
    float c[3] = {0.5f * (lo.x + hi.x), 0.5f * (lo.y + hi.y), 0.5f * (lo.z + hi.z)};
    uint32_t q[3] = {0, 0, 0};
    if (finite3(c)) {
        for (int k = 0; k < 3; k++) {
            float mn = o2f(st->cb[k]), mx = o2f(st->cb[3 + k]);
            float ext = mx - mn;
            float x = ext > 0.0f ? (c[k] - mn) / ext : 0.0f;
            float s = fminf(fmaxf(x * 1024.0f, 0.0f), 1023.0f);
            q[k] = (uint32_t)s;
        }
    }
    keys[i] = (expand_bits10(q[0]) << 2) | (expand_bits10(q[1]) << 1) | expand_bits10(q[2]);
    vals[i] = i;
}

// Exclusive scan of m values in place by one block of 1024 threads (all of
// them call it); returns the total to every thread.  Values are read through
// L2: other blocks of the same launch may have written them.
__device__ uint32_t block_exclusive_scan(uint32_t* data, uint32_t m, uint32_t* warp_sums) {
    const uint32_t per = (m + 1023) / 1024;
    const uint32_t b = threadIdx.x * per, e = min(m, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; i++) sum += __ldcg(&data[i]);
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t incl = sum;
    for (int off = 1; off < 32; off <<= 1) {
        uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= (uint32_t)off) incl += o;
    }
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = warp_sums[lane];
        uint32_t wi = w;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t o = __shfl_up_sync(0xFFFFFFFFu, wi, off);
            if (lane >= (uint32_t)off) wi += o;
        }
        warp_sums[lane] = wi - w;
        if (lane == 31) warp_sums[32] = wi;
    }
    __syncthreads();
    uint32_t run = warp_sums[warp] + incl - sum;
    for (uint32_t i = b; i < e; i++) {
        const uint32_t v = __ldcg(&data[i]);
        data[i] = run;
        run += v;
    }
    const uint32_t total = warp_sums[32];
    __syncthreads();
    return total;
}

struct SortTileShared {
    uint32_t digit_base[256];
    uint32_t run[256];
    uint32_t warp_cnt[kSortThreads / 32][256];
};

// Stable scatter of tile `tile` (kSortTile keys) by digit (key >> shift) & 255,
// to digit_base[d] plus the key's rank among the tile's keys of digit d.
// Expects digit_base filled, run zeroed and a barrier before the call.
__device__ void scatter_tile(SortTileShared& sm, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                             uint32_t* vout, uint32_t n, int shift, uint32_t tile);

// All four passes of the radix sort in one block, for n <= kSortTile keys:
// k0 / v0 -> k1 / v1 -> k0 / v0 ..., the result in k0 / v0.
__global__ void __launch_bounds__(kSortThreads) k_radix_sort_small(uint32_t* k0, uint32_t* v0, uint32_t* k1,
                                                                   uint32_t* v1, uint32_t n) {
    __shared__ SortTileShared sm;
    __shared__ uint32_t warp_sums[kSortThreads / 32];
    uint32_t* kin = k0;
    uint32_t* vin = v0;
    uint32_t* kout = k1;
    uint32_t* vout = v1;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    for (int pass = 0; pass < 4; pass++) {
        const int shift = pass * 8;
        for (int d = threadIdx.x; d < 256; d += blockDim.x) {
            sm.digit_base[d] = 0;
            sm.run[d] = 0;
        }
        __syncthreads();
        for (uint32_t i = threadIdx.x; i < n; i += blockDim.x) atomicAdd(&sm.digit_base[(kin[i] >> shift) & 255u], 1u);
        __syncthreads();
        // exclusive scan of the 256 digit counts (one per thread; kSortThreads == 256)
        const uint32_t c = sm.digit_base[threadIdx.x];
        uint32_t incl = c;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= (uint32_t)off) incl += o;
        }
        if (lane == 31u) warp_sums[warp] = incl;
        __syncthreads();
        uint32_t before = 0;
        for (uint32_t w = 0; w < warp; w++) before += warp_sums[w];
        sm.digit_base[threadIdx.x] = before + incl - c;
        __syncthreads();
        scatter_tile(sm, kin, vin, kout, vout, n, shift, 0);
        __syncthreads();
        uint32_t* t = kin; kin = kout; kout = t;
        t = vin; vin = vout; vout = t;
    }
}

__device__ void scatter_tile(SortTileShared& sm, const uint32_t* kin, const uint32_t* vin, uint32_t* kout,
                             uint32_t* vout, uint32_t n, int shift, uint32_t tile) {
    uint32_t* digit_base = sm.digit_base;
    uint32_t* run = sm.run;
    auto& warp_cnt = sm.warp_cnt;
    const uint32_t lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const uint32_t lanemask_lt = (1u << lane) - 1u;
    uint32_t base = tile * kSortTile;
    for (int j = 0; j < kSortItems; j++) {
        for (int i = threadIdx.x; i < (kSortThreads / 32) * 256; i += blockDim.x) (&warp_cnt[0][0])[i] = 0;
        __syncthreads();
        uint32_t idx = base + j * kSortThreads + threadIdx.x;
        bool valid = idx < n;
        uint32_t key = valid ? kin[idx] : 0u;
        uint32_t val = valid ? vin[idx] : 0u;
        uint32_t d = valid ? ((key >> shift) & 255u) : 256u;
        uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        uint32_t rank = __popc(peers & lanemask_lt);
        if (valid && rank == 0) warp_cnt[warp][d] = __popc(peers);
        __syncthreads();
        if (threadIdx.x < 256) {
            uint32_t dd = threadIdx.x;
            uint32_t r = run[dd];
            for (int w = 0; w < kSortThreads / 32; w++) {
                uint32_t c = warp_cnt[w][dd];
                warp_cnt[w][dd] = r;
                r += c;
            }
            run[dd] = r;
        }
        __syncthreads();
        if (valid) {
            uint32_t pos = digit_base[d] + warp_cnt[warp][d] + rank;
            if (pos < n) {
                kout[pos] = key;
                vout[pos] = val;
            }
        }
        __syncthreads();
    }
}

// ---- onesweep radix sort ------------------------------------------------------
// Keys of more than one sort tile are sorted by the single-pass LSD scheme of
// Adinets & Merrill ("Onesweep", 2022): one upfront histogram of all four
// 8-bit digits, then one kernel per digit.  In a digit pass each block takes
// the next partition of kOsTile keys from a counter (so every earlier
// partition belongs to a block that is already running), ranks its keys
// stably per digit (warp match_any, warps over consecutive chunks), publishes
// its per-digit counts, and finds the keys of each digit in all earlier
// partitions by decoupled look-back: it walks back over their descriptors,
// adding aggregates until one carries the inclusive prefix.  The tile is then
// staged in shared memory in digit order and written out so that consecutive
// threads write consecutive positions.  Each look-back wait is bounded: after
// kOsSpinLimit polls the build records RT_ERR_TIMEOUT and goes on.
constexpr int kOsThreads = 256;
constexpr int kOsItems = 15;
constexpr uint32_t kOsTile = kOsThreads * kOsItems;  // 3840 keys per partition
constexpr int kOsWarps = kOsThreads / 32;
constexpr uint32_t kOsAggregate = 1u << 30, kOsPrefix = 2u << 30, kOsValue = (1u << 30) - 1u;
constexpr uint32_t kOsSpinLimit = 1u << 22;

// The sort's scratch header: digit counts of the four passes (scanned in
// place to each digit's first output position) and each pass's partition
// counter.  The partition descriptors follow: [pass][partition][digit].
struct OnesweepState {
    uint32_t count[4][256];
    uint32_t next_partition[4];
};

__host__ __device__ inline uint32_t onesweep_partitions(uint32_t n) { return (n + kOsTile - 1) / kOsTile; }

__device__ __forceinline__ uint32_t ld_relaxed(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed(uint32_t* p, uint32_t v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__global__ void __launch_bounds__(kOsThreads) k_onesweep_hist(const uint32_t* keys, uint32_t n, OnesweepState* os) {
    __shared__ uint32_t h[4][256];
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) (&h[0][0])[i] = 0;
    __syncthreads();
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint32_t k = keys[i];
        atomicAdd(&h[0][k & 255u], 1u);
        atomicAdd(&h[1][(k >> 8) & 255u], 1u);
        atomicAdd(&h[2][(k >> 16) & 255u], 1u);
        atomicAdd(&h[3][k >> 24], 1u);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 1024; i += blockDim.x) {
        const uint32_t c = (&h[0][0])[i];
        if (c) atomicAdd(&(&os->count[0][0])[i], c);
    }
}

// Exclusive scan of 256 values by 256 threads (one value each).
__device__ __forceinline__ uint32_t block_scan256(uint32_t c, uint32_t* warp_sums) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = c;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= (uint32_t)off) incl += o;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    uint32_t before = 0;
    for (uint32_t w = 0; w < warp; w++) before += warp_sums[w];
    return before + incl - c;
}

// Block b: the digit counts of pass b -> each digit's first output position.
__global__ void __launch_bounds__(256) k_onesweep_scan(OnesweepState* os) {
    __shared__ uint32_t warp_sums[8];
    const uint32_t d = threadIdx.x;
    os->count[blockIdx.x][d] = block_scan256(os->count[blockIdx.x][d], warp_sums);
}

struct OnesweepShared {
    uint32_t keys[kOsTile];
    uint32_t vals[kOsTile];
    uint32_t warp_cnt[kOsWarps][256];  // keys of each digit per warp, then each warp's offset among them
    uint32_t tile_start[256];          // first position of each digit in the staged tile
    uint32_t out_start[256];           // first output position of the tile's keys of each digit
    uint32_t warp_sums[8];
    uint32_t partition;
};

// One digit pass (bits pass*8 .. pass*8+7) over n keys: kin / vin -> kout / vout.
// desc: this pass's descriptors, 256 per partition, zeroed.
__global__ void __launch_bounds__(kOsThreads) k_onesweep_pass(const uint32_t* kin, const uint32_t* vin,
                                                               uint32_t* kout, uint32_t* vout, uint32_t n, int pass,
                                                               OnesweepState* os, uint32_t* desc,
                                                               uint32_t* error) {
    __shared__ OnesweepShared sm;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    const int shift = pass * 8;
    if (tid == 0) sm.partition = atomicAdd(&os->next_partition[pass], 1u);
    for (uint32_t i = tid; i < kOsWarps * 256; i += kOsThreads) (&sm.warp_cnt[0][0])[i] = 0;
    __syncthreads();
    const uint32_t p = sm.partition;
    const uint32_t base = p * kOsTile;
    const uint32_t lt = (1u << lane) - 1u;
    uint32_t key[kOsItems], val[kOsItems], rank[kOsItems];
    // warp w ranks keys base + w*32*kOsItems .. in rounds of 32, in order: stable within the tile
#pragma unroll
    for (int r = 0; r < kOsItems; r++) {
        const uint32_t idx = base + ((uint32_t)warp * kOsItems + r) * 32u + lane;
        const bool valid = idx < n;
        key[r] = valid ? kin[idx] : 0u;
        val[r] = valid ? vin[idx] : 0u;
        const uint32_t d = valid ? ((key[r] >> shift) & 255u) : 256u;
        const uint32_t peers = __match_any_sync(0xFFFFFFFFu, d);
        const uint32_t before = valid ? sm.warp_cnt[warp][d] : 0u;
        __syncwarp();
        if (valid && (peers & lt) == 0u) sm.warp_cnt[warp][d] = before + (uint32_t)__popc(peers);
        __syncwarp();
        rank[r] = valid ? before + (uint32_t)__popc(peers & lt) : 0xFFFFFFFFu;
    }
    __syncthreads();
    // thread d: the tile's keys of digit d, and each warp's offset among them
    const uint32_t d = tid;
    uint32_t total = 0;
    for (int w = 0; w < kOsWarps; w++) {
        const uint32_t c = sm.warp_cnt[w][d];
        sm.warp_cnt[w][d] = total;
        total += c;
    }
    // publish, then look back for the keys of digit d in the earlier partitions
    uint32_t* mine = desc + (size_t)p * 256u + d;
    uint32_t excl = 0;
    if (p == 0) {
        st_relaxed(mine, kOsPrefix | total);
    } else {
        st_relaxed(mine, kOsAggregate | total);
        uint32_t q = p - 1, spins = 0;
        for (;;) {
            const uint32_t v = ld_relaxed(desc + (size_t)q * 256u + d);
            const uint32_t flag = v & ~kOsValue;
            if (flag == 0u) {
                if (++spins > kOsSpinLimit) {  // bounded: report and go on with what was found
                    atomicOr(error, 1u << RT_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(32);
                continue;
            }
            excl += v & kOsValue;
            if (flag == kOsPrefix || q == 0u) break;
            q--;
        }
        st_relaxed(mine, kOsPrefix | (excl + total));
    }
    sm.tile_start[d] = block_scan256(total, sm.warp_sums);
    sm.out_start[d] = os->count[pass][d] + excl;
    __syncthreads();
    // stage the tile in digit order, then write it out in that order
#pragma unroll
    for (int r = 0; r < kOsItems; r++) {
        if (rank[r] == 0xFFFFFFFFu) continue;
        const uint32_t dg = (key[r] >> shift) & 255u;
        const uint32_t local = sm.tile_start[dg] + sm.warp_cnt[warp][dg] + rank[r];
        sm.keys[local] = key[r];
        sm.vals[local] = val[r];
    }
    __syncthreads();
    const uint32_t cnt = min(kOsTile, n - base);
    for (uint32_t i = tid; i < cnt; i += kOsThreads) {
        const uint32_t k = sm.keys[i];
        const uint32_t dg = (k >> shift) & 255u;
        const uint32_t pos = sm.out_start[dg] + (i - sm.tile_start[dg]);
        if (pos < n) {
            kout[pos] = k;
            vout[pos] = sm.vals[i];
        }
    }
}

}  // namespace

uint64_t key_sort_state_bytes(uint32_t n) {
    return sizeof(OnesweepState) + (uint64_t)4 * onesweep_partitions(n ? n : 1) * 256u * 4u;
}

cudaError_t launch_key_sort(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, uint8_t* state,
                            uint32_t* error, cudaStream_t stream) {
    if (n <= 1) return cudaSuccess;
    if (n <= kSortTile) {
        // one block sorts all four digits
        note_launch(), k_radix_sort_small<<<1, kSortThreads, 0, stream>>>(k0, v0, k1, v1, n);
        return cudaGetLastError();
    }
    OnesweepState* os = reinterpret_cast<OnesweepState*>(state);
    uint32_t* desc = reinterpret_cast<uint32_t*>(state + sizeof(OnesweepState));
    const uint32_t parts = onesweep_partitions(n);
    cudaError_t e = cudaMemsetAsync(state, 0, key_sort_state_bytes(n), stream);
    if (e != cudaSuccess) return e;
    note_launch(), k_onesweep_hist<<<std::min<uint32_t>(parts, 1024u), kOsThreads, 0, stream>>>(k0, n, os);
    note_launch(), k_onesweep_scan<<<4, 256, 0, stream>>>(os);
    uint32_t* kin = k0;
    uint32_t* vin = v0;
    uint32_t* kout = k1;
    uint32_t* vout = v1;
    for (int pass = 0; pass < 4; pass++) {
        note_launch(), k_onesweep_pass<<<parts, kOsThreads, 0, stream>>>(kin, vin, kout, vout, n, pass, os,
                                                                          desc + (size_t)pass * parts * 256u, error);
        std::swap(kin, kout);
        std::swap(vin, vout);
    }
    return cudaGetLastError();
}

namespace {

__global__ void k_gather_boxes(const float4* boxes, const uint32_t* vals, uint32_t n, float4* sboxes) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = vals[i];
    sboxes[2 * (size_t)i] = boxes[2 * (size_t)p];
    sboxes[2 * (size_t)i + 1] = boxes[2 * (size_t)p + 1];
}

// ---- Karras hierarchy -------------------------------------------------------
__device__ __forceinline__ int kdelta(const uint32_t* k, int n, int i, int j) {
    if (j < 0 || j >= n) return -1;
    uint32_t a = k[i], b = k[j];
    if (a == b) return 32 + __clz((uint32_t)i ^ (uint32_t)j);
    return __clz(a ^ b);
}

__global__ void k_karras(const uint32_t* keys, uint32_t n_u, uint4* inodes, uint32_t* iparent, uint32_t* lparent) {
    int n = (int)n_u;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n - 1) return;
    int d = (kdelta(keys, n, i, i + 1) - kdelta(keys, n, i, i - 1)) >= 0 ? 1 : -1;
    int dmin = kdelta(keys, n, i, i - d);
    int lmax = 2;
    while (kdelta(keys, n, i, i + lmax * d) > dmin) lmax <<= 1;
    int l = 0;
    for (int t = lmax >> 1; t >= 1; t >>= 1)
        if (kdelta(keys, n, i, i + (l + t) * d) > dmin) l += t;
    int j = i + l * d;
    int dnode = kdelta(keys, n, i, j);
    int s = 0;
    int t = l;
    do {
        t = (t + 1) >> 1;
        if (kdelta(keys, n, i, i + (s + t) * d) > dnode) s += t;
    } while (t > 1);
    int gamma = i + s * d + min(d, 0);
    int first = min(i, j), last = max(i, j);
    uint32_t left = (first == gamma) ? (kLeafBit | (uint32_t)gamma) : (uint32_t)gamma;
    uint32_t right = (last == gamma + 1) ? (kLeafBit | (uint32_t)(gamma + 1)) : (uint32_t)(gamma + 1);
    inodes[i] = make_uint4(left, right, (uint32_t)first, (uint32_t)last);
    if (left & kLeafBit) lparent[gamma] = (uint32_t)i;
    else iparent[gamma] = (uint32_t)i;
    if (right & kLeafBit) lparent[gamma + 1] = (uint32_t)i;
    else iparent[gamma + 1] = (uint32_t)i;
    if (i == 0) iparent[0] = kNone;
}

__device__ __forceinline__ void load_box_cg(const float4* b, size_t i, float lo[3], float hi[3]) {
    float4 l = __ldcg(&b[2 * i]), h = __ldcg(&b[2 * i + 1]);
    lo[0] = l.x; lo[1] = l.y; lo[2] = l.z;
    hi[0] = h.x; hi[1] = h.y; hi[2] = h.z;
}

__global__ void k_bottom_up(const uint4* inodes, const uint32_t* lparent, const uint32_t* iparent,
                            const float4* sboxes, float4* iboxes, uint32_t* flags, uint32_t n, uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    uint32_t p = lparent[i];
    for (int guard = 0; p != kNone; guard++) {
        if (guard >= 160 || p >= n - 1) {  // deeper than any Karras tree of 2^28 keys
            atomicOr(err, 1u << RT_ERR_BAD_AS);
            return;
        }
        __threadfence();
        if (atomicAdd(&flags[p], 1u) == 0u) return;
        uint4 nd = __ldcg(&inodes[p]);
        float llo[3], lhi[3], rlo[3], rhi[3];
        if (nd.x & kLeafBit) load_box_cg(sboxes, nd.x & ~kLeafBit, llo, lhi);
        else load_box_cg(iboxes, nd.x, llo, lhi);
        if (nd.y & kLeafBit) load_box_cg(sboxes, nd.y & ~kLeafBit, rlo, rhi);
        else load_box_cg(iboxes, nd.y, rlo, rhi);
        iboxes[2 * (size_t)p] = make_float4(fminf(llo[0], rlo[0]), fminf(llo[1], rlo[1]), fminf(llo[2], rlo[2]), 0.0f);
        iboxes[2 * (size_t)p + 1] =
            make_float4(fmaxf(lhi[0], rhi[0]), fmaxf(lhi[1], rhi[1]), fmaxf(lhi[2], rhi[2]), 0.0f);
        p = __ldcg(&iparent[p]);
    }
}

// ---- PLOC hierarchy (RT_BUILD_PREFER_FAST_TRACE) --------------------------------
// Parallel locally-ordered clustering (Meister & Bittner, "Parallel
// Locally-Ordered Clustering for Bounding Volume Hierarchy Construction",
// IEEE TVCG 2018).  The clusters start as the Morton-ordered primitives.
// Each round every cluster finds, among the kPlocRadius clusters on either
// side of it, the one whose merged box has the smallest surface area; mutual
// nearest neighbours merge into a new internal node at the lower position,
// and the surviving clusters are compacted in order.  Internal node ids are
// handed out from n - 2 down, so the last merge (the root) is node 0, where
// the collapse starts.  Rounds over more than kPlocSmall clusters run as
// grid-wide launches (their cluster count stays on the device: a round that
// finds kPlocSmall or fewer clusters does nothing); one CTA with every
// cluster in shared memory finishes.  If a round merges nothing (equal or NaN
// areas), the next one merges neighbour pairs (i, i ^ 1) so the loop always
// ends.  The host launches ploc_grid_rounds(n) grid-wide rounds: enough
// nearest-neighbour rounds for the count to fall to kPlocSmall at the
// measured rate (about 0.58 of the primitives survive the first round, 0.81
// of the clusters each later one), then pair rounds, each halving the count,
// in case it has not.
constexpr int kPlocRadius = 16;
constexpr uint32_t kPlocSmall = 4096;
constexpr uint32_t kPlocChunk = 256;        // clusters per block of the neighbour search
constexpr uint32_t kPlocScanBlock = 1024;   // clusters per block of the compaction scan
constexpr uint32_t kPlocSmallThreads = 1024;
constexpr uint32_t kPlocSmallPer = kPlocSmall / kPlocSmallThreads;
constexpr size_t kPlocSmallSmem = (size_t)kPlocSmall * 10 * 4;  // 6 box floats, ref, neighbour, keep, size

__device__ __forceinline__ float merged_half_area(float ax, float ay, float az, float bx, float by, float bz,
                                                  float cx, float cy, float cz, float dx, float dy, float dz) {
    // boxes (a, b) and (c, d) as lo, hi corners
    float ex = fmaxf(bx, dx) - fminf(ax, cx), ey = fmaxf(by, dy) - fminf(ay, cy), ez = fmaxf(bz, dz) - fminf(az, cz);
    return ex * ey + ey * ez + ez * ex;
}

__device__ __forceinline__ uint32_t ploc_size(const uint32_t* counts, uint32_t r) {
    return (r & kLeafBit) ? 1u : __ldcg(&counts[r]);
}

__global__ void k_ploc_init(const float4* sboxes, uint32_t n, uint32_t* cref, float4* cbox, BuildState* st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) st->ploc_count[0] = n;
    if (i >= n) return;
    cref[i] = kLeafBit | i;
    cbox[2 * (size_t)i] = sboxes[2 * (size_t)i];
    cbox[2 * (size_t)i + 1] = sboxes[2 * (size_t)i + 1];
}

// Nearest neighbour of every cluster within kPlocRadius positions (smallest
// merged-box surface area, the lower position on ties).  The area of a pair
// does not depend on the order of its boxes (min / max per axis), so each pair
// is evaluated once: a block stages kPlocChunk clusters' boxes plus the halo in
// shared memory, every position p of [c0 - R, c0 + kPlocChunk) writes the
// areas of (p, p + o) for o = 1..R, and then each cluster scans its candidates
// in ascending position, the pairs below it first.
__global__ void __launch_bounds__(kPlocChunk) k_ploc_nn(const float4* cbox, uint32_t* nn, const BuildState* st,
                                                          int round, int forced) {
    const uint32_t count = st->ploc_count[round & 1];
    if (count <= kPlocSmall) return;
    constexpr int R = kPlocRadius;
    constexpr int kSpan = (int)kPlocChunk + R;  // positions whose forward pairs a tile needs
    __shared__ float4 slo[kPlocChunk + 2 * R], shi[kPlocChunk + 2 * R];
    __shared__ float area[R][kSpan];            // area[o - 1][p - (c0 - R)] = area of (p, p + o)
    for (uint32_t c0 = blockIdx.x * kPlocChunk; c0 < count; c0 += gridDim.x * kPlocChunk) {
        const uint32_t i = c0 + threadIdx.x;
        if (forced) {  // pair rounds: neighbours are fixed pairs
            if (i < count) nn[i] = (i ^ 1u) < count ? (i ^ 1u) : i;
            continue;
        }
        for (uint32_t t = threadIdx.x; t < kPlocChunk + 2 * R; t += blockDim.x) {
            const int64_t g = (int64_t)c0 - R + t;
            if (g >= 0 && g < (int64_t)count) {
                slo[t] = __ldcg(&cbox[2 * g]);
                shi[t] = __ldcg(&cbox[2 * g + 1]);
            }
        }
        __syncthreads();
        for (int lp = threadIdx.x; lp < kSpan; lp += blockDim.x) {
            const int64_t gp = (int64_t)c0 - R + lp;
            if (gp < 0 || gp >= (int64_t)count) continue;
            const float4 a = slo[lp], b = shi[lp];
#pragma unroll
            for (int o = 1; o <= R; o++) {
                const float4 c = slo[lp + o], d = shi[lp + o];
                area[o - 1][lp] = merged_half_area(a.x, a.y, a.z, b.x, b.y, b.z, c.x, c.y, c.z, d.x, d.y, d.z);
            }
        }
        __syncthreads();
        if (i < count) {
            const int li = (int)threadIdx.x + R;
            uint32_t best = i;
            float bd = INFINITY;
            for (int o = R; o >= 1; o--) {  // candidates i - R .. i - 1
                if ((int64_t)i - o < 0) continue;
                const float h = area[o - 1][li - o];
                if (h < bd) {  // ties keep the lower position
                    bd = h;
                    best = i - o;
                }
            }
            for (int o = 1; o <= R; o++) {  // candidates i + 1 .. i + R
                if (i + o >= count) break;
                const float h = area[o - 1][li];
                if (h < bd) {
                    bd = h;
                    best = i + o;
                }
            }
            nn[i] = best;
        }
        __syncthreads();
    }
}

// One round's merges and the compaction offsets.  Block b takes tiles of
// kPlocScanBlock clusters.  Cluster i merges with its nearest neighbour j
// when j's nearest is i: the lower position keeps the new node, the higher
// one drops out.  One scan per tile counts survivors (low 16 bits) and merges
// (high 16 bits): the survivors' offsets go to scan and their total to blk,
// and the tile claims its merges' node ids (counting down from n - 2) with
// one atomic.  The block that finishes last turns the tile totals into tile
// offsets and sets the next round's cluster count (a count of finished
// blocks: no block waits for another).
__global__ void __launch_bounds__(kPlocScanBlock) k_ploc_merge(
    const uint32_t* cref, const float4* cbox, const uint32_t* nn, uint32_t* tref, float4* tbox, uint32_t* keep,
    uint32_t* scan, uint32_t* blk, uint4* inodes, float4* iboxes, uint32_t* counts, BuildState* st, int round,
    uint32_t n) {
    const uint32_t count = st->ploc_count[round & 1];
    if (count <= kPlocSmall) return;
    __shared__ uint32_t warp_sums[33];
    __shared__ uint32_t tile_base, last;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t tiles = (count + kPlocScanBlock - 1) / kPlocScanBlock;
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        const uint32_t i = tile * kPlocScanBlock + threadIdx.x;
        const bool valid = i < count;
        uint32_t r = 0u, k = 0u, j = i;
        bool merging = false;
        float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
        if (valid) {
            j = __ldcg(&nn[i]);
            r = __ldcg(&cref[i]);
            lo = __ldcg(&cbox[2 * (size_t)i]);
            hi = __ldcg(&cbox[2 * (size_t)i + 1]);
            k = 1u;
            if (j != i && j < count && __ldcg(&nn[j]) == i) {
                if (i < j) merging = true;
                else k = 0u;
            }
        }
        const uint32_t v = k | (merging ? 1u << 16 : 0u);
        uint32_t incl = v;
        for (int off = 1; off < 32; off <<= 1) {
            const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= (uint32_t)off) incl += o;
        }
        if (lane == 31u) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            const uint32_t w = warp_sums[lane];
            uint32_t wi = w;
            for (int off = 1; off < 32; off <<= 1) {
                const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, wi, off);
                if (lane >= (uint32_t)off) wi += o;
            }
            warp_sums[lane] = wi - w;
            if (lane == 31u) {
                blk[tile] = wi & 0xFFFFu;
                tile_base = (wi >> 16) ? atomicAdd(&st->merge_counter, wi >> 16) : 0u;
            }
        }
        __syncthreads();
        const uint32_t excl = warp_sums[warp] + incl - v;
        if (merging) {
            const uint32_t claim = tile_base + (excl >> 16);
            if (claim + 2u > n) {  // more merges than a binary tree over n primitives has
                atomicOr(&st->error, 1u << RT_ERR_BAD_AS);
            } else {
                const uint32_t id = n - 2u - claim;
                const uint32_t rj = __ldcg(&cref[j]);
                const float4 lj = __ldcg(&cbox[2 * (size_t)j]), hj = __ldcg(&cbox[2 * (size_t)j + 1]);
                lo = make_float4(fminf(lo.x, lj.x), fminf(lo.y, lj.y), fminf(lo.z, lj.z), 0.0f);
                hi = make_float4(fmaxf(hi.x, hj.x), fmaxf(hi.y, hj.y), fmaxf(hi.z, hj.z), 0.0f);
                inodes[id] = make_uint4(r, rj, 0u, 0u);
                iboxes[2 * (size_t)id] = lo;
                iboxes[2 * (size_t)id + 1] = hi;
                counts[id] = ploc_size(counts, r) + ploc_size(counts, rj);
                r = id;
            }
        }
        if (valid) {
            tref[i] = r;
            tbox[2 * (size_t)i] = lo;
            tbox[2 * (size_t)i + 1] = hi;
            keep[i] = k;
            scan[i] = excl & 0xFFFFu;
        }
        __syncthreads();
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&st->ploc_blocks_done, 1u) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (last) {
        __threadfence();
        const uint32_t total = block_exclusive_scan(blk, tiles, warp_sums);
        if (threadIdx.x == 0) {
            st->ploc_count[(round + 1) & 1] = total;
            st->ploc_blocks_done = 0;
        }
    }
}

// Survivors to their compacted positions (tile offset + offset in the tile).
__global__ void k_ploc_scatter(const uint32_t* tref, const float4* tbox, const uint32_t* keep, const uint32_t* scan,
                               const uint32_t* blk, uint32_t* cref, float4* cbox, BuildState* st, int round) {
    const uint32_t count = st->ploc_count[round & 1];
    if (count <= kPlocSmall) {
        if (blockIdx.x == 0 && threadIdx.x == 0) st->ploc_count[(round + 1) & 1] = count;
        return;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
        const uint32_t k = __ldcg(&keep[i]);
        const uint32_t pos = __ldcg(&blk[i / kPlocScanBlock]) + __ldcg(&scan[i]);
        if (k) {
            cref[pos] = __ldcg(&tref[i]);
            cbox[2 * (size_t)pos] = __ldcg(&tbox[2 * (size_t)i]);
            cbox[2 * (size_t)pos + 1] = __ldcg(&tbox[2 * (size_t)i + 1]);
        }
    }
}

// The last rounds, in one CTA: every cluster (at most kPlocSmall) in shared
// memory with its size; node ids are claimed from a shared counter.  With
// few clusters, G = 2..32 threads share one cluster's neighbour search (each
// takes every G-th offset, then a shuffle reduction keeps the smallest area,
// the lower position on ties); otherwise thread t owns the contiguous
// positions [t * per, t * per + per).
__global__ void __launch_bounds__(kPlocSmallThreads) k_ploc_small(const uint32_t* cref, const float4* cbox,
                                                                   uint4* inodes, float4* iboxes, uint32_t* counts,
                                                                   BuildState* st, int round, uint32_t n) {
    extern __shared__ float psm[];
    float* lx = psm;
    float* ly = lx + kPlocSmall;
    float* lz = ly + kPlocSmall;
    float* hx = lz + kPlocSmall;
    float* hy = hx + kPlocSmall;
    float* hz = hy + kPlocSmall;
    uint32_t* ref = reinterpret_cast<uint32_t*>(hz + kPlocSmall);
    uint32_t* nbr = ref + kPlocSmall;
    uint32_t* keep = nbr + kPlocSmall;
    uint32_t* sz = keep + kPlocSmall;
    __shared__ uint32_t warp_sums[32];
    __shared__ uint32_t s_count, s_forced, s_merges, s_error;
    const uint32_t tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    uint32_t count = st->ploc_count[round & 1];
    if (count > kPlocSmall || count == 0u) {
        if (tid == 0) atomicOr(&st->error, 1u << RT_ERR_BAD_AS);
        return;
    }
    for (uint32_t t = tid; t < count; t += blockDim.x) {
        float4 a = __ldcg(&cbox[2 * (size_t)t]), b = __ldcg(&cbox[2 * (size_t)t + 1]);
        lx[t] = a.x; ly[t] = a.y; lz[t] = a.z;
        hx[t] = b.x; hy[t] = b.y; hz[t] = b.z;
        const uint32_t r = __ldcg(&cref[t]);
        ref[t] = r;
        sz[t] = ploc_size(counts, r);
    }
    if (tid == 0) {
        s_forced = 0u;
        s_merges = st->merge_counter;
        s_error = 0u;
    }
    __syncthreads();
    for (uint32_t guard = 0; count > 1u; guard++) {
        if (guard > kPlocSmall) {  // every round merges at least one pair: never reached
            if (tid == 0) atomicOr(&st->error, 1u << RT_ERR_BAD_AS);
            return;
        }
        const uint32_t per = (count + blockDim.x - 1) / blockDim.x;
        const uint32_t b0 = min(count, tid * per), b1 = min(count, b0 + per);
        const bool forced = s_forced != 0u;
        uint32_t g = 1;  // threads per cluster in the neighbour search
        while (g < 32u && count * g * 2u <= blockDim.x) g <<= 1;
        if (g > 1u) {
            const uint32_t i = tid / g, sub = tid % g;
            const bool on = i < count;
            uint32_t best = i;
            float bd = INFINITY;
            if (on && !forced) {
                for (uint32_t k = sub; k <= 2u * kPlocRadius; k += g) {
                    const int64_t j = (int64_t)i - kPlocRadius + k;
                    if (k == (uint32_t)kPlocRadius || j < 0 || j >= (int64_t)count) continue;
                    float h = merged_half_area(lx[i], ly[i], lz[i], hx[i], hy[i], hz[i], lx[j], ly[j], lz[j], hx[j],
                                               hy[j], hz[j]);
                    if (h < bd) {
                        bd = h;
                        best = (uint32_t)j;
                    }
                }
            }
            // groups of g lanes are aligned inside the warp (g divides 32)
            for (uint32_t off = 1; off < g; off <<= 1) {
                const float ob = __shfl_xor_sync(0xFFFFFFFFu, bd, off);
                const uint32_t oj = __shfl_xor_sync(0xFFFFFFFFu, best, off);
                if (ob < bd || (ob == bd && oj < best && ob < INFINITY)) {
                    bd = ob;
                    best = oj;
                }
            }
            if (on && sub == 0u) nbr[i] = forced ? ((i ^ 1u) < count ? (i ^ 1u) : i) : best;
        } else {
            for (uint32_t i = b0; i < b1; i++) {
                uint32_t best = i;
                if (forced) {
                    best = (i ^ 1u) < count ? (i ^ 1u) : i;
                } else {
                    float bd = INFINITY;
                    const uint32_t j0 = i >= (uint32_t)kPlocRadius ? i - kPlocRadius : 0u;
                    const uint32_t j1 = min(count - 1u, i + kPlocRadius);
                    for (uint32_t j = j0; j <= j1; j++) {
                        if (j == i) continue;
                        float h = merged_half_area(lx[i], ly[i], lz[i], hx[i], hy[i], hz[i], lx[j], ly[j], lz[j],
                                                   hx[j], hy[j], hz[j]);
                        if (h < bd) {
                            bd = h;
                            best = j;
                        }
                    }
                }
                nbr[i] = best;
            }
        }
        __syncthreads();
        uint32_t local = 0;
        for (uint32_t i = b0; i < b1; i++) {
            const uint32_t j = nbr[i];
            uint32_t k = 1u;
            if (j != i && nbr[j] == i) {
                if (i < j) {
                    const float ax = fminf(lx[i], lx[j]), ay = fminf(ly[i], ly[j]), az = fminf(lz[i], lz[j]);
                    const float bx = fmaxf(hx[i], hx[j]), by = fmaxf(hy[i], hy[j]), bz = fmaxf(hz[i], hz[j]);
                    const uint32_t m = atomicAdd(&s_merges, 1u);
                    if (m + 2u <= n) {
                        const uint32_t id = n - 2u - m;
                        const uint32_t size = sz[i] + sz[j];
                        inodes[id] = make_uint4(ref[i], ref[j], 0u, 0u);
                        iboxes[2 * (size_t)id] = make_float4(ax, ay, az, 0.0f);
                        iboxes[2 * (size_t)id + 1] = make_float4(bx, by, bz, 0.0f);
                        counts[id] = size;
                        ref[i] = id;
                        sz[i] = size;
                    } else {
                        s_error = 1u;
                    }
                    lx[i] = ax; ly[i] = ay; lz[i] = az;
                    hx[i] = bx; hy[i] = by; hz[i] = bz;
                } else {
                    k = 0u;
                }
            }
            keep[i] = k;
            local += k;
        }
        // block-wide exclusive scan of the per-thread survivor counts
        uint32_t incl = local;
        for (int off = 1; off < 32; off <<= 1) {
            uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
            if (lane >= (uint32_t)off) incl += o;
        }
        __syncthreads();  // merges done (other threads read ref / box / size of their pair above)
        if (lane == 31u) warp_sums[warp] = incl;
        __syncthreads();
        if (warp == 0) {
            uint32_t w = warp_sums[lane], wi = w;
            for (int off = 1; off < 32; off <<= 1) {
                uint32_t o = __shfl_up_sync(0xFFFFFFFFu, wi, off);
                if (lane >= (uint32_t)off) wi += o;
            }
            warp_sums[lane] = wi - w;
            if (lane == 31u) s_count = wi;
        }
        __syncthreads();
        // in-order compaction through registers
        uint32_t pos = warp_sums[warp] + incl - local;
        float v[kPlocSmallPer][6];
        uint32_t rr[kPlocSmallPer], ss[kPlocSmallPer], kk[kPlocSmallPer];
#pragma unroll
        for (uint32_t q = 0; q < kPlocSmallPer; q++) {
            const uint32_t i = b0 + q;
            kk[q] = i < b1 ? keep[i] : 0u;
            if (i < b1) {
                v[q][0] = lx[i]; v[q][1] = ly[i]; v[q][2] = lz[i];
                v[q][3] = hx[i]; v[q][4] = hy[i]; v[q][5] = hz[i];
                rr[q] = ref[i];
                ss[q] = sz[i];
            }
        }
        __syncthreads();
#pragma unroll
        for (uint32_t q = 0; q < kPlocSmallPer; q++) {
            if (!kk[q]) continue;
            lx[pos] = v[q][0]; ly[pos] = v[q][1]; lz[pos] = v[q][2];
            hx[pos] = v[q][3]; hy[pos] = v[q][4]; hz[pos] = v[q][5];
            ref[pos] = rr[q];
            sz[pos] = ss[q];
            pos++;
        }
        const uint32_t next = s_count;
        __syncthreads();
        if (tid == 0) s_forced = next == count ? 1u : 0u;
        count = next;
        __syncthreads();
    }
    if (tid == 0) {
        st->merge_counter = s_merges;
        if (s_error) atomicOr(&st->error, 1u << RT_ERR_BAD_AS);
    }
}

// ---- collapse to 8-wide -------------------------------------------------------
struct CollapseCtx {
    const uint4* inodes;
    const float4* iboxes;
    const float4* sboxes;
    WideNode* nodes;
    uint32_t* parents;   // may be null
    BuildState* st;
    const uint32_t* counts;  // primitives under each internal node (PLOC); null = the Karras ranges
    uint32_t* perm;          // final primitive order: position -> Morton-sorted position
    uint32_t leaf_max;
    uint32_t width;      // children per node: 8, or 4 (RT_BUILD_EXT_NODE_WIDTH_4)
    uint32_t max_nodes;
    uint32_t n;          // primitives
};

// Primitives under a binary reference.
__device__ __forceinline__ uint32_t ref_count(const CollapseCtx& c, uint32_t r) {
    if (r & kLeafBit) return 1u;
    if (c.counts) return c.counts[r];
    uint4 nd = c.inodes[r];
    return nd.w - nd.z + 1u;
}

// A leaf child's primitives take positions [first, first + count) of the
// final order, left to right.  The subtree holds at most leaf_max (<= 8)
// primitives, so the walk needs a few stack entries.
__device__ void write_leaf_order(const CollapseCtx& c, uint32_t r, uint32_t first) {
    uint32_t stack[8];
    int sp = 0;
    stack[sp++] = r;
    uint32_t k = first;
    while (sp > 0) {
        const uint32_t x = stack[--sp];
        if (x & kLeafBit) {
            if (k < c.n) c.perm[k++] = x & ~kLeafBit;
            continue;
        }
        if (x + 1u >= c.n || sp + 2 > 8) {
            atomicOr(&c.st->error, 1u << RT_ERR_BAD_AS);
            return;
        }
        const uint4 nd = c.inodes[x];
        stack[sp++] = nd.y;
        stack[sp++] = nd.x;
    }
}
__device__ __forceinline__ void ref_box(const CollapseCtx& c, uint32_t r, float lo[3], float hi[3]) {
    const float4* b = (r & kLeafBit) ? c.sboxes : c.iboxes;
    size_t i = r & ~kLeafBit;
    float4 l = b[2 * i], h = b[2 * i + 1];
    lo[0] = l.x; lo[1] = l.y; lo[2] = l.z;
    hi[0] = h.x; hi[1] = h.y; hi[2] = h.z;
}
__device__ __forceinline__ float half_area(const float lo[3], const float hi[3]) {
    float dx = fmaxf(hi[0] - lo[0], 0.0f), dy = fmaxf(hi[1] - lo[1], 0.0f), dz = fmaxf(hi[2] - lo[2], 0.0f);
    return dx * dy + dy * dz + dz * dx;
}

__device__ void write_node(WideNode* dst, const float lo[8][3], const float hi[8][3], const uint32_t ref[8],
                           const uint32_t meta[8], int cnt) {
    WideNode nd;
    for (int k = 0; k < 8; k++) {
        bool v = k < cnt && meta[k] != 0u;
        nd.lox[k] = v ? lo[k][0] : 0.0f;
        nd.loy[k] = v ? lo[k][1] : 0.0f;
        nd.loz[k] = v ? lo[k][2] : 0.0f;
        nd.hix[k] = v ? hi[k][0] : 0.0f;
        nd.hiy[k] = v ? hi[k][1] : 0.0f;
        nd.hiz[k] = v ? hi[k][2] : 0.0f;
        // the traversal's stack entry: node index, or leaf | (count-1) << 28 | first
        nd.child_ref[k] = !v ? kChildEmpty
                             : (meta[k] == kMetaInternal ? ref[k] : (kChildLeaf | ((meta[k] - 1u) << 28) | ref[k]));
    }
    uint32_t m0 = 0, m1 = 0;
    for (int k = 0; k < 4; k++) {
        m0 |= (k < cnt ? meta[k] : 0u) << (8 * k);
        m1 |= (k + 4 < cnt ? meta[k + 4] : 0u) << (8 * k);
    }
    nd.meta[0] = m0;
    nd.meta[1] = m1;
    for (int k = 0; k < 6; k++) nd._pad[k] = 0;
    const uint4* s = reinterpret_cast<const uint4*>(&nd);
    uint4* d = reinterpret_cast<uint4*>(dst);
    for (int k = 0; k < 16; k++) d[k] = s[k];
}

// A binary reference is in range: leaf < n, internal < n - 1.
__device__ __forceinline__ bool ref_ok(const CollapseCtx& c, uint32_t r) {
    return (r & kLeafBit) ? ((r & ~kLeafBit) < c.n) : (r + 1u < c.n);
}

// One wide node from binary node bref; its primitives take positions
// [first, first + count) of the final order.
template <class Push>
__device__ void collapse_task(const CollapseCtx& c, uint32_t bref, uint32_t slot, uint32_t depth, uint32_t first,
                              Push push) {
    // Each child's box, size and surface area are loaded once, when it joins
    // the node: choosing the child to open reads no memory, and opening one
    // loads only its two children (independent loads).  area < 0: the child
    // cannot be opened (a leaf, or a subtree small enough to be one).
    uint32_t refs[8], size[8];
    float lo[8][3], hi[8][3], area[8];
    int cnt = 0;
    if (bref + 1u >= c.n || slot >= c.max_nodes) {
        atomicOr(&c.st->error, 1u << RT_ERR_BAD_AS);
        return;
    }
    auto load = [&](int k, uint32_t r) {
        refs[k] = r;
        ref_box(c, r, lo[k], hi[k]);
        size[k] = ref_count(c, r);
        area[k] = (!(r & kLeafBit) && size[k] > c.leaf_max) ? half_area(lo[k], hi[k]) : -1.0f;
    };
    const uint4 root = c.inodes[bref];
    if (ref_ok(c, root.x) && ref_ok(c, root.y)) {
        load(0, root.x);
        load(1, root.y);
        cnt = 2;
    }
    while (cnt >= 2 && cnt < (int)c.width) {
        int best = -1;
        float best_area = -1.0f;
        for (int k = 0; k < cnt; k++) {
            if (area[k] > best_area) {
                best_area = area[k];
                best = k;
            }
        }
        if (best < 0) break;
        const uint4 nd = c.inodes[refs[best]];
        if (!ref_ok(c, nd.x) || !ref_ok(c, nd.y)) {
            cnt = 0;
            break;
        }
        load(best, nd.x);
        load(cnt, nd.y);
        cnt++;
    }
    if (cnt == 0) atomicOr(&c.st->error, 1u << RT_ERR_BAD_AS);  // malformed hierarchy: empty node
    uint32_t ref[8], meta[8];
    uint32_t at = first;  // the children's primitives follow each other in slot order
    for (int k = 0; k < cnt; k++) {
        const uint32_t r = refs[k];
        const uint32_t sz = size[k];
        const uint32_t f = at;
        at += sz;
        if (sz == 0u || at > c.n) {  // malformed hierarchy
            atomicOr(&c.st->error, 1u << RT_ERR_BAD_AS);
            meta[k] = 0;
            ref[k] = 0;
            continue;
        }
        if ((r & kLeafBit) || sz <= c.leaf_max) {
            meta[k] = sz;
            ref[k] = f;
            write_leaf_order(c, r, f);
        } else {
            uint32_t cs = atomicAdd(&c.st->node_counter, 1u);
            if (cs >= c.max_nodes) {
                atomicOr(&c.st->error, 1u << RT_ERR_TOO_LARGE);
                meta[k] = 0;
                ref[k] = 0;
                continue;
            }
            meta[k] = kMetaInternal;
            ref[k] = cs;
            if (c.parents) c.parents[cs] = slot;
            push(r, cs, depth + 1, f);
        }
    }
    write_node(&c.nodes[slot], lo, hi, ref, meta, cnt);
    atomicMax(&c.st->depth, depth + 1);
}

// A collapse task waiting for its level: the binary node, the wide node's
// depth and its first primitive position, stashed in the first 16 bytes of
// the wide-node slot it will write (nothing else writes that slot before).
__device__ __forceinline__ void stash_task(const CollapseCtx& c, uint32_t slot, uint32_t bref, uint32_t depth,
                                           uint32_t first) {
    *reinterpret_cast<uint4*>(&c.nodes[slot]) = make_uint4(bref, depth, first, 0u);
}
__device__ __forceinline__ uint4 stashed_task(const CollapseCtx& c, uint32_t slot) {
    return *reinterpret_cast<const uint4*>(&c.nodes[slot]);
}

// Root wide node: a single leaf for n <= leaf_max, else the level-0 task.
__global__ void k_collapse_root(CollapseCtx c, uint32_t n) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    if (c.parents) c.parents[0] = kNone;
    if (n == 0 || n <= c.leaf_max) {
        float lo[8][3], hi[8][3];
        uint32_t ref[8] = {0}, meta[8] = {0};
        int cnt = 0;
        if (n > 0) {
            for (int k = 0; k < 3; k++) {
                lo[0][k] = o2f(c.st->bb[k]);
                hi[0][k] = o2f(c.st->bb[3 + k]);
            }
            ref[0] = 0;
            meta[0] = n;
            cnt = 1;
            for (uint32_t i = 0; i < n; i++) c.perm[i] = i;
        }
        write_node(&c.nodes[0], lo, hi, ref, meta, cnt);
        return;
    }
    stash_task(c, 0, 0u, 0u, 0u);
    c.st->level_lo = 0;
    c.st->level_hi = 1;
}

// One breadth-first level: the tasks stashed in slots [level_lo, level_hi).
// Every internal child gets the next slot from node_counter and its task is
// stashed there, so the slots this launch allocates are the next level.  The
// block that finishes last publishes that range (a count of finished blocks;
// no block waits for another).
__global__ void k_collapse_level(CollapseCtx c) {
    const uint32_t lo = c.st->level_lo, hi = c.st->level_hi;
    for (uint32_t t = lo + blockIdx.x * blockDim.x + threadIdx.x; t < hi; t += gridDim.x * blockDim.x) {
        const uint4 task = stashed_task(c, t);
        collapse_task(c, task.x, t, task.y, task.z, [&](uint32_t r, uint32_t s, uint32_t d, uint32_t f) {
            stash_task(c, s, r, d, f);
        });
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&c.st->level_blocks_done, 1u) == gridDim.x - 1) {
            __threadfence();
            const uint32_t allocated = atomicAdd(&c.st->node_counter, 0u);
            c.st->level_lo = hi;
            c.st->level_hi = min(allocated, c.max_nodes);
            c.st->level_blocks_done = 0;
        }
    }
}

// The levels below the last breadth-first launch: each stashed task of the
// last range is collapsed depth-first by one thread.
__global__ void k_collapse_tail(CollapseCtx c) {
    const uint32_t lo = c.st->level_lo, hi = c.st->level_hi;
    for (uint32_t t = lo + blockIdx.x * blockDim.x + threadIdx.x; t < hi; t += gridDim.x * blockDim.x) {
        uint2 stack[kTailStack];
        uint2 dstack[kTailStack];   // depth, first primitive position
        int sp = 0;
        const uint4 task = stashed_task(c, t);
        stack[sp] = make_uint2(task.x, t);
        dstack[sp++] = make_uint2(task.y, task.z);
        while (sp > 0) {
            --sp;
            uint2 e = stack[sp];
            uint2 d = dstack[sp];
            collapse_task(c, e.x, e.y, d.x, d.y, [&](uint32_t r, uint32_t s, uint32_t dd, uint32_t f) {
                if (sp < kTailStack) {
                    stack[sp] = make_uint2(r, s);
                    dstack[sp++] = make_uint2(dd, f);
                } else {
                    atomicOr(&c.st->error, 1u << RT_ERR_STACK_OVERFLOW);
                }
            });
        }
    }
}

// ---- primitive records ----------------------------------------------------------
__global__ void k_write_tris(const __grid_constant__ BlasInput in, const uint32_t* vals, const uint32_t* perm,
                             TriRecord* tris, BuildState* st) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool here = i < in.n;  // every thread takes part in the block's reductions below
    uint32_t p = here ? vals[min(perm[i], in.n - 1u)] : 0u;
    int g = 0;
    uint32_t prim = 0;
    float v[3][3];
    bool ok = here && fetch_triangle(in, p, &g, &prim, v);
    if (!ok) {
        float qn = __int_as_float(0x7FC00000);
        for (int c = 0; c < 3; c++) v[c][0] = v[c][1] = v[c][2] = qn;
    }
    // bounding sphere radius: the largest vertex distance from the bounds
    // centre over the triangles that have a box (finite vertices)
    uint32_t rb = 0;
    if (ok && finite3(v[0]) && finite3(v[1]) && finite3(v[2])) {
        const float c[3] = {bounds_center(st, 0), bounds_center(st, 1), bounds_center(st, 2)};
        float r = fmaxf(fmaxf(distance_ru(v[0], c), distance_ru(v[1], c)), distance_ru(v[2], c));
        rb = __float_as_uint(r);  // an overflow (+inf) turns the sphere off
    }
    // the radius and the 14-DOP's extreme projections (sums of +-coordinates,
    // rounded up for the maxima and down for the minima) are reduced over the
    // warp, then over the block, and each block makes one atomic per value
    __shared__ uint32_t red[32][15];  // [warp][radius, 7 maxima, 7 minima]
    const uint32_t w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    const bool leader = (threadIdx.x & 31u) == 0u;
    rb = __reduce_max_sync(0xFFFFFFFFu, rb);
    if (leader) red[w][0] = rb;
    const bool valid = ok && finite3(v[0]) && finite3(v[1]) && finite3(v[2]);
#pragma unroll
    for (int k = 0; k < 7; k++) {
        uint32_t hi = 0u, lo = 0xFFFFFFFFu;
        if (valid) {
            float ph = -INFINITY, pl = INFINITY;
            for (int c = 0; c < 3; c++) {
                float u = 0.0f, d = 0.0f;
                for (int a = 0; a < 3; a++) {
                    const float x = kDopAxis[k][a] > 0 ? v[c][a] : (kDopAxis[k][a] < 0 ? -v[c][a] : 0.0f);
                    u = __fadd_ru(u, x);
                    d = __fadd_rd(d, x);
                }
                ph = fmaxf(ph, u);
                pl = fminf(pl, d);
            }
            hi = f2o(ph);
            lo = f2o(pl);
        }
        hi = __reduce_max_sync(0xFFFFFFFFu, hi);
        lo = __reduce_min_sync(0xFFFFFFFFu, lo);
        if (leader) {
            red[w][1 + k] = hi;
            red[w][8 + k] = lo;
        }
    }
    __syncthreads();
    if (threadIdx.x < 15) {
        const int k = threadIdx.x;
        uint32_t r = red[0][k];
        for (uint32_t j = 1; j < nw; j++) r = k < 8 ? max(r, red[j][k]) : min(r, red[j][k]);
        if (k == 0) {
            if (r) atomicMax(&st->radius_bits, r);
        } else if (k < 8) {
            if (r != 0u) atomicMax(&st->dop_hi[k - 1], r);  // 0: no valid triangle in the block
        } else if (r != 0xFFFFFFFFu) {
            atomicMin(&st->dop_lo[k - 8], r);
        }
    }
    if (!here) return;
    uint32_t flags = (in.g[g].flags & RT_GEOMETRY_OPAQUE) ? 1u : 0u;
    TriRecord r;
    r.v0 = make_float4(v[0][0], v[0][1], v[0][2], __uint_as_float(prim));
    r.v1 = make_float4(v[1][0], v[1][1], v[1][2], __uint_as_float((uint32_t)g));
    r.v2 = make_float4(v[2][0], v[2][1], v[2][2], __uint_as_float(flags));
    tris[i] = r;
}

// The 14-DOP's vertices: every triple of its 14 planes solved in double, one
// thread per triple over kDopBlocks blocks, kept when the point satisfies all
// 14 planes (with a relative tolerance).  The block that finishes last (a
// count of finished blocks: no block waits) gathers the points in triple
// order and merges duplicates: a point within the tolerance of an earlier one
// is dropped, one thread per point (a serial pass over all pairs in double
// took hundreds of microseconds at this part's FP64 rate).  More than
// kDopMaxVertices distinct points (only through rounding) or a non-finite
// projection leave the header's dop_count at 0.  The vertices' float rounding
// (a few 1e-8 relative) is covered by the instance box padding (1e-5
// relative).
__global__ void __launch_bounds__(kDopThreads) k_dop_vertices(AsHeader* h, BuildState* st) {
    __shared__ double pn[14][3], ph[14];
    __shared__ double cand[kDopTriples][3];  // the points found, in triple order (last block)
    __shared__ float candf[kDopTriples][3];
    __shared__ uint8_t dup[kDopTriples];      // 1: within the tolerance of an earlier point
    __shared__ uint32_t warp_sums[kDopThreads / 32];
    __shared__ uint32_t npts;
    __shared__ bool ok;
    __shared__ uint32_t last;
    const int t = blockIdx.x * kDopThreads + threadIdx.x;
    if (threadIdx.x == 0) {
        ok = true;
        for (int k = 0; k < 7; k++) {
            const float hi = o2f(st->dop_hi[k]), lo = o2f(st->dop_lo[k]);
            if (!(lo <= hi) || !(fabsf(hi) <= FLT_MAX) || !(fabsf(lo) <= FLT_MAX)) ok = false;
            for (int a = 0; a < 3; a++) {
                pn[2 * k][a] = (double)kDopAxis[k][a];
                pn[2 * k + 1][a] = -(double)kDopAxis[k][a];
            }
            ph[2 * k] = (double)hi;
            ph[2 * k + 1] = -(double)lo;
        }
        if (blockIdx.x == 0) h->dop_count = 0;
    }
    __syncthreads();
    if (!ok) return;  // the same in every block
    double scale = 1e-30;
    for (int j = 0; j < 14; j++) scale = fmax(scale, fabs(ph[j]));
    if (t < kDopTriples) {
        int a = 0, b = 1, c = 2;
        for (int idx = 0; idx < t; idx++) {  // the t-th triple a < b < c in lexicographic order
            if (++c == 14) {
                if (++b == 13) {
                    ++a;
                    b = a + 1;
                }
                c = b + 1;
            }
        }
        uint32_t found = 0;
        // Cramer's rule on the rows pn[a], pn[b], pn[c]
        const double* A = pn[a];
        const double* B = pn[b];
        const double* C = pn[c];
        const double det = A[0] * (B[1] * C[2] - B[2] * C[1]) - A[1] * (B[0] * C[2] - B[2] * C[0]) +
                           A[2] * (B[0] * C[1] - B[1] * C[0]);
        if (fabs(det) >= 1e-9) {
            const double x = (ph[a] * (B[1] * C[2] - B[2] * C[1]) - A[1] * (ph[b] * C[2] - B[2] * ph[c]) +
                              A[2] * (ph[b] * C[1] - B[1] * ph[c])) / det;
            const double y = (A[0] * (ph[b] * C[2] - B[2] * ph[c]) - ph[a] * (B[0] * C[2] - B[2] * C[0]) +
                              A[2] * (B[0] * ph[c] - ph[b] * C[0])) / det;
            const double z = (A[0] * (B[1] * ph[c] - ph[b] * C[1]) - A[1] * (B[0] * ph[c] - ph[b] * C[0]) +
                              ph[a] * (B[0] * C[1] - B[1] * C[0])) / det;
            bool inside = true;
            for (int j = 0; j < 14 && inside; j++)
                inside = pn[j][0] * x + pn[j][1] * y + pn[j][2] * z <= ph[j] + 1e-9 * scale;
            if (inside) {
                st->dop_cand[t][0] = x;
                st->dop_cand[t][1] = y;
                st->dop_cand[t][2] = z;
                found = 1;
            }
        }
        st->dop_state[t] = found;
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) last = atomicAdd(&st->dop_blocks_done, 1u) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (!last) return;
    __threadfence();
    // the points, in triple order (each thread takes kDopPer consecutive triples)
    const int t0 = threadIdx.x * kDopPer;
    uint32_t mine = 0;
    for (int k = 0; k < kDopPer; k++)
        if (t0 + k < kDopTriples && __ldcg(&st->dop_state[t0 + k])) mine++;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    uint32_t incl = mine;
    for (int off = 1; off < 32; off <<= 1) {
        const uint32_t o = __shfl_up_sync(0xFFFFFFFFu, incl, off);
        if (lane >= (uint32_t)off) incl += o;
    }
    if (lane == 31u) warp_sums[warp] = incl;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t run = 0;
        for (uint32_t w = 0; w < kDopThreads / 32; w++) {
            const uint32_t v = warp_sums[w];
            warp_sums[w] = run;
            run += v;
        }
        npts = run;
    }
    __syncthreads();
    uint32_t at = warp_sums[warp] + incl - mine;
    for (int k = 0; k < kDopPer; k++) {
        const int i = t0 + k;
        if (i < kDopTriples && __ldcg(&st->dop_state[i])) {
            for (int a = 0; a < 3; a++) {
                cand[at][a] = __ldcg(&st->dop_cand[i][a]);
                candf[at][a] = (float)cand[at][a];
            }
            dup[at] = 0;
            at++;
        }
    }
    __syncthreads();
    // A pair is a duplicate when every coordinate differs by at most 1e-7
    // scale (in double).  The float copies screen the pairs first: every
    // coordinate is within scale (1 + 1e-9) (the axis planes bound it), so
    // rounding to float moves a difference by at most 2^-23 scale, and a
    // pair whose float difference exceeds 4e-7 scale cannot pass the double
    // test.  Only the few pairs that pass the screen use the slow FP64 pipe.
    const double tol = 1e-7 * scale;
    const float tolf = 4e-7f * (float)scale;
    for (uint32_t i = threadIdx.x; i < npts; i += kDopThreads) {
        bool d = false;
        for (uint32_t j = 0; j < i && !d; j++) {
            if (fabsf(candf[i][0] - candf[j][0]) > tolf || fabsf(candf[i][1] - candf[j][1]) > tolf ||
                fabsf(candf[i][2] - candf[j][2]) > tolf)
                continue;
            d = fabs(cand[i][0] - cand[j][0]) <= tol && fabs(cand[i][1] - cand[j][1]) <= tol &&
                fabs(cand[i][2] - cand[j][2]) <= tol;
        }
        dup[i] = d ? 1 : 0;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    st->dop_blocks_done = 0;
    uint32_t nv = 0;
    for (uint32_t i = 0; i < npts; i++) {
        if (dup[i]) continue;
        if (nv == kDopMaxVertices) return;  // more points than a 14-DOP has: leave it off
        for (int a = 0; a < 3; a++) h->dop_vertex[nv][a] = (float)cand[i][a];
        nv++;
    }
    if (nv >= 4u) h->dop_count = nv;
}

__global__ void k_write_insts(const InstRecord* temp, const uint32_t* vals, const uint32_t* perm, uint32_t n,
                              InstRecord* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = temp[vals[min(perm[i], n - 1u)]];
}

// ---- 8-bit quantised nodes ----------------------------------------------------
// Smallest biased exponent e (quantum s = 2^(e-127)) with ext <= 252 s and
// |floor(L / s)| + 512 < 2^24, so that the grid origin (floor(L/s) - 1) s and
// every decoded plane origin + q s (q <= 255) are exact floats.
// e_floor keeps a thin axis's quantum at least 2^-24 of the node's largest
// extent: a flat node (a ground plane's, zero extent on one axis) would
// otherwise get the smallest quantum there, whose scale times any ray's
// inverse direction falls below the fast test's range, and every ray would
// take the exact decode.  The box grows by a quarter of that quantum at most.
__device__ uint32_t quantum_exponent(float L, float ext, uint32_t e_floor) {
    uint32_t e = (__float_as_uint(ext / 252.0f) >> 23) & 0xFFu;
    uint32_t el = (__float_as_uint(fabsf(L)) >> 23) & 0xFFu;
    e = max(e, el > 23u ? el - 23u : 1u);
    e = max(e, e_floor);
    if (e < 1u) e = 1u;
    for (; e < 254u; e++) {
        float s = __uint_as_float(e << 23);
        if (ext > 252.0f * s) continue;
        float k = floorf(L / s);
        if (!(fabsf(k) < 16776704.0f)) continue;
        return e;
    }
    return 254u;
}

__global__ void k_quantize_nodes(const WideNode* in, const uint32_t* node_count, uint32_t max_nodes, QNode* out) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t count = min(*node_count, max_nodes);
    if (i >= count) return;
    const WideNode& nd = in[i];
    QNode q;
    float lo[3][8], hi[3][8];
    bool valid[8];
    float L[3] = {INFINITY, INFINITY, INFINITY}, H[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int k = 0; k < 8; k++) {
        q.child_ref[k] = nd.child_ref[k];
        lo[0][k] = nd.lox[k]; lo[1][k] = nd.loy[k]; lo[2][k] = nd.loz[k];
        hi[0][k] = nd.hix[k]; hi[1][k] = nd.hiy[k]; hi[2][k] = nd.hiz[k];
        valid[k] = nd.child_ref[k] != kChildEmpty;
        for (int a = 0; a < 3; a++) valid[k] = valid[k] && lo[a][k] <= hi[a][k] && fabsf(lo[a][k]) <= FLT_MAX &&
                                               fabsf(hi[a][k]) <= FLT_MAX;
        if (!valid[k]) continue;
        for (int a = 0; a < 3; a++) {
            L[a] = fminf(L[a], lo[a][k]);
            H[a] = fmaxf(H[a], hi[a][k]);
        }
    }
    uint8_t* qlo[3] = {q.qlo_x, q.qlo_y, q.qlo_z};
    uint8_t* qhi[3] = {q.qhi_x, q.qhi_y, q.qhi_z};
    float mext = 0.0f;  // the node's largest extent
    for (int a = 0; a < 3; a++)
        if (L[a] <= H[a]) mext = fmaxf(mext, __fsub_ru(H[a], L[a]));
    const uint32_t em = (__float_as_uint(mext) >> 23) & 0xFFu;
    const uint32_t e_floor = em > 24u ? em - 24u : 1u;
    for (int a = 0; a < 3; a++) {
        if (!(L[a] <= H[a])) {  // no valid child: any grid, every child empty
            q.origin[a] = 0.0f;
            q.exp[a] = 127u;
            for (int k = 0; k < 8; k++) { qlo[a][k] = 255u; qhi[a][k] = 0u; }
            continue;
        }
        float ext = __fsub_ru(H[a], L[a]);
        uint32_t e = quantum_exponent(L[a], ext, e_floor);
        float s = __uint_as_float(e << 23);
        float origin = (floorf(L[a] / s) - 1.0f) * s;
        q.origin[a] = origin;
        q.exp[a] = (uint8_t)e;
        for (int k = 0; k < 8; k++) {
            if (!valid[k]) { qlo[a][k] = 255u; qhi[a][k] = 0u; continue; }
            // outward to the grid with at least kQuantSlack of a quantum to
            // spare on each side (origin + ql s <= lo - slack s); the
            // division by the power of two s is exact
            float ql = floorf(__fsub_rd(__fsub_rd(lo[a][k], origin) / s, kQuantSlack));
            float qh = ceilf(__fadd_ru(__fsub_ru(hi[a][k], origin) / s, kQuantSlack));
            qlo[a][k] = (uint8_t)fminf(fmaxf(ql, 0.0f), 255.0f);
            qhi[a][k] = (uint8_t)fminf(fmaxf(qh, 0.0f), 255.0f);
        }
    }
    q._pad = 0;
    const uint4* src = reinterpret_cast<const uint4*>(&q);
    uint4* dst = reinterpret_cast<uint4*>(&out[i]);
    for (int w = 0; w < 6; w++) dst[w] = src[w];
}

struct HeaderStatic {
    uint32_t type, build_flags, prim_count, max_nodes, geometry_count, leaf_max, node_bytes;
    uint64_t total_size, nodes_offset, prims_offset, parents_offset;
    uint64_t prim_bytes;
};

__global__ void k_finalize(AsHeader* h, const BuildState* st, HeaderStatic hs) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    h->magic = kAsMagic;
    h->type = hs.type;
    h->build_flags = hs.build_flags;
    uint32_t err = st->error;
    uint32_t status = RT_OK;
    for (uint32_t e = 1; e < 32; e++)
        if (err & (1u << e)) {
            status = e;
            break;
        }
    h->status = status;
    uint32_t nc = st->node_counter;
    if (nc > hs.max_nodes) nc = hs.max_nodes;
    h->node_count = nc;
    h->prim_count = hs.prim_count;
    h->max_nodes = hs.max_nodes;
    h->node_bytes = hs.node_bytes;
    h->total_size = hs.total_size;
    h->nodes_offset = hs.nodes_offset;
    h->prims_offset = hs.prims_offset;
    h->parents_offset = hs.parents_offset;
    for (int k = 0; k < 3; k++) {
        float lo = o2f(st->bb[k]), hi = o2f(st->bb[3 + k]);
        if (hs.prim_count == 0 || !(lo <= hi)) {
            lo = INFINITY;
            hi = -INFINITY;
        }
        h->bounds_lo[k] = lo;
        h->bounds_hi[k] = hi;
    }
    h->geometry_count = hs.geometry_count;
    h->depth = st->depth;
    h->leaf_max = hs.leaf_max;
    h->blas_kinds = hs.type == kAsTypeTop ? st->blas_kinds : 0u;
    // the sphere is written only where every triangle's distance was taken
    const float rad = __uint_as_float(st->radius_bits);
    const bool sphere = hs.type == kAsTypeBottom && hs.prim_count > 0 && st->radius_bits != 0u && rad <= FLT_MAX;
    for (int k = 0; k < 3; k++) h->sphere_center[k] = sphere ? bounds_center(st, k) : 0.0f;
    h->sphere_radius = sphere ? __fmul_ru(rad, 1.0000010f) : 0.0f;
    uint64_t nodes_end = hs.nodes_offset + (uint64_t)nc * hs.node_bytes;
    uint64_t par = hs.parents_offset ? align_up(nodes_end, 256) : 0;
    uint64_t par_end = par ? par + (uint64_t)nc * 4 : nodes_end;
    h->compacted_size = align_up(align_up(par_end, 256) + hs.prim_count * hs.prim_bytes, 256);
}

// ---- TLAS refit ---------------------------------------------------------------------
__global__ void k_refit_insts(const RtAccelerationStructureInstance* inst, uint32_t n, AsHeader* h,
                              float4* sboxes, uint32_t* err) {
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    InstRecord* recs = reinterpret_cast<InstRecord*>(reinterpret_cast<uint8_t*>(h) + h->prims_offset);
    InstRecord rec = recs[i];
    uint32_t id = rec.instance_id;
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    uint32_t kinds = 0;
    if (id < n) {
        RtAccelerationStructureInstance r = inst[id];
        if (fill_instance(r, id, &rec, lo, hi, err)) kinds = blas_kind(rec.node_count);
    } else {
        rec.tri_count = 0;
        atomicOr(err, 1u << RT_ERR_INVALID);
    }
    // the kinds only grow here: a refit may add a BLAS kind, never drop one
    const uint32_t active = __activemask();
    kinds = __reduce_or_sync(active, kinds);
    if ((threadIdx.x & 31u) == (uint32_t)(__ffs(active) - 1) && kinds) atomicOr(&h->blas_kinds, kinds);
    recs[i] = rec;
    sboxes[2 * (size_t)i] = make_float4(lo[0], lo[1], lo[2], 0.0f);
    sboxes[2 * (size_t)i + 1] = make_float4(hi[0], hi[1], hi[2], 0.0f);
}

__device__ __forceinline__ int internal_children(const WideNode* nd) {
    uint32_t m0 = __ldcg(&nd->meta[0]), m1 = __ldcg(&nd->meta[1]);
    int c = 0;
    for (int k = 0; k < 8; k++) c += node_meta(m0, m1, k) == kMetaInternal;
    return c;
}

__global__ void k_refit_nodes(AsHeader* h, const float4* sboxes, uint32_t* counters, uint32_t cap, uint32_t* err) {
    uint32_t count = h->node_count;
    uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x;
    if (count > cap) {  // a TLAS of more instances than this update was given
        if (slot == 0) atomicOr(err, 1u << RT_ERR_INVALID);
        return;
    }
    if (slot >= count) return;
    uint8_t* base = reinterpret_cast<uint8_t*>(h);
    WideNode* nodes = reinterpret_cast<WideNode*>(base + h->nodes_offset);
    const uint32_t* parents = reinterpret_cast<const uint32_t*>(base + h->parents_offset);
    if (internal_children(&nodes[slot]) != 0) return;
    for (int guard = 0; guard < 64; guard++) {
        WideNode* nd = &nodes[slot];
        uint32_t m0 = __ldcg(&nd->meta[0]), m1 = __ldcg(&nd->meta[1]);
        float ulo[3] = {INFINITY, INFINITY, INFINITY}, uhi[3] = {-INFINITY, -INFINITY, -INFINITY};
        for (int k = 0; k < 8; k++) {
            uint32_t m = node_meta(m0, m1, k);
            if (m == 0) continue;
            uint32_t r = __ldcg(&nd->child_ref[k]);
            if (m != kMetaInternal) r &= 0x0FFFFFFFu;  // leaf: first primitive
            float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
            if (m == kMetaInternal ? r >= count : (m > 8u || r + m > h->prim_count)) {
                atomicOr(err, 1u << RT_ERR_BAD_AS);  // malformed child: leave its box empty
            } else if (m == kMetaInternal) {
                const WideNode* cn = &nodes[r];
                uint32_t c0 = __ldcg(&cn->meta[0]), c1 = __ldcg(&cn->meta[1]);
                for (int q = 0; q < 8; q++) {
                    if (node_meta(c0, c1, q) == 0) continue;
                    lo[0] = fminf(lo[0], __ldcg(&cn->lox[q]));
                    lo[1] = fminf(lo[1], __ldcg(&cn->loy[q]));
                    lo[2] = fminf(lo[2], __ldcg(&cn->loz[q]));
                    hi[0] = fmaxf(hi[0], __ldcg(&cn->hix[q]));
                    hi[1] = fmaxf(hi[1], __ldcg(&cn->hiy[q]));
                    hi[2] = fmaxf(hi[2], __ldcg(&cn->hiz[q]));
                }
            } else {
                for (uint32_t q = 0; q < m; q++) {
                    float4 l = sboxes[2 * (size_t)(r + q)], u = sboxes[2 * (size_t)(r + q) + 1];
                    lo[0] = fminf(lo[0], l.x);
                    lo[1] = fminf(lo[1], l.y);
                    lo[2] = fminf(lo[2], l.z);
                    hi[0] = fmaxf(hi[0], u.x);
                    hi[1] = fmaxf(hi[1], u.y);
                    hi[2] = fmaxf(hi[2], u.z);
                }
            }
            nd->lox[k] = lo[0];
            nd->loy[k] = lo[1];
            nd->loz[k] = lo[2];
            nd->hix[k] = hi[0];
            nd->hiy[k] = hi[1];
            nd->hiz[k] = hi[2];
            for (int a = 0; a < 3; a++) {
                ulo[a] = fminf(ulo[a], lo[a]);
                uhi[a] = fmaxf(uhi[a], hi[a]);
            }
        }
        __threadfence();
        uint32_t p = __ldcg(&parents[slot]);
        if (p == kNone || p >= count) {
            for (int a = 0; a < 3; a++) {
                h->bounds_lo[a] = ulo[a];
                h->bounds_hi[a] = uhi[a];
            }
            return;
        }
        int need = internal_children(&nodes[p]);
        if ((int)atomicAdd(&counters[p], 1u) + 1 < need) return;
        slot = p;
    }
    atomicOr(err, 1u << RT_ERR_STACK_OVERFLOW);
}

__global__ void k_refit_status(AsHeader* h, const uint32_t* err) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    uint32_t e = *err;
    for (uint32_t b = 1; b < 32; b++)
        if (e & (1u << b)) {
            h->status = b;
            return;
        }
}

// ---- AS copy (CLONE / COMPACT) ------------------------------------------------------
__global__ void k_as_copy(const uint8_t* src, uint8_t* dst, uint64_t dst_size, uint32_t mode) {
    const AsHeader* h = reinterpret_cast<const AsHeader*>(src);
    if (h->magic != kAsMagic) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && dst_size >= kHeaderBytes)
            reinterpret_cast<AsHeader*>(dst)->status = RT_ERR_BAD_AS;
        return;
    }
    uint64_t nodes_bytes = (uint64_t)h->node_count * h->node_bytes;
    uint64_t prim_bytes = (uint64_t)h->prim_count * (h->type == kAsTypeTop ? kInstBytes : kTriBytes);
    uint64_t par_bytes = h->parents_offset ? (uint64_t)h->node_count * 4 : 0;
    uint64_t need = mode == RT_COPY_MODE_COMPACT ? h->compacted_size : h->total_size;
    if (need > dst_size) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && dst_size >= kHeaderBytes) {
            AsHeader* d = reinterpret_cast<AsHeader*>(dst);
            d->magic = 0;
            d->status = RT_ERR_INVALID;
        }
        return;
    }
    uint64_t tid = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x, stride = (uint64_t)gridDim.x * blockDim.x;
    if (mode != RT_COPY_MODE_COMPACT) {
        // CLONE: the whole blob, position independent (offsets only).
        const uint4* s = reinterpret_cast<const uint4*>(src);
        uint4* d = reinterpret_cast<uint4*>(dst);
        uint64_t n16 = h->total_size / 16;
        for (uint64_t i = tid; i < n16; i += stride) d[i] = s[i];
        return;
    }
    // COMPACT: header | nodes[node_count] | parents[node_count] | prims
    uint64_t c_nodes = h->nodes_offset;
    uint64_t c_par = h->parents_offset ? align_up(c_nodes + nodes_bytes, 256) : 0;
    uint64_t c_prims = align_up(c_par ? c_par + par_bytes : c_nodes + nodes_bytes, 256);
    auto copy = [&](uint64_t so, uint64_t dof, uint64_t bytes) {
        const uint32_t* s = reinterpret_cast<const uint32_t*>(src + so);
        uint32_t* d = reinterpret_cast<uint32_t*>(dst + dof);
        for (uint64_t i = tid; i < bytes / 4; i += stride) d[i] = s[i];
    };
    copy(h->nodes_offset, c_nodes, nodes_bytes);
    if (par_bytes) copy(h->parents_offset, c_par, par_bytes);
    copy(h->prims_offset, c_prims, prim_bytes);
    if (tid == 0) {
        AsHeader hd = *h;
        hd.max_nodes = h->node_count;
        hd.parents_offset = c_par;
        hd.prims_offset = c_prims;
        hd.total_size = h->compacted_size;
        *reinterpret_cast<AsHeader*>(dst) = hd;
    }
}

inline uint32_t blocks_for(uint64_t n, uint32_t t) { return (uint32_t)((n + t - 1) / t); }
// Breadth-first collapse launches for n primitives and `width` children per
// node: ceil(log_width n) wide levels plus three for unbalanced trees; deeper
// subtrees finish depth-first.
inline int collapse_levels(uint32_t n, uint32_t width) {
    int l = 0;
    for (uint64_t c = 1; c < n; c *= width) l++;
    return std::min(std::max(l + 3, kMinLevels), kMaxLevels);
}

// PLOC hierarchy for builds that prefer trace speed (the reference's BLAS and
// TLAS flags); the Karras LBVH for PREFER_FAST_BUILD or no preference, and
// whenever one leaf holds everything.
inline bool uses_ploc(uint32_t n, bool top, uint32_t build_flags) {
    return (build_flags & RT_BUILD_PREFER_FAST_TRACE) && !(build_flags & RT_BUILD_PREFER_FAST_BUILD) &&
           n > (top ? kTlasLeafMax : kBlasLeafMax);
}

// Grid-wide PLOC rounds for n > kPlocSmall primitives: nearest-neighbour
// rounds to reach kPlocSmall clusters at the measured survival rates with a
// margin of 6, then pair rounds that reach it from n even if none merged.
inline void ploc_grid_rounds(uint32_t n, int* nn_rounds, int* pair_rounds) {
    const double x = 0.58 * (double)n / (double)kPlocSmall;
    *nn_rounds = 1 + (x > 1.0 ? (int)std::ceil(std::log(x) / -std::log(0.81)) : 0) + 6;
    *pair_rounds = 1 + (int)std::ceil(std::log2((double)n / (double)kPlocSmall));
}

}  // namespace

// ---------------------------------------------------------------------------
// Layouts
// ---------------------------------------------------------------------------
AsLayout AsLayout::make(uint32_t n, bool top, uint32_t build_flags) {
    const bool quantized = !top && (build_flags & RT_BUILD_QUANTIZED_NODES) != 0;
    AsLayout l;
    l.max_nodes = (uint32_t)max_wide_nodes(n, node_width(build_flags));
    l.node_bytes = (quantized && !top) ? kQNodeBytes : kNodeBytes;
    l.nodes = kHeaderBytes;
    uint64_t end = l.nodes + (uint64_t)l.max_nodes * l.node_bytes;
    if (top) {
        l.parents = align_up(end, 256);
        end = l.parents + (uint64_t)l.max_nodes * 4;
    } else {
        l.parents = 0;
    }
    l.prims = align_up(end, 256);
    l.total = align_up(l.prims + (uint64_t)n * (top ? kInstBytes : kTriBytes), 256);
    return l;
}

ScratchLayout ScratchLayout::make(uint32_t n, bool top, uint32_t build_flags) {
    const bool quantized = !top && (build_flags & RT_BUILD_QUANTIZED_NODES) != 0;
    const uint64_t cap = max_wide_nodes(n, node_width(build_flags));
    ScratchLayout s{};
    uint64_t nn = n ? n : 1;
    uint64_t ni = n > 1 ? n - 1 : 1;
    uint64_t o = 0;
    auto take = [&](uint64_t bytes) {
        uint64_t r = o;
        o = align_up(o + bytes, 256);
        return r;
    };
    s.sort_blocks = onesweep_partitions((uint32_t)nn);
    s.state = take(sizeof(BuildState));
    s.boxes = take(nn * 32);
    s.sboxes = take(nn * 32);
    s.keys0 = take(nn * 4);
    s.keys1 = take(nn * 4);
    s.vals0 = take(nn * 4);
    s.vals1 = take(nn * 4);
    s.hist = take(key_sort_state_bytes((uint32_t)nn));  // onesweep state + partition descriptors
    s.inodes = take(ni * 16);
    s.iboxes = take(ni * 32);
    s.iparent = take(ni * 4);
    s.lparent = take(nn * 4);
    s.flags = take(ni * 4);
    s.temp_inst = top ? take(nn * kInstBytes) : 0;
    s.fp32_nodes = quantized ? take(cap * kNodeBytes) : 0;
    s.perm = take(nn * 4);
    s.ploc = uses_ploc(n, top, build_flags);
    if (s.ploc) {
        s.ploc_ref0 = take(nn * 4);
        s.ploc_ref1 = take(nn * 4);
        s.ploc_box0 = take(nn * 32);
        s.ploc_box1 = take(nn * 32);
        s.ploc_nn = take(nn * 4);
        s.ploc_keep = take(nn * 4);
        s.ploc_scan = take(nn * 4);
        s.ploc_blk = take(((nn + kPlocScanBlock - 1) / kPlocScanBlock) * 4);
        s.counts = take(ni * 4);
    }
    s.refit_counters = 0;
    s.build_total = o;
    // update (refit) scratch: sorted boxes + one counter per node, sized for
    // either node width (the refit does not know which one the TLAS was built with)
    uint64_t u = 0;
    u = align_up(u + nn * 32, 256);
    s.refit_counters = u;
    u = align_up(u + max_wide_nodes(n, 4) * 4 + 4, 256);  // + error word
    s.update_total = u;
    return s;
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------
namespace {

cudaError_t build_common(uint32_t n, bool top, uint32_t build_flags, uint32_t geometry_count, uint8_t* dst,
                         uint8_t* scratch, cudaStream_t stream, const BlasInput* blas,
                         const RtAccelerationStructureInstance* inst) {
    const bool quantized = !top && (build_flags & RT_BUILD_QUANTIZED_NODES) != 0;
    ScratchLayout sl = ScratchLayout::make(n, top, build_flags);
    AsLayout al = AsLayout::make(n, top, build_flags);
    // quantised builds collapse into FP32 nodes in scratch, then quantise
    WideNode* fp32_nodes = quantized ? reinterpret_cast<WideNode*>(scratch + sl.fp32_nodes)
                                     : reinterpret_cast<WideNode*>(dst + al.nodes);
    BuildState* st = reinterpret_cast<BuildState*>(scratch + sl.state);
    float4* boxes = reinterpret_cast<float4*>(scratch + sl.boxes);
    float4* sboxes = reinterpret_cast<float4*>(scratch + sl.sboxes);
    uint32_t* keys[2] = {reinterpret_cast<uint32_t*>(scratch + sl.keys0), reinterpret_cast<uint32_t*>(scratch + sl.keys1)};
    uint32_t* vals[2] = {reinterpret_cast<uint32_t*>(scratch + sl.vals0), reinterpret_cast<uint32_t*>(scratch + sl.vals1)};
    uint32_t* hist = reinterpret_cast<uint32_t*>(scratch + sl.hist);
    uint4* inodes = reinterpret_cast<uint4*>(scratch + sl.inodes);
    float4* iboxes = reinterpret_cast<float4*>(scratch + sl.iboxes);
    uint32_t* iparent = reinterpret_cast<uint32_t*>(scratch + sl.iparent);
    uint32_t* lparent = reinterpret_cast<uint32_t*>(scratch + sl.lparent);
    uint32_t* flags = reinterpret_cast<uint32_t*>(scratch + sl.flags);
    InstRecord* temp = top ? reinterpret_cast<InstRecord*>(scratch + sl.temp_inst) : nullptr;
    const uint32_t T = 256;

    note_launch(), k_init_state<<<1, 32, 0, stream>>>(st);
    if (n > 0) {
        if (top) note_launch(), k_tlas_prims<<<blocks_for(n, T), T, 0, stream>>>(inst, n, boxes, temp, st);
        else note_launch(), k_blas_prims<<<blocks_for(n, T), T, 0, stream>>>(*blas, boxes, st);
        note_launch(), k_morton<<<blocks_for(n, T), T, 0, stream>>>(boxes, n, st, keys[0], vals[0]);
        // four stable digit passes: the sorted pairs land back in keys[0] / vals[0]
        const int cur = 0;
        if (cudaError_t e = launch_key_sort(keys[0], vals[0], keys[1], vals[1], n,
                                            reinterpret_cast<uint8_t*>(hist), &st->error, stream);
            e != cudaSuccess)
            return e;
        note_launch(), k_gather_boxes<<<blocks_for(n, T), T, 0, stream>>>(boxes, vals[cur], n, sboxes);
        uint32_t* counts = nullptr;
        if (sl.ploc) {
            counts = reinterpret_cast<uint32_t*>(scratch + sl.counts);
            uint32_t* cref[2] = {reinterpret_cast<uint32_t*>(scratch + sl.ploc_ref0),
                                 reinterpret_cast<uint32_t*>(scratch + sl.ploc_ref1)};
            float4* cbox[2] = {reinterpret_cast<float4*>(scratch + sl.ploc_box0),
                               reinterpret_cast<float4*>(scratch + sl.ploc_box1)};
            uint32_t* nnb = reinterpret_cast<uint32_t*>(scratch + sl.ploc_nn);
            uint32_t* keep = reinterpret_cast<uint32_t*>(scratch + sl.ploc_keep);
            uint32_t* scan = reinterpret_cast<uint32_t*>(scratch + sl.ploc_scan);
            uint32_t* blk = reinterpret_cast<uint32_t*>(scratch + sl.ploc_blk);
            note_launch(), k_ploc_init<<<blocks_for(n, T), T, 0, stream>>>(sboxes, n, cref[0], cbox[0], st);
            int round = 0;
            if (n > kPlocSmall) {
                // grid-wide rounds until kPlocSmall clusters remain (later rounds
                // do nothing); grids of at most one full SM load (152 SMs x 2048
                // threads), grid-stride beyond
                const uint32_t g = std::min<uint32_t>(blocks_for(n, kPlocChunk), 1216u);
                const uint32_t gm = std::min<uint32_t>(blocks_for(n, kPlocScanBlock), 304u);
                int nn_rounds = 0, pair_rounds = 0;
                ploc_grid_rounds(n, &nn_rounds, &pair_rounds);
                for (; round < nn_rounds + pair_rounds; round++) {
                    const int forced = round >= nn_rounds;
                    note_launch(), k_ploc_nn<<<g, kPlocChunk, 0, stream>>>(cbox[0], nnb, st, round, forced);
                    note_launch(), k_ploc_merge<<<gm, kPlocScanBlock, 0, stream>>>(
                        cref[0], cbox[0], nnb, cref[1], cbox[1], keep, scan, blk, inodes, iboxes, counts, st, round, n);
                    note_launch(), k_ploc_scatter<<<g, 256, 0, stream>>>(cref[1], cbox[1], keep, scan, blk, cref[0],
                                                                        cbox[0], st, round);
                }
            }
            // a per-device attribute: set on every build (a host-side call, no device work)
            const cudaError_t smem_ok =
                cudaFuncSetAttribute(k_ploc_small, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kPlocSmallSmem);
            if (smem_ok != cudaSuccess) return smem_ok;
            note_launch(), k_ploc_small<<<1, kPlocSmallThreads, kPlocSmallSmem, stream>>>(cref[0], cbox[0], inodes,
                                                                                        iboxes, counts, st, round, n);
        } else if (n > 1) {
            note_launch(), k_karras<<<blocks_for(n - 1, T), T, 0, stream>>>(keys[cur], n, inodes, iparent, lparent);
            cudaMemsetAsync(flags, 0, (size_t)(n - 1) * 4, stream);
            note_launch(), k_bottom_up<<<blocks_for(n, T), T, 0, stream>>>(inodes, lparent, iparent, sboxes, iboxes,
                                                                             flags, n, &st->error);
        }
        uint32_t* perm = reinterpret_cast<uint32_t*>(scratch + sl.perm);
        CollapseCtx cc;
        cc.inodes = inodes;
        cc.iboxes = iboxes;
        cc.sboxes = sboxes;
        cc.counts = counts;
        cc.perm = perm;
        cc.nodes = fp32_nodes;
        cc.parents = top ? reinterpret_cast<uint32_t*>(dst + al.parents) : nullptr;
        cc.st = st;
        cc.leaf_max = top ? kTlasLeafMax : kBlasLeafMax;
        cc.width = node_width(build_flags);
        cc.max_nodes = al.max_nodes;
        cc.n = n;
        note_launch(), k_collapse_root<<<1, 32, 0, stream>>>(cc, n);
        if (n > cc.leaf_max) {
            // level lv holds at most width^lv nodes: its grid covers 8^lv tasks
            // (grid-stride beyond kCollapseBlocks blocks)
            const int levels = collapse_levels(n, cc.width);
            uint64_t cap = 1;
            for (int lv = 0; lv < levels; lv++) {
                const uint32_t g = blocks_for(std::min<uint64_t>(cap, (uint64_t)kCollapseBlocks * 128), 128);
                note_launch(), k_collapse_level<<<g, 128, 0, stream>>>(cc);
                cap = std::min<uint64_t>(cap * 8, al.max_nodes);
            }
            const uint32_t g = blocks_for(std::min<uint64_t>(al.max_nodes, (uint64_t)kCollapseBlocks * 128), 128);
            note_launch(), k_collapse_tail<<<g, 128, 0, stream>>>(cc);
        }
        if (top) {
            note_launch(), k_write_insts<<<blocks_for(n, T), T, 0, stream>>>(temp, vals[cur], perm, n,
                                                              reinterpret_cast<InstRecord*>(dst + al.prims));
        } else {
            note_launch(), k_write_tris<<<blocks_for(n, T), T, 0, stream>>>(*blas, vals[cur], perm,
                                                                             reinterpret_cast<TriRecord*>(dst + al.prims),
                                                                             st);
            note_launch(), k_dop_vertices<<<kDopBlocks, kDopThreads, 0, stream>>>(reinterpret_cast<AsHeader*>(dst), st);
        }
    } else {
        CollapseCtx cc{};
        cc.nodes = fp32_nodes;
        cc.parents = top ? reinterpret_cast<uint32_t*>(dst + al.parents) : nullptr;
        cc.st = st;
        cc.leaf_max = 1;
        cc.width = node_width(build_flags);
        cc.max_nodes = al.max_nodes;
        cc.n = n;
        note_launch(), k_collapse_root<<<1, 32, 0, stream>>>(cc, 0);
    }
    if (quantized) {
        uint32_t g = blocks_for(al.max_nodes, 128);
        note_launch(), k_quantize_nodes<<<g, 128, 0, stream>>>(fp32_nodes, &st->node_counter, al.max_nodes,
                                                               reinterpret_cast<QNode*>(dst + al.nodes));
    }
    HeaderStatic hs;
    hs.node_bytes = al.node_bytes;
    hs.type = top ? kAsTypeTop : kAsTypeBottom;
    hs.build_flags = build_flags;
    hs.prim_count = n;
    hs.max_nodes = al.max_nodes;
    hs.geometry_count = geometry_count;
    hs.leaf_max = top ? kTlasLeafMax : kBlasLeafMax;
    hs.total_size = al.total;
    hs.nodes_offset = al.nodes;
    hs.prims_offset = al.prims;
    hs.parents_offset = al.parents;
    hs.prim_bytes = top ? kInstBytes : kTriBytes;
    note_launch(), k_finalize<<<1, 32, 0, stream>>>(reinterpret_cast<AsHeader*>(dst), st, hs);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_blas_build(const BlasInput& in, uint32_t build_flags, uint8_t* dst, uint8_t* scratch,
                              cudaStream_t stream) {
    return build_common(in.n, false, build_flags, in.geometry_count, dst, scratch, stream, &in, nullptr);
}

cudaError_t launch_tlas_build(const RtAccelerationStructureInstance* instances, uint32_t n, uint32_t build_flags,
                              uint8_t* dst, uint8_t* scratch, cudaStream_t stream) {
    return build_common(n, true, build_flags, 1, dst, scratch, stream, nullptr, instances);
}

cudaError_t launch_as_copy(const uint8_t* src, uint8_t* dst, uint64_t dst_size, uint32_t mode, cudaStream_t stream) {
    note_launch(), k_as_copy<<<1024, 256, 0, stream>>>(src, dst, dst_size, mode);
    return cudaGetLastError();
}

cudaError_t launch_tlas_update(const RtAccelerationStructureInstance* instances, uint32_t n, const uint8_t* src,
                               uint8_t* dst, uint64_t dst_size, uint8_t* scratch, cudaStream_t stream) {
    ScratchLayout sl = ScratchLayout::make(n, true);
    // node capacity of either node width: the grid and the counters cover any TLAS of n instances
    const uint32_t cap = (uint32_t)max_wide_nodes(n, 4);
    if (src != dst) {
        note_launch(), k_as_copy<<<1024, 256, 0, stream>>>(src, dst, dst_size, RT_COPY_MODE_CLONE);
    }
    float4* sboxes = reinterpret_cast<float4*>(scratch);
    uint32_t* counters = reinterpret_cast<uint32_t*>(scratch + sl.refit_counters);
    // the error word lives after the counters
    uint32_t* err = counters + cap;
    cudaMemsetAsync(counters, 0, (size_t)cap * 4 + 4, stream);
    AsHeader* h = reinterpret_cast<AsHeader*>(dst);
    if (n > 0) note_launch(), k_refit_insts<<<blocks_for(n, 256), 256, 0, stream>>>(instances, n, h, sboxes, err);
    note_launch(), k_refit_nodes<<<blocks_for(cap, 128), 128, 0, stream>>>(h, sboxes, counters, cap, err);
    note_launch(), k_refit_status<<<1, 32, 0, stream>>>(h, err);
    return cudaGetLastError();
}

}  // namespace rt
