// rt_internal.h — host-side launch interface between the C ABI and kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "rt_device.cuh"

namespace rt {

// Counts every kernel this library launches (rt_kernel_launch_count).
void note_launch();

// kBlasKind* bits of every BLAS node format this process has built.  A BLAS
// blob only comes from a build here (or a copy of one), so a TLAS can only
// name these formats; the trace launchers pick their kernel variants by it.
void note_blas_kind(uint32_t kind);
uint32_t blas_kinds_built();

// Whether the context was created with RT_CTX_THREADSAFE.
bool ctx_is_threadsafe(const rt_ctx* ctx);

// One BLAS geometry as the build kernels see it.
struct BuildGeom {
    const float* pos;
    const uint32_t* idx;      // nullptr = non-indexed
    uint32_t stride_floats;
    uint32_t max_vertex;
    uint32_t prim_count;
    uint32_t flags;
    uint32_t prefix;          // first global primitive of this geometry
    uint32_t _pad;
};

struct BlasInput {
    BuildGeom g[RT_MAX_BLAS_GEOMETRIES];
    uint32_t geometry_count;
    uint32_t n;
};

// Byte offsets of the build scratch regions for n primitives.
struct ScratchLayout {
    uint64_t boxes, sboxes, keys0, keys1, vals0, vals1, hist, inodes, iboxes, iparent, lparent, flags;
    uint64_t state, temp_inst, refit_counters;
    uint64_t fp32_nodes;       // quantised builds: FP32 nodes before quantisation
    uint64_t perm;             // final primitive order
    // PLOC builds (RT_BUILD_PREFER_FAST_TRACE): cluster refs / boxes (two
    // buffers), neighbours, survivor flags and their scan, block totals,
    // primitives per internal node
    uint64_t ploc_ref0, ploc_ref1, ploc_box0, ploc_box1, ploc_nn, ploc_keep, ploc_scan, ploc_blk, counts;
    bool ploc;
    uint64_t build_total;
    uint64_t update_total;
    uint32_t sort_blocks;
    static ScratchLayout make(uint32_t n, bool top_level, uint32_t build_flags = 0);
};

// Byte offsets inside the AS blob.
struct AsLayout {
    uint64_t nodes, parents, prims, total;
    uint32_t max_nodes;
    uint32_t node_bytes;
    static AsLayout make(uint32_t n, bool top_level, uint32_t build_flags = 0);
};

constexpr uint32_t kMaxPrimitives = (1u << 28) - 1;  // leaf refs carry 28 bits

// The builder's key sort: n (key, value) pairs, stably by key (four 8-bit
// digit passes; one block for small n, else the onesweep scheme).  The
// result lands back in k0 / v0; k1 / v1 are the second buffers; `state` is
// key_sort_state_bytes(n) of scratch; a bounded wait that gave up sets bit
// RT_ERR_TIMEOUT in *error.
uint64_t key_sort_state_bytes(uint32_t n);
cudaError_t launch_key_sort(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, uint32_t n, uint8_t* state,
                            uint32_t* error, cudaStream_t stream);

cudaError_t launch_blas_build(const BlasInput& in, uint32_t build_flags, uint8_t* dst, uint8_t* scratch,
                              cudaStream_t stream);
cudaError_t launch_tlas_build(const RtAccelerationStructureInstance* instances, uint32_t n, uint32_t build_flags,
                              uint8_t* dst, uint8_t* scratch, cudaStream_t stream);
cudaError_t launch_tlas_update(const RtAccelerationStructureInstance* instances, uint32_t n, const uint8_t* src,
                               uint8_t* dst, uint64_t dst_size, uint8_t* scratch, cudaStream_t stream);
cudaError_t launch_as_copy(const uint8_t* src, uint8_t* dst, uint64_t dst_size, uint32_t mode, cudaStream_t stream);

// Trace entry points (rt_trace.cu).
// One scene of a wavefront launch (rt_cmd_trace_rays is a batch of one).
struct TraceScene {
    RtPushConstantBufferAddresses push;
    RtTraceRaysDesc desc;
    const RtTextureDesc* textures;  // device table of texture_count; nullptr = the context's table
    uint32_t texture_count;
    uint32_t _pad;
};
struct TraceBatch {
    const TraceScene* scenes;       // host array
    uint32_t count;
    uint32_t stats;                 // collect RtStats traversal counters
    RtShaderBindingTable sbt;
    const RtTextureDesc* ctx_textures;  // host copy of the context's RT_MAX_BOUND_IMAGES table
    RtStats* stats_dev;             // device
    uint32_t* status;               // device (same block)
    uint32_t kinds_built;           // blas_kinds_built() when the launch was recorded
    RtTraversalConfig config;       // launch shape of the traversal kernels
};
// Whether the traversal kernels are built for `c` (block size, shared stack depth, leaf_wait <= 32).
bool traversal_config_supported(const RtTraversalConfig& c);
// Bytes of the wavefront workspace a batch needs.
uint64_t trace_workspace_bytes(const TraceScene* scenes, uint32_t count);
// Bytes that hold the workspace of any batch of at most `count` scenes with
// at most `slots` ray slots (pixels padded to 8x4 tiles), `pixels` pixels
// and `shadow_rays` shadow rays in total.
uint64_t trace_workspace_bound(uint32_t count, uint64_t slots, uint64_t pixels, uint64_t shadow_rays);
// Sizes the context's wavefront workspace of `stream` to at least `bytes`
// now (stream-ordered), so that launches within that size never grow it.
cudaError_t ctx_reserve_workspace(rt_ctx* ctx, cudaStream_t stream, uint64_t bytes);

// CUDA events recorded after each kernel of a trace launch
// (RT_TRACE_FLAG_KERNEL_TIMINGS); kind[i] names the kernel that ended at ev[i].
enum : uint8_t { kKernStart = 0, kKernOther = 1, kKernClosest = 2, kKernShadow = 3, kKernShade = 4 };
struct KernelTimer {
    static constexpr int kMax = 160;
    cudaEvent_t ev[kMax];
    uint8_t kind[kMax];
    int n = 0;
    bool created = false;
};
cudaError_t launch_trace_batch(const TraceBatch& b, uint8_t* workspace, int num_sms, cudaStream_t stream,
                               KernelTimer* timer);

struct RayBufferLaunch {
    RtPushConstantBufferAddresses push;  // model_info may be 0
    RtShaderBindingTable sbt;
    RtTextureDesc textures[RT_MAX_BOUND_IMAGES];
    uint64_t tlas;
    const RtRay* rays;
    RtHit* hits;
    uint32_t count;
    uint32_t ray_flags;
    uint32_t cull_mask;
    uint32_t sbt_offset;
    uint32_t collect_stats;
    RtStats* stats;
    uint32_t* status;
    uint32_t* work;            // device fetch counter for this launch (zeroed by the launcher)
    uint32_t kinds_built;      // blas_kinds_built() when the launch was recorded
};
cudaError_t launch_trace_ray_buffer(const RayBufferLaunch& p, int num_sms, cudaStream_t stream);

cudaError_t launch_debug_eval(uint32_t fn, const float* in, float* out, uint32_t count, cudaStream_t stream);
cudaError_t upload_srgb_table();

}  // namespace rt
