// rt_api.cu — the C ABI declared in include/rtcore.h.
//
// Argument validation happens here, on the host, before anything is queued:
// a bad size, alignment or index returns RT_ERR_INVALID / RT_ERR_TOO_LARGE
// with a message in rt_last_error_string() and launches nothing.  Errors the
// device finds (a stack overflow, an out-of-range vertex index) are recorded
// in the AS header's status word or the context's statistics block.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "rt_error.h"
#include "rt_internal.h"

using namespace rt;

namespace {

constexpr uint32_t kWorkSlots = 256;

struct CtxDevice {
    RtStats stats;
    uint32_t work[kWorkSlots];
};

thread_local std::string g_last_error;
std::atomic<unsigned long long> g_kernel_launches{0};
std::atomic<uint32_t> g_blas_kinds{0};

int32_t fail(int32_t code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

}  // namespace

int32_t rt::report_error(int32_t code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return code;
}

namespace {

int32_t cuda_fail(cudaError_t e, const char* what) {
    return fail(e == cudaErrorMemoryAllocation ? RT_ERR_OOM : RT_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

bool aligned(uint64_t a, uint64_t n) { return (a % n) == 0; }

RtShaderBindingTable reference_sbt() {
    // src/main.rs:289-305: hit groups {any-hit 3, closest-hit 4 | 5 | 6}
    RtShaderBindingTable s;
    memset(&s, 0, sizeof s);
    s.hit_group_count = 3;
    s.hit_groups[0].closest_hit = RT_PROGRAM_CLOSEST_HIT_TEXTURED;
    s.hit_groups[1].closest_hit = RT_PROGRAM_CLOSEST_HIT_MIRROR;
    s.hit_groups[2].closest_hit = RT_PROGRAM_CLOSEST_HIT_PORTAL;
    for (int i = 0; i < 3; i++) s.hit_groups[i].any_hit = RT_PROGRAM_ANY_HIT_ALPHA_CLIP;
    return s;
}

int32_t check_sbt(const RtShaderBindingTable* sbt) {
    if (sbt->hit_group_count > RT_MAX_HIT_GROUPS)
        return fail(RT_ERR_INVALID, "hit_group_count %u > %u", sbt->hit_group_count, RT_MAX_HIT_GROUPS);
    for (uint32_t i = 0; i < sbt->hit_group_count; i++) {
        if (sbt->hit_groups[i].closest_hit > RT_PROGRAM_CLOSEST_HIT_PORTAL)
            return fail(RT_ERR_INVALID, "hit group %u: unknown closest-hit program %u", i, sbt->hit_groups[i].closest_hit);
        if (sbt->hit_groups[i].any_hit > RT_PROGRAM_ANY_HIT_ALPHA_CLIP)
            return fail(RT_ERR_INVALID, "hit group %u: unknown any-hit program %u", i, sbt->hit_groups[i].any_hit);
    }
    return RT_OK;
}

}  // namespace

void rt::note_launch() { g_kernel_launches.fetch_add(1, std::memory_order_relaxed); }
void rt::note_blas_kind(uint32_t kind) { g_blas_kinds.fetch_or(kind, std::memory_order_relaxed); }
uint32_t rt::blas_kinds_built() { return g_blas_kinds.load(std::memory_order_relaxed); }

// Wavefront workspace of one stream: grown stream-ordered (cudaFreeAsync /
// cudaMallocAsync on that stream), so launches on one stream reuse it
// safely and launches on different streams never share one.
struct Workspace {
    cudaStream_t stream;
    void* ptr;
    uint64_t size;
};

struct rt_ctx {
    uint32_t flags = 0;
    int device = 0;
    int num_sms = 1;
    RtTextureDesc textures[RT_MAX_BOUND_IMAGES];
    CtxDevice* dev = nullptr;
    std::atomic<uint32_t> work_slot{0};
    std::mutex mu;
    std::vector<Workspace> workspaces;
    KernelTimer timer;
    RtTraversalConfig traversal{128, 0, 20, 0};
    // rt_trace_ray_buffer_host: two streams and their device staging (rays, then hits)
    struct HostQuery {
        std::mutex mu;
        bool created = false;
        cudaStream_t st[2] = {nullptr, nullptr};
        cudaEvent_t start = nullptr, done[2] = {nullptr, nullptr};
        uint8_t* staging[2] = {nullptr, nullptr};
        uint64_t chunk = 0;  // rays each staging buffer holds
    } hq;
};

bool rt::ctx_is_threadsafe(const rt_ctx* c) { return c && (c->flags & RT_CTX_THREADSAFE) != 0; }

namespace {
bool stream_capturing(cudaStream_t s) {
    cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
    return cudaStreamIsCapturing(s, &st) == cudaSuccess && st != cudaStreamCaptureStatusNone;
}

// Returns cudaErrorStreamCaptureUnsupported when the workspace would have to
// grow while `s` is being captured into a CUDA graph (memory allocated in a
// capture belongs to the graph): trace once outside the capture first.
cudaError_t ctx_workspace(rt_ctx* c, cudaStream_t s, uint64_t need, uint8_t** out) {
    for (auto& w : c->workspaces) {
        if (w.stream != s) continue;
        if (w.size < need) {
            if (stream_capturing(s)) return cudaErrorStreamCaptureUnsupported;
            cudaError_t e = cudaFreeAsync(w.ptr, s);
            w.ptr = nullptr;
            w.size = 0;
            if (e == cudaSuccess) e = cudaMallocAsync(&w.ptr, need, s);
            if (e != cudaSuccess) return e;
            w.size = need;
        }
        *out = reinterpret_cast<uint8_t*>(w.ptr);
        return cudaSuccess;
    }
    if (stream_capturing(s)) return cudaErrorStreamCaptureUnsupported;
    Workspace w{s, nullptr, need};
    cudaError_t e = cudaMallocAsync(&w.ptr, need, s);
    if (e != cudaSuccess) return e;
    c->workspaces.push_back(w);
    *out = reinterpret_cast<uint8_t*>(w.ptr);
    return cudaSuccess;
}
}  // namespace

namespace {
struct MaybeLock {
    std::unique_lock<std::mutex> lk;
    explicit MaybeLock(rt_ctx* c) {
        if (c && (c->flags & RT_CTX_THREADSAFE)) lk = std::unique_lock<std::mutex>(c->mu);
    }
};
}  // namespace

cudaError_t rt::ctx_reserve_workspace(rt_ctx* ctx, cudaStream_t s, uint64_t bytes) {
    MaybeLock l(ctx);
    uint8_t* p = nullptr;
    return ctx_workspace(ctx, s, bytes, &p);
}

extern "C" {

RTCORE_API const char* rt_last_error_string(void) { return g_last_error.c_str(); }

RTCORE_API const char* rt_version_string(void) { return "rtcore-gb300 0.1 (sm_103a)"; }

RTCORE_API uint64_t rt_kernel_launch_count(void) { return g_kernel_launches.load(std::memory_order_relaxed); }

RTCORE_API int32_t rt_ctx_create(uint32_t flags, rt_ctx** out) {
    if (!out) return fail(RT_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (flags & ~RT_CTX_THREADSAFE) return fail(RT_ERR_INVALID, "unknown context flags 0x%x", flags);
    rt_ctx* c = new (std::nothrow) rt_ctx();
    if (!c) return fail(RT_ERR_OOM, "context allocation failed");
    c->flags = flags;
    memset(c->textures, 0, sizeof c->textures);
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
    if (e == cudaSuccess) e = cudaMalloc(&c->dev, sizeof(CtxDevice));
    if (e == cudaSuccess) e = cudaMemset(c->dev, 0, sizeof(CtxDevice));
    if (e == cudaSuccess) e = upload_srgb_table();
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        if (c->dev) cudaFree(c->dev);
        delete c;
        return cuda_fail(e, "rt_ctx_create");
    }
    *out = c;
    return RT_OK;
}

RTCORE_API int32_t rt_ctx_read_trace_timings(rt_ctx* ctx, RtTraceTimings* out) {
    if (!ctx || !out) return fail(RT_ERR_INVALID, "ctx or out is NULL");
    memset(out, 0, sizeof *out);
    const KernelTimer& t = ctx->timer;
    if (!t.created || t.n < 2) return fail(RT_ERR_INVALID, "no trace launch was timed (RT_TRACE_FLAG_KERNEL_TIMINGS)");
    cudaError_t e = cudaEventSynchronize(t.ev[t.n - 1]);
    if (e != cudaSuccess) return cuda_fail(e, "rt_ctx_read_trace_timings");
    for (int i = 1; i < t.n; i++) {
        float ms = 0.0f;
        e = cudaEventElapsedTime(&ms, t.ev[i - 1], t.ev[i]);
        if (e != cudaSuccess) return cuda_fail(e, "rt_ctx_read_trace_timings");
        out->total_ms += ms;
        switch (t.kind[i]) {
            case kKernClosest: out->closest_ms += ms; out->trace_ms += ms; out->trace_launches++; break;
            case kKernShadow: out->shadow_ms += ms; out->trace_ms += ms; out->trace_launches++; break;
            case kKernShade: out->shade_ms += ms; break;
            default: out->other_ms += ms; break;
        }
    }
    return RT_OK;
}

RTCORE_API int32_t rt_ctx_destroy(rt_ctx* ctx) {
    if (!ctx) return RT_OK;
    cudaDeviceSynchronize();
    if (ctx->timer.created)
        for (int i = 0; i < KernelTimer::kMax; i++) cudaEventDestroy(ctx->timer.ev[i]);
    for (auto& w : ctx->workspaces)
        if (w.ptr) cudaFree(w.ptr);
    if (ctx->hq.created) {
        for (int k = 0; k < 2; k++) {
            if (ctx->hq.staging[k]) cudaFree(ctx->hq.staging[k]);
            cudaEventDestroy(ctx->hq.done[k]);
            cudaStreamDestroy(ctx->hq.st[k]);
        }
        cudaEventDestroy(ctx->hq.start);
    }
    if (ctx->dev) cudaFree(ctx->dev);
    delete ctx;
    return RT_OK;
}

RTCORE_API int32_t rt_ctx_set_texture(rt_ctx* ctx, uint32_t index, const RtTextureDesc* desc) {
    if (!ctx || !desc) return fail(RT_ERR_INVALID, "ctx or desc is NULL");
    if (index >= RT_MAX_BOUND_IMAGES) return fail(RT_ERR_INVALID, "texture index %u >= %u", index, RT_MAX_BOUND_IMAGES);
    if (desc->address != 0) {
        uint32_t texel = 0;
        if (desc->format == RT_FORMAT_R8G8B8A8_UNORM || desc->format == RT_FORMAT_R8G8B8A8_SRGB) texel = 4;
        else if (desc->format == RT_FORMAT_R32G32B32A32_SFLOAT) texel = 16;
        else return fail(RT_ERR_UNSUPPORTED, "texture format %u", desc->format);
        if (desc->filter > RT_FILTER_LINEAR) return fail(RT_ERR_INVALID, "texture filter %u", desc->filter);
        if (desc->width == 0 || desc->height == 0) return fail(RT_ERR_INVALID, "empty texture");
        if ((uint64_t)desc->row_pitch < (uint64_t)desc->width * texel)
            return fail(RT_ERR_INVALID, "row_pitch %u < width*%u", desc->row_pitch, texel);
        if (!aligned(desc->address, texel) || !aligned(desc->row_pitch, texel))
            return fail(RT_ERR_INVALID, "texture address/pitch not %u-byte aligned", texel);
    }
    MaybeLock l(ctx);
    ctx->textures[index] = *desc;
    return RT_OK;
}

RTCORE_API int32_t rt_ctx_read_stats(rt_ctx* ctx, RtStats* out, int32_t reset, void* stream) {
    if (!ctx || !out) return fail(RT_ERR_INVALID, "ctx or out is NULL");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpy(out, &ctx->dev->stats, sizeof(RtStats), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && reset) e = cudaMemset(&ctx->dev->stats, 0, sizeof(RtStats));
    if (e != cudaSuccess) return cuda_fail(e, "rt_ctx_read_stats");
    return RT_OK;
}

// ---------------------------------------------------------------------------
// Acceleration structures
// ---------------------------------------------------------------------------
static int32_t blas_prim_count(const RtGeometryTriangles* g, uint32_t count, uint32_t* n_out) {
    if (count > RT_MAX_BLAS_GEOMETRIES)
        return fail(RT_ERR_TOO_LARGE, "geometry_count %u > %u", count, RT_MAX_BLAS_GEOMETRIES);
    if (count > 0 && !g) return fail(RT_ERR_INVALID, "geometries is NULL");
    uint64_t n = 0;
    for (uint32_t i = 0; i < count; i++) {
        if (g[i].primitive_count > 0) {
            if (g[i].vertex_address == 0) return fail(RT_ERR_INVALID, "geometry %u: vertex_address is 0", i);
            if (g[i].vertex_stride < 12 || (g[i].vertex_stride % 4) != 0)
                return fail(RT_ERR_INVALID, "geometry %u: vertex_stride %u (need >= 12, multiple of 4)", i,
                            g[i].vertex_stride);
            if (!aligned(g[i].vertex_address, 4) || !aligned(g[i].index_address, 4))
                return fail(RT_ERR_INVALID, "geometry %u: buffers must be 4-byte aligned", i);
        }
        n += g[i].primitive_count;
    }
    if (n > kMaxPrimitives) return fail(RT_ERR_TOO_LARGE, "%llu triangles > %u", (unsigned long long)n, kMaxPrimitives);
    *n_out = (uint32_t)n;
    return RT_OK;
}

RTCORE_API int32_t rt_get_blas_build_sizes(const RtGeometryTriangles* geometries, uint32_t geometry_count,
                                           uint32_t build_flags, RtBuildSizes* out) {
    if (!out) return fail(RT_ERR_INVALID, "out is NULL");
    uint32_t n = 0;
    int32_t r = blas_prim_count(geometries, geometry_count, &n);
    if (r) return r;
    AsLayout al = AsLayout::make(n, false, build_flags);
    ScratchLayout sl = ScratchLayout::make(n, false, build_flags);
    out->acceleration_structure_size = al.total;
    out->build_scratch_size = sl.build_total;
    out->update_scratch_size = sl.update_total;
    return RT_OK;
}

RTCORE_API int32_t rt_cmd_build_blas(rt_ctx* ctx, const RtGeometryTriangles* geometries, uint32_t geometry_count,
                                     uint32_t build_flags, uint64_t dst, uint64_t dst_size, uint64_t scratch,
                                     uint64_t scratch_size, void* stream) {
    MaybeLock l(ctx);
    uint32_t n = 0;
    int32_t r = blas_prim_count(geometries, geometry_count, &n);
    if (r) return r;
    AsLayout al = AsLayout::make(n, false, build_flags);
    ScratchLayout sl = ScratchLayout::make(n, false, build_flags);
    if (!dst || !aligned(dst, RT_AS_ALIGNMENT)) return fail(RT_ERR_INVALID, "dst must be non-null and 256-byte aligned");
    if (dst_size < al.total)
        return fail(RT_ERR_INVALID, "dst_size %llu < required %llu", (unsigned long long)dst_size,
                    (unsigned long long)al.total);
    if (!scratch || !aligned(scratch, RT_AS_ALIGNMENT))
        return fail(RT_ERR_INVALID, "scratch must be non-null and 256-byte aligned");
    if (scratch_size < sl.build_total)
        return fail(RT_ERR_INVALID, "scratch_size %llu < required %llu", (unsigned long long)scratch_size,
                    (unsigned long long)sl.build_total);
    BlasInput in;
    memset(&in, 0, sizeof in);
    in.geometry_count = geometry_count ? geometry_count : 1;
    in.n = n;
    uint32_t prefix = 0;
    for (uint32_t i = 0; i < geometry_count; i++) {
        in.g[i].pos = reinterpret_cast<const float*>(geometries[i].vertex_address);
        in.g[i].idx = reinterpret_cast<const uint32_t*>(geometries[i].index_address);
        in.g[i].stride_floats = geometries[i].vertex_stride / 4;
        in.g[i].max_vertex = geometries[i].max_vertex;
        in.g[i].prim_count = geometries[i].primitive_count;
        in.g[i].flags = geometries[i].flags;
        in.g[i].prefix = prefix;
        prefix += geometries[i].primitive_count;
    }
    cudaError_t e = launch_blas_build(in, build_flags, reinterpret_cast<uint8_t*>(dst),
                                      reinterpret_cast<uint8_t*>(scratch), reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_build_blas");
    note_blas_kind((build_flags & RT_BUILD_QUANTIZED_NODES) ? kBlasKindQ8 : kBlasKindF32);
    return RT_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// BLAS build without allocation (rt_cmd_build_blas_static_scratch)
// ---------------------------------------------------------------------------
namespace {
// The scratch of the allocation-free BLAS build.  Host code may not use the
// symbol's host-side name as a device address; static_scratch_address()
// looks the device address up once per device.
static __device__ __align__(256) uint8_t g_static_scratch[RT_STATIC_SCRATCH_BYTES];

struct StaticScratchAddress {
    int device;
    uint8_t* ptr;
};
std::mutex g_static_scratch_mu;
std::vector<StaticScratchAddress> g_static_scratch_addrs;

cudaError_t static_scratch_address(uint8_t** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> lk(g_static_scratch_mu);
    for (const auto& a : g_static_scratch_addrs) {
        if (a.device == dev) {
            *out = a.ptr;
            return cudaSuccess;
        }
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return e;
    g_static_scratch_addrs.push_back({dev, reinterpret_cast<uint8_t*>(p)});
    *out = reinterpret_cast<uint8_t*>(p);
    return cudaSuccess;
}
}  // namespace

extern "C" {

RTCORE_API int32_t rt_cmd_build_blas_static_scratch(rt_ctx* ctx, const RtGeometryTriangles* geometries,
                                                    uint32_t geometry_count, uint32_t build_flags, uint64_t dst,
                                                    uint64_t dst_size, void* stream) {
    MaybeLock l(ctx);
    uint32_t n = 0;
    int32_t r = blas_prim_count(geometries, geometry_count, &n);
    if (r) return r;
    if (build_flags & RT_BUILD_QUANTIZED_NODES)
        return fail(RT_ERR_UNSUPPORTED, "RT_BUILD_QUANTIZED_NODES is not supported by the static-scratch build");
    AsLayout al = AsLayout::make(n, false, build_flags);
    ScratchLayout sl = ScratchLayout::make(n, false, build_flags);
    if (!dst || !aligned(dst, RT_AS_ALIGNMENT)) return fail(RT_ERR_INVALID, "dst must be non-null and 256-byte aligned");
    if (dst_size < al.total)
        return fail(RT_ERR_INVALID, "dst_size %llu < required %llu", (unsigned long long)dst_size,
                    (unsigned long long)al.total);
    if (sl.build_total > RT_STATIC_SCRATCH_BYTES)
        return fail(RT_ERR_TOO_LARGE,
                    "a BLAS of %u triangles needs %llu bytes of build scratch; the static scratch holds %llu "
                    "(use rt_cmd_build_blas with caller-allocated scratch)",
                    n, (unsigned long long)sl.build_total, (unsigned long long)RT_STATIC_SCRATCH_BYTES);
    uint8_t* scratch = nullptr;
    cudaError_t e = static_scratch_address(&scratch);
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_build_blas_static_scratch (scratch address)");
    BlasInput in;
    memset(&in, 0, sizeof in);
    in.geometry_count = geometry_count ? geometry_count : 1;
    in.n = n;
    uint32_t prefix = 0;
    for (uint32_t i = 0; i < geometry_count; i++) {
        in.g[i].pos = reinterpret_cast<const float*>(geometries[i].vertex_address);
        in.g[i].idx = reinterpret_cast<const uint32_t*>(geometries[i].index_address);
        in.g[i].stride_floats = geometries[i].vertex_stride / 4;
        in.g[i].max_vertex = geometries[i].max_vertex;
        in.g[i].prim_count = geometries[i].primitive_count;
        in.g[i].flags = geometries[i].flags;
        in.g[i].prefix = prefix;
        prefix += geometries[i].primitive_count;
    }
    e = launch_blas_build(in, build_flags, reinterpret_cast<uint8_t*>(dst), scratch,
                          reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_build_blas_static_scratch");
    note_blas_kind(kBlasKindF32);
    return RT_OK;
}

RTCORE_API int32_t rt_get_tlas_build_sizes(uint32_t instance_count, uint32_t build_flags, RtBuildSizes* out) {
    if (!out) return fail(RT_ERR_INVALID, "out is NULL");
    if (instance_count > kMaxPrimitives) return fail(RT_ERR_TOO_LARGE, "%u instances > %u", instance_count, kMaxPrimitives);
    AsLayout al = AsLayout::make(instance_count, true, build_flags);
    ScratchLayout sl = ScratchLayout::make(instance_count, true, build_flags);
    out->acceleration_structure_size = al.total;
    out->build_scratch_size = sl.build_total;
    out->update_scratch_size = sl.update_total;
    return RT_OK;
}

RTCORE_API int32_t rt_cmd_build_tlas(rt_ctx* ctx, uint64_t instances, uint32_t instance_count, uint32_t build_flags,
                                     uint64_t dst, uint64_t dst_size, uint64_t scratch, uint64_t scratch_size,
                                     void* stream) {
    MaybeLock l(ctx);
    if (instance_count > kMaxPrimitives) return fail(RT_ERR_TOO_LARGE, "%u instances > %u", instance_count, kMaxPrimitives);
    if (instance_count > 0 && (!instances || !aligned(instances, 16)))
        return fail(RT_ERR_INVALID, "instances must be non-null and 16-byte aligned");
    AsLayout al = AsLayout::make(instance_count, true, build_flags);
    ScratchLayout sl = ScratchLayout::make(instance_count, true, build_flags);
    if (!dst || !aligned(dst, RT_AS_ALIGNMENT)) return fail(RT_ERR_INVALID, "dst must be non-null and 256-byte aligned");
    if (dst_size < al.total)
        return fail(RT_ERR_INVALID, "dst_size %llu < required %llu", (unsigned long long)dst_size,
                    (unsigned long long)al.total);
    if (!scratch || !aligned(scratch, RT_AS_ALIGNMENT))
        return fail(RT_ERR_INVALID, "scratch must be non-null and 256-byte aligned");
    if (scratch_size < sl.build_total)
        return fail(RT_ERR_INVALID, "scratch_size %llu < required %llu", (unsigned long long)scratch_size,
                    (unsigned long long)sl.build_total);
    cudaError_t e = launch_tlas_build(reinterpret_cast<const RtAccelerationStructureInstance*>(instances), instance_count,
                                      build_flags, reinterpret_cast<uint8_t*>(dst), reinterpret_cast<uint8_t*>(scratch),
                                      reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_build_tlas");
    return RT_OK;
}

RTCORE_API int32_t rt_cmd_update_tlas(rt_ctx* ctx, uint64_t instances, uint32_t instance_count, uint64_t src,
                                      uint64_t dst, uint64_t dst_size, uint64_t scratch, uint64_t scratch_size,
                                      void* stream) {
    MaybeLock l(ctx);
    if (instance_count > kMaxPrimitives) return fail(RT_ERR_TOO_LARGE, "%u instances > %u", instance_count, kMaxPrimitives);
    if (instance_count > 0 && (!instances || !aligned(instances, 16)))
        return fail(RT_ERR_INVALID, "instances must be non-null and 16-byte aligned");
    if (!src || !dst || !aligned(src, RT_AS_ALIGNMENT) || !aligned(dst, RT_AS_ALIGNMENT))
        return fail(RT_ERR_INVALID, "src/dst must be non-null and 256-byte aligned");
    AsLayout al = AsLayout::make(instance_count, true);
    ScratchLayout sl = ScratchLayout::make(instance_count, true);
    if (dst_size < al.total)
        return fail(RT_ERR_INVALID, "dst_size %llu < required %llu", (unsigned long long)dst_size,
                    (unsigned long long)al.total);
    if (!scratch || !aligned(scratch, RT_AS_ALIGNMENT))
        return fail(RT_ERR_INVALID, "scratch must be non-null and 256-byte aligned");
    if (scratch_size < sl.update_total)
        return fail(RT_ERR_INVALID, "scratch_size %llu < required %llu", (unsigned long long)scratch_size,
                    (unsigned long long)sl.update_total);
    cudaError_t e = launch_tlas_update(reinterpret_cast<const RtAccelerationStructureInstance*>(instances),
                                       instance_count, reinterpret_cast<const uint8_t*>(src),
                                       reinterpret_cast<uint8_t*>(dst), dst_size, reinterpret_cast<uint8_t*>(scratch),
                                       reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_update_tlas");
    return RT_OK;
}

RTCORE_API int32_t rt_cmd_copy_acceleration_structure(rt_ctx* ctx, uint64_t src, uint64_t dst, uint64_t dst_size,
                                                      uint32_t mode, void* stream) {
    MaybeLock l(ctx);
    if (!src || !dst || !aligned(src, RT_AS_ALIGNMENT) || !aligned(dst, RT_AS_ALIGNMENT))
        return fail(RT_ERR_INVALID, "src/dst must be non-null and 256-byte aligned");
    if (src == dst) return fail(RT_ERR_INVALID, "src == dst");
    if (mode != RT_COPY_MODE_CLONE && mode != RT_COPY_MODE_COMPACT) return fail(RT_ERR_INVALID, "copy mode %u", mode);
    if (dst_size < kHeaderBytes) return fail(RT_ERR_INVALID, "dst_size %llu < header", (unsigned long long)dst_size);
    cudaError_t e = launch_as_copy(reinterpret_cast<const uint8_t*>(src), reinterpret_cast<uint8_t*>(dst), dst_size,
                                   mode, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_copy_acceleration_structure");
    return RT_OK;
}

RTCORE_API int32_t rt_get_acceleration_structure_info(uint64_t as, RtAccelerationStructureInfo* out, void* stream) {
    if (!as || !out || !aligned(as, RT_AS_ALIGNMENT)) return fail(RT_ERR_INVALID, "bad AS address or out");
    AsHeader h;
    cudaError_t e = cudaStreamSynchronize(reinterpret_cast<cudaStream_t>(stream));
    if (e == cudaSuccess) e = cudaMemcpy(&h, reinterpret_cast<const void*>(as), sizeof h, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(e, "rt_get_acceleration_structure_info");
    if (h.magic != kAsMagic) return fail(RT_ERR_BAD_AS, "not an acceleration structure written by this library");
    memset(out, 0, sizeof *out);
    out->type = h.type;
    out->build_flags = h.build_flags;
    out->node_count = h.node_count;
    out->primitive_count = h.prim_count;
    out->node_bytes = h.node_bytes;
    out->tree_depth = h.depth;
    out->total_size = h.total_size;
    out->compacted_size = h.compacted_size;
    for (int k = 0; k < 3; k++) {
        out->bounds_lo[k] = h.bounds_lo[k];
        out->bounds_hi[k] = h.bounds_hi[k];
    }
    out->status = h.status;
    return RT_OK;
}

RTCORE_API uint64_t rt_get_acceleration_structure_device_address(uint64_t as_memory) {
    if (!aligned(as_memory, RT_AS_ALIGNMENT)) {
        fail(RT_ERR_INVALID, "AS memory not 256-byte aligned");
        return 0;
    }
    return as_memory;
}

// ---------------------------------------------------------------------------
// Dispatch
// ---------------------------------------------------------------------------
}  // extern "C"

namespace {
int32_t check_scene(const RtPushConstantBufferAddresses* push, const RtTraceRaysDesc* desc, uint32_t index) {
    if (!push->uniforms || !push->acceleration_structure)
        return fail(RT_ERR_INVALID, "scene %u: push constants need uniforms and acceleration_structure", index);
    if (!aligned(push->acceleration_structure, RT_AS_ALIGNMENT) || !aligned(push->uniforms, 16) ||
        !aligned(push->model_info, 8))
        return fail(RT_ERR_INVALID, "scene %u: misaligned push-constant address", index);
    if (desc->width == 0 || desc->height == 0)
        return fail(RT_ERR_INVALID, "scene %u: empty launch %ux%u", index, desc->width, desc->height);
    if ((uint64_t)desc->width * desc->height > (1ull << 31))
        return fail(RT_ERR_TOO_LARGE, "scene %u: launch %ux%u too large", index, desc->width, desc->height);
    if (desc->max_trace_depth == 0 || desc->max_trace_depth > 64)
        return fail(RT_ERR_INVALID, "scene %u: max_trace_depth %u (need 1..64)", index, desc->max_trace_depth);
    if (desc->shadow_ray_count > 256)
        return fail(RT_ERR_INVALID, "scene %u: shadow_ray_count %u > 256", index, desc->shadow_ray_count);
    if (!desc->image_address && !desc->radiance_address) return fail(RT_ERR_INVALID, "scene %u: no output buffer", index);
    if (!aligned(desc->image_address, 4) || !aligned(desc->radiance_address, 16))
        return fail(RT_ERR_INVALID, "scene %u: misaligned output buffer", index);
    return RT_OK;
}

int32_t trace_scenes(rt_ctx* ctx, const std::vector<TraceScene>& scenes, const RtShaderBindingTable* sbt,
                     uint32_t flags, void* stream, const char* what) {
    RtShaderBindingTable table = sbt ? *sbt : reference_sbt();
    int32_t r = check_sbt(&table);
    if (r) return r;
    uint64_t slots = 0, shadow_rays = 0;
    for (const TraceScene& t : scenes) {
        slots += (uint64_t)((t.desc.width + 7) / 8) * ((t.desc.height + 3) / 4) * 32;
        shadow_rays += (uint64_t)t.desc.width * t.desc.height * t.desc.shadow_ray_count;
    }
    if (slots > (1ull << 31) || shadow_rays > (1ull << 31))
        return fail(RT_ERR_TOO_LARGE, "%s: %llu ray slots / %llu shadow rays exceed 2^31", what,
                    (unsigned long long)slots, (unsigned long long)shadow_rays);
    MaybeLock l(ctx);
    TraceBatch b;
    b.scenes = scenes.data();
    b.count = (uint32_t)scenes.size();
    b.stats = (flags & RT_TRACE_FLAG_COLLECT_STATS) ? 1u : 0u;
    b.sbt = table;
    b.ctx_textures = ctx->textures;
    b.stats_dev = &ctx->dev->stats;
    b.status = &ctx->dev->stats.status;
    b.kinds_built = blas_kinds_built();
    b.config = ctx->traversal;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    uint8_t* ws = nullptr;
    cudaError_t e = ctx_workspace(ctx, s, trace_workspace_bytes(b.scenes, b.count), &ws);
    if (e == cudaErrorStreamCaptureUnsupported)
        return fail(RT_ERR_INVALID, "%s: the workspace must grow, which a stream capture cannot do; "
                    "trace the same scenes once outside the capture first", what);
    if (e != cudaSuccess) return cuda_fail(e, what);
    KernelTimer* timer = nullptr;
    if (flags & RT_TRACE_FLAG_KERNEL_TIMINGS) {
        if (!ctx->timer.created) {
            for (int i = 0; i < KernelTimer::kMax && e == cudaSuccess; i++) e = cudaEventCreate(&ctx->timer.ev[i]);
            if (e != cudaSuccess) return cuda_fail(e, what);
            ctx->timer.created = true;
        }
        timer = &ctx->timer;
    }
    e = launch_trace_batch(b, ws, ctx->num_sms, s, timer);
    if (e != cudaSuccess) return cuda_fail(e, what);
    return RT_OK;
}
}  // namespace

extern "C" {

RTCORE_API int32_t rt_cmd_trace_rays(rt_ctx* ctx, const RtPushConstantBufferAddresses* push,
                                     const RtShaderBindingTable* sbt, const RtTraceRaysDesc* desc, void* stream) {
    if (!ctx || !push || !desc) return fail(RT_ERR_INVALID, "ctx, push or desc is NULL");
    int32_t r = check_scene(push, desc, 0);
    if (r) return r;
    std::vector<TraceScene> one(1);
    one[0].push = *push;
    one[0].desc = *desc;
    one[0].textures = nullptr;
    one[0].texture_count = 0;
    one[0]._pad = 0;
    return trace_scenes(ctx, one, sbt, desc->flags, stream, "rt_cmd_trace_rays");
}

RTCORE_API int32_t rt_cmd_trace_rays_batched(rt_ctx* ctx, const RtBatchScene* scenes, uint32_t scene_count,
                                             const RtShaderBindingTable* sbt, uint32_t flags, void* stream) {
    if (!ctx || (!scenes && scene_count)) return fail(RT_ERR_INVALID, "ctx or scenes is NULL");
    if (scene_count == 0) return RT_OK;
    if (scene_count > RT_MAX_BATCH_SCENES)
        return fail(RT_ERR_TOO_LARGE, "%u scenes > RT_MAX_BATCH_SCENES", scene_count);
    if (flags & ~(RT_TRACE_FLAG_COLLECT_STATS | RT_TRACE_FLAG_KERNEL_TIMINGS))
        return fail(RT_ERR_INVALID, "unknown batch flags 0x%x", flags);
    std::vector<TraceScene> v(scene_count);
    for (uint32_t i = 0; i < scene_count; i++) {
        const RtBatchScene& b = scenes[i];
        int32_t r = check_scene(&b.push, &b.desc, i);
        if (r) return r;
        if (b.texture_table && (b.texture_count == 0 || b.texture_count > RT_MAX_BOUND_IMAGES ||
                                !aligned(b.texture_table, 16)))
            return fail(RT_ERR_INVALID, "scene %u: texture table needs 1..%u entries, 16-byte aligned", i,
                        RT_MAX_BOUND_IMAGES);
        v[i].push = b.push;
        v[i].desc = b.desc;
        v[i].desc.flags &= RT_TRACE_FLAG_LAMBERT_DIFFUSE;
        v[i].textures = reinterpret_cast<const RtTextureDesc*>(b.texture_table);
        v[i].texture_count = b.texture_table ? b.texture_count : 0u;
        v[i]._pad = 0;
    }
    return trace_scenes(ctx, v, sbt, flags, stream, "rt_cmd_trace_rays_batched");
}

RTCORE_API int32_t rt_ctx_set_traversal_config(rt_ctx* ctx, const RtTraversalConfig* config) {
    if (!ctx || !config) return fail(RT_ERR_INVALID, "ctx or config is NULL");
    if (!traversal_config_supported(*config))
        return fail(RT_ERR_UNSUPPORTED, "traversal config {%u, %u, %u, 0x%x} is not built (block 64/128/256, shared "
                    "stack depth 0/16/24/32, leaf_wait <= 32, packet_lists <= 3)", config->block_size,
                    config->shared_stack_depth, config->leaf_wait, config->packet_lists);
    MaybeLock l(ctx);
    ctx->traversal = *config;
    return RT_OK;
}

RTCORE_API int32_t rt_ctx_get_traversal_config(rt_ctx* ctx, RtTraversalConfig* out) {
    if (!ctx || !out) return fail(RT_ERR_INVALID, "ctx or out is NULL");
    MaybeLock l(ctx);
    *out = ctx->traversal;
    return RT_OK;
}

RTCORE_API int32_t rt_ctx_autotune(rt_ctx* ctx, const RtBatchScene* scenes, uint32_t scene_count,
                                   const RtShaderBindingTable* sbt, uint32_t reps, void* stream,
                                   RtAutotuneReport* report) {
    if (!ctx || !scenes || scene_count == 0) return fail(RT_ERR_INVALID, "ctx or scenes is NULL / empty");
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    if (stream_capturing(s)) return fail(RT_ERR_INVALID, "rt_ctx_autotune cannot run inside a stream capture");
    reps = std::max(1u, std::min(reps, 64u));
    // stage 1: the per-lane launch shapes (the default among them); stage 2:
    // the packet_lists choices on the fastest shape
    static const uint32_t kBlocks[] = {64, 128, 256}, kDepths[] = {0, 16, 24, 32}, kWaits[] = {16, 20, 24};
    std::vector<RtTraversalConfig> cands;
    for (uint32_t b : kBlocks)
        for (uint32_t d : kDepths)
            for (uint32_t w : kWaits) cands.push_back(RtTraversalConfig{b, d, w, 0});
    const RtTraversalConfig saved = ctx->traversal;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t ce = cudaEventCreate(&e0);
    if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
    if (ce != cudaSuccess) return cuda_fail(ce, "rt_ctx_autotune (events)");
    std::vector<float> med;
    int32_t r = RT_OK;
    auto time_cands = [&](size_t from) {
        for (size_t i = from; i < cands.size() && r == RT_OK; i++) {
            ctx->traversal = cands[i];
            std::vector<float> t;
            for (uint32_t k = 0; k <= reps && r == RT_OK; k++) {
                ce = cudaEventRecord(e0, s);
                if (ce == cudaSuccess) r = rt_cmd_trace_rays_batched(ctx, scenes, scene_count, sbt, 0, stream);
                if (r == RT_OK && ce == cudaSuccess) ce = cudaEventRecord(e1, s);
                if (r == RT_OK && ce == cudaSuccess) ce = cudaEventSynchronize(e1);
                float ms = 0.0f;
                if (r == RT_OK && ce == cudaSuccess) ce = cudaEventElapsedTime(&ms, e0, e1);
                if (ce != cudaSuccess) r = cuda_fail(ce, "rt_ctx_autotune");
                if (k > 0) t.push_back(ms);  // the first run is the warm-up
            }
            if (r == RT_OK) {
                std::sort(t.begin(), t.end());
                med.push_back(t[t.size() / 2]);
            }
        }
    };
    auto fastest = [&] {
        size_t best = 0;
        for (size_t i = 1; i < med.size(); i++)
            if (med[i] < med[best]) best = i;
        return best;
    };
    time_cands(0);
    if (r == RT_OK) {
        const RtTraversalConfig shape = cands[fastest()];
        const size_t n1 = cands.size();
        const uint32_t P1 = RT_TRAVERSAL_PACKET_PRIMARY, P2 = RT_TRAVERSAL_PACKET_SHADOW,
                       LB = RT_TRAVERSAL_PACKET_LANE_BOUNCES;
        for (uint32_t pl : {P1, P2, P1 | P2, P1 | LB, P1 | P2 | LB})
            cands.push_back(RtTraversalConfig{shape.block_size, shape.shared_stack_depth, shape.leaf_wait, pl});
        time_cands(n1);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (r != RT_OK) {
        ctx->traversal = saved;
        return r;
    }
    const size_t best = fastest();
    ctx->traversal = cands[best];
    if (report) {
        memset(report, 0, sizeof *report);
        report->count = (uint32_t)std::min<size_t>(cands.size(), RT_AUTOTUNE_MAX_CONFIGS);
        report->best = (uint32_t)best;
        for (uint32_t i = 0; i < report->count; i++) {
            report->configs[i] = cands[i];
            report->median_ms[i] = med[i];
        }
    }
    return RT_OK;
}

RTCORE_API int32_t rt_cmd_trace_ray_buffer(rt_ctx* ctx, uint64_t tlas, const RtPushConstantBufferAddresses* push,
                                           const RtShaderBindingTable* sbt, uint32_t ray_flags, uint32_t cull_mask,
                                           uint32_t sbt_offset, uint64_t rays, uint32_t ray_count, uint64_t hits,
                                           void* stream) {
    if (!ctx) return fail(RT_ERR_INVALID, "ctx is NULL");
    if (!tlas || !aligned(tlas, RT_AS_ALIGNMENT)) return fail(RT_ERR_INVALID, "tlas must be non-null and 256-byte aligned");
    if (ray_count > 0 && (!rays || !hits || !aligned(rays, 16) || !aligned(hits, 16)))
        return fail(RT_ERR_INVALID, "rays/hits must be non-null and 16-byte aligned");
    if (ray_flags & ~(0xFFu | RT_RAY_FLAG_EXT_COLLECT_STATS))
        return fail(RT_ERR_INVALID, "unknown ray flags 0x%x", ray_flags);
    RtShaderBindingTable table = sbt ? *sbt : reference_sbt();
    int32_t r = check_sbt(&table);
    if (r) return r;
    MaybeLock l(ctx);
    RayBufferLaunch p;
    memset(&p.push, 0, sizeof p.push);
    if (push) p.push = *push;
    p.sbt = table;
    memcpy(p.textures, ctx->textures, sizeof p.textures);
    p.tlas = tlas;
    p.rays = reinterpret_cast<const RtRay*>(rays);
    p.hits = reinterpret_cast<RtHit*>(hits);
    p.count = ray_count;
    p.ray_flags = ray_flags & 0xFFu;
    p.cull_mask = cull_mask & 0xFFu;
    p.sbt_offset = sbt_offset;
    p.collect_stats = (ray_flags & RT_RAY_FLAG_EXT_COLLECT_STATS) ? 1u : 0u;
    p.stats = &ctx->dev->stats;
    p.status = &ctx->dev->stats.status;
    p.work = &ctx->dev->work[ctx->work_slot.fetch_add(1) % kWorkSlots];
    p.kinds_built = blas_kinds_built();
    cudaError_t e = launch_trace_ray_buffer(p, ctx->num_sms, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_cmd_trace_ray_buffer");
    return RT_OK;
}

RTCORE_API int32_t rt_trace_ray_buffer_host(rt_ctx* ctx, uint64_t tlas, const RtPushConstantBufferAddresses* push,
                                            const RtShaderBindingTable* sbt, uint32_t ray_flags,
                                            uint32_t cull_mask, uint32_t sbt_offset, const RtRay* host_rays,
                                            uint32_t ray_count, RtHit* host_hits, uint32_t chunk_rays,
                                            void* stream) {
    if (!ctx) return fail(RT_ERR_INVALID, "ctx is NULL");
    if (ray_count == 0) return RT_OK;
    if (!host_rays || !host_hits) return fail(RT_ERR_INVALID, "host_rays / host_hits is NULL");
    cudaStream_t caller = reinterpret_cast<cudaStream_t>(stream);
    if (stream_capturing(caller)) return fail(RT_ERR_INVALID, "rt_trace_ray_buffer_host cannot run in a capture");
    if (chunk_rays == 0) {
        // Page-locked host buffers are mapped into the GPU's address space
        // (over NVLink-C2C on Grace systems): the traversal reads each ray
        // from and writes each hit to host memory itself, in one launch,
        // with no staging copies to overlap.
        cudaPointerAttributes ra{}, ha{};
        if (cudaPointerGetAttributes(&ra, host_rays) == cudaSuccess && ra.type == cudaMemoryTypeHost &&
            ra.devicePointer && cudaPointerGetAttributes(&ha, host_hits) == cudaSuccess &&
            ha.type == cudaMemoryTypeHost && ha.devicePointer)
            return rt_cmd_trace_ray_buffer(ctx, tlas, push, sbt, ray_flags, cull_mask, sbt_offset,
                                           reinterpret_cast<uint64_t>(ra.devicePointer), ray_count,
                                           reinterpret_cast<uint64_t>(ha.devicePointer), stream);
        cudaGetLastError();  // a pageable pointer is not an error here
    }
    const uint64_t chunk = std::min<uint64_t>(chunk_rays ? chunk_rays : (1u << 20), ray_count);
    auto& hq = ctx->hq;
    std::lock_guard<std::mutex> lk(hq.mu);
    cudaError_t e = cudaSuccess;
    if (!hq.created) {
        for (int k = 0; k < 2 && e == cudaSuccess; k++) {
            e = cudaStreamCreateWithFlags(&hq.st[k], cudaStreamNonBlocking);
            if (e == cudaSuccess) e = cudaEventCreateWithFlags(&hq.done[k], cudaEventDisableTiming);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&hq.start, cudaEventDisableTiming);
        if (e != cudaSuccess) return cuda_fail(e, "rt_trace_ray_buffer_host (streams)");
        hq.created = true;
    }
    if (hq.chunk < chunk) {
        for (int k = 0; k < 2; k++) {
            if (hq.staging[k]) {
                cudaStreamSynchronize(hq.st[k]);
                cudaFree(hq.staging[k]);
                hq.staging[k] = nullptr;
            }
        }
        hq.chunk = 0;
        for (int k = 0; k < 2 && e == cudaSuccess; k++)
            e = cudaMalloc(reinterpret_cast<void**>(&hq.staging[k]), chunk * (sizeof(RtRay) + sizeof(RtHit)));
        if (e != cudaSuccess) return cuda_fail(e, "rt_trace_ray_buffer_host (staging)");
        hq.chunk = chunk;
    }
    e = cudaEventRecord(hq.start, caller);
    for (int k = 0; k < 2 && e == cudaSuccess; k++) e = cudaStreamWaitEvent(hq.st[k], hq.start, 0);
    if (e != cudaSuccess) return cuda_fail(e, "rt_trace_ray_buffer_host (ordering)");
    const uint64_t nchunks = (ray_count + chunk - 1) / chunk;
    for (uint64_t i = 0; i < nchunks; i++) {
        const int k = (int)(i & 1);
        const uint64_t first = i * chunk, n = std::min<uint64_t>(chunk, ray_count - first);
        uint8_t* rays_dev = hq.staging[k];
        uint8_t* hits_dev = hq.staging[k] + hq.chunk * sizeof(RtRay);
        e = cudaMemcpyAsync(rays_dev, host_rays + first, n * sizeof(RtRay), cudaMemcpyHostToDevice, hq.st[k]);
        if (e != cudaSuccess) return cuda_fail(e, "rt_trace_ray_buffer_host (rays in)");
        int32_t r = rt_cmd_trace_ray_buffer(ctx, tlas, push, sbt, ray_flags, cull_mask, sbt_offset,
                                            reinterpret_cast<uint64_t>(rays_dev), (uint32_t)n,
                                            reinterpret_cast<uint64_t>(hits_dev), hq.st[k]);
        if (r != RT_OK) return r;
        e = cudaMemcpyAsync(host_hits + first, hits_dev, n * sizeof(RtHit), cudaMemcpyDeviceToHost, hq.st[k]);
        if (e != cudaSuccess) return cuda_fail(e, "rt_trace_ray_buffer_host (hits out)");
    }
    for (int k = 0; k < 2 && e == cudaSuccess; k++) {
        e = cudaEventRecord(hq.done[k], hq.st[k]);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(caller, hq.done[k], 0);
    }
    if (e != cudaSuccess) return cuda_fail(e, "rt_trace_ray_buffer_host (join)");
    return RT_OK;
}

RTCORE_API int32_t rt_debug_eval(uint32_t function, uint64_t in, uint64_t out, uint32_t count, void* stream) {
    if (function > RT_FN_WATERTIGHT) return fail(RT_ERR_INVALID, "unknown function %u", function);
    if (count > 0 && (!in || !out || !aligned(in, 4) || !aligned(out, 4)))
        return fail(RT_ERR_INVALID, "in/out must be non-null and 4-byte aligned");
    cudaError_t e = launch_debug_eval(function, reinterpret_cast<const float*>(in), reinterpret_cast<float*>(out), count,
                                      reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "rt_debug_eval");
    return RT_OK;
}

RTCORE_API int32_t rt_debug_sort_pairs(uint64_t keys, uint64_t values, uint32_t count, uint64_t scratch,
                                       uint64_t scratch_size, uint64_t* scratch_needed, void* stream) {
    // scratch: an error word, the second key / value buffers, the sort state
    const uint64_t off_k1 = 256, off_v1 = align_up(off_k1 + (uint64_t)count * 4, 256);
    const uint64_t off_state = align_up(off_v1 + (uint64_t)count * 4, 256);
    const uint64_t need = off_state + key_sort_state_bytes(count);
    if (scratch_needed) *scratch_needed = need;
    if (!scratch) return RT_OK;
    if (count > kMaxPrimitives) return fail(RT_ERR_TOO_LARGE, "%u pairs > %u", count, kMaxPrimitives);
    if (scratch_size < need)
        return fail(RT_ERR_INVALID, "scratch_size %llu < %llu", (unsigned long long)scratch_size,
                    (unsigned long long)need);
    if (count > 0 && (!keys || !values || !aligned(keys, 4) || !aligned(values, 4) || !aligned(scratch, 256)))
        return fail(RT_ERR_INVALID, "keys / values must be 4-byte aligned, scratch 256-byte aligned");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint8_t* base = reinterpret_cast<uint8_t*>(scratch);
    uint32_t* err = reinterpret_cast<uint32_t*>(base);
    cudaError_t e = cudaMemsetAsync(err, 0, 4, st);
    if (e == cudaSuccess)
        e = launch_key_sort(reinterpret_cast<uint32_t*>(keys), reinterpret_cast<uint32_t*>(values),
                            reinterpret_cast<uint32_t*>(base + off_k1), reinterpret_cast<uint32_t*>(base + off_v1), count,
                            base + off_state, err, st);
    uint32_t h_err = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "rt_debug_sort_pairs");
    if (h_err & (1u << RT_ERR_TIMEOUT)) return fail(RT_ERR_TIMEOUT, "rt_debug_sort_pairs: a bounded wait gave up");
    return RT_OK;
}

}  // extern "C"
