// rt_serve.cu — the serving form: a request loop over device-resident scenes.
//
// One worker thread per server forms batches from the request queue in
// arrival order and hands each to rt_cmd_trace_rays_batched on the server's
// stream; up to max_in_flight batches are queued on the GPU at once, so a
// batch is formed (and its uniforms uploaded) while the previous one renders,
// and requests that arrive meanwhile join the next batch.  Admission is by
// bytes: resident scenes + the frame buffers of admitted requests + the batch
// workspace stay within the HBM budget; a request that cannot fit waits for
// completions to release memory, one that could never fit is rejected.
// Completion is signalled by a host callback queued after the batch's image
// copies, which releases the batch's bytes and wakes waiters; device memory
// is returned to the server's stream-ordered pool by the worker, outside the
// lock (host callbacks may not call CUDA, and a CUDA call that waits for the
// stream must not hold the lock the callback needs).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rt_internal.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
}

constexpr uint64_t kUniformSlot = 256;  // bytes per request for its uniforms

struct Request {
    uint64_t ticket;
    RtServeRequest req;
    Clock::time_point t_submit, t_launch, t_done;
    uint64_t frame_bytes;   // server-owned bytes: uniforms slot + image (if server-owned)
    bool host_direct;       // image_host is page-locked: the output kernel writes it directly
    RtServeResult result;
};

struct Batch {
    uint32_t id;
    std::vector<Request*> reqs;
    uint8_t* device = nullptr;  // uniforms slots, then server-owned images
    uint64_t bytes = 0;         // frame bytes counted in the budget
    uint32_t slot = 0;          // pinned staging slot of its uniforms
    bool done = false;
    struct rt_server* server = nullptr;
};

uint64_t align256(uint64_t v) { return (v + 255) & ~255ull; }

}  // namespace

struct rt_server {
    rt_ctx* ctx = nullptr;
    RtServerConfig cfg{};
    cudaStream_t stream = nullptr;
    cudaMemPool_t pool = nullptr;      // frame buffers, stream-ordered
    uint8_t* staging = nullptr;        // pinned: max_in_flight slots of max_batch_requests uniforms
    std::vector<uint32_t> free_slots;
    int device = 0;
    std::vector<RtServeScene> scenes;
    std::mutex mu;
    std::condition_variable cv;      // worker: queue / budget / slots changed
    std::condition_variable done_cv; // waiters: a request finished
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, Request*> tickets;
    std::vector<Batch*> in_flight;
    uint64_t next_ticket = 1;
    uint32_t next_batch = 0;
    uint64_t resident = 0, frames = 0, workspace = 0, peak = 0;
    RtServeStats stats{};
    bool stop = false;
    std::thread worker;

    uint64_t used() const { return resident + frames + workspace; }
    void note_peak() { peak = std::max(peak, used()); }
};

namespace {

// Whether the GPU can write `p` directly: page-locked host memory
// (cudaHostAlloc / cudaHostRegister), which the output kernel reaches through
// its mapping instead of a device frame buffer and a copy.
bool page_locked(uint64_t p) {
    if (!p) return false;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, reinterpret_cast<void*>(p)) != cudaSuccess) {
        cudaGetLastError();  // pageable memory may report an error on older runtimes: clear it
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

uint64_t frame_bytes_of(const RtServeRequest& r, bool host_direct) {
    uint64_t b = kUniformSlot;
    if (!r.image_device && !host_direct) b += align256((uint64_t)r.width * r.height * 4);
    return b;
}

// Ray slots of a request: its pixels padded to whole 8x4 tiles.
uint64_t slots_of(const RtServeRequest& r) {
    return (uint64_t)((r.width + 7) / 8) * 8 * (uint64_t)((r.height + 3) / 4) * 4;
}

rt::TraceScene trace_scene_of(const RtServeScene& s, const RtServeRequest& r) {
    rt::TraceScene t{};
    t.push.model_info = s.model_info;
    t.push.acceleration_structure = s.acceleration_structure;
    t.desc.width = r.width;
    t.desc.height = r.height;
    t.desc.max_trace_depth = r.max_trace_depth;
    t.desc.shadow_ray_count = r.shadow_ray_count;
    t.desc.flags = r.flags & RT_TRACE_FLAG_LAMBERT_DIFFUSE;
    t.textures = reinterpret_cast<const RtTextureDesc*>(s.texture_table);
    t.texture_count = s.texture_table ? s.texture_count : 0u;
    return t;
}

// Workspace a batch of these requests needs (the per-stream workspace only grows).
uint64_t batch_workspace(const rt_server* sv, const std::vector<Request*>& reqs) {
    std::vector<rt::TraceScene> ts;
    ts.reserve(reqs.size());
    for (const Request* q : reqs) ts.push_back(trace_scene_of(sv->scenes[q->req.scene], q->req));
    return rt::trace_workspace_bytes(ts.data(), (uint32_t)ts.size());
}

void CUDART_CB batch_done(void* p) {
    Batch* b = static_cast<Batch*>(p);
    rt_server* sv = b->server;
    const Clock::time_point now = Clock::now();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        for (Request* q : b->reqs) {
            q->t_done = now;
            q->result.state = RT_SERVE_DONE;
            q->result.latency_ms = ms_between(q->t_submit, now);
            sv->stats.completed++;
            sv->stats.pixels += (uint64_t)q->req.width * q->req.height;
        }
        sv->frames -= b->bytes;
        sv->free_slots.push_back(b->slot);
        b->done = true;
    }
    sv->cv.notify_all();
    sv->done_cv.notify_all();
}

// Takes the finished batches out of the in-flight list (lock held); the
// caller frees them with the lock released (free_batches).
std::vector<Batch*> take_finished(rt_server* sv) {
    std::vector<Batch*> out;
    auto it = sv->in_flight.begin();
    while (it != sv->in_flight.end()) {
        if ((*it)->done) {
            out.push_back(*it);
            it = sv->in_flight.erase(it);
        } else {
            ++it;
        }
    }
    return out;
}

void free_batches(rt_server* sv, const std::vector<Batch*>& bs) {
    for (Batch* b : bs) {
        if (b->device) cudaFreeAsync(b->device, sv->stream);
        delete b;
    }
}

// Launches one batch (worker thread, lock NOT held).
int32_t launch(rt_server* sv, Batch* b) {
    const uint32_t n = (uint32_t)b->reqs.size();
    cudaError_t e = cudaMallocFromPoolAsync(reinterpret_cast<void**>(&b->device), b->bytes, sv->pool, sv->stream);
    if (e != cudaSuccess) return RT_ERR_OOM;
    uint8_t* staging = sv->staging + (size_t)b->slot * sv->cfg.max_batch_requests * kUniformSlot;
    std::vector<RtBatchScene> items(n);
    uint64_t off = (uint64_t)n * kUniformSlot;
    for (uint32_t i = 0; i < n; i++) {
        const RtServeRequest& r = b->reqs[i]->req;
        const RtServeScene& s = sv->scenes[r.scene];
        memcpy(staging + (size_t)i * kUniformSlot, &r.uniforms, sizeof(RtUniforms));
        RtBatchScene& it = items[i];
        memset(&it, 0, sizeof it);
        it.push.model_info = s.model_info;
        it.push.uniforms = reinterpret_cast<uint64_t>(b->device) + (uint64_t)i * kUniformSlot;
        it.push.acceleration_structure = s.acceleration_structure;
        it.texture_table = s.texture_table;
        it.texture_count = s.texture_table ? s.texture_count : 0u;
        it.desc.width = r.width;
        it.desc.height = r.height;
        it.desc.max_trace_depth = r.max_trace_depth;
        it.desc.shadow_ray_count = r.shadow_ray_count;
        it.desc.flags = r.flags & RT_TRACE_FLAG_LAMBERT_DIFFUSE;
        if (r.image_device) {
            it.desc.image_address = r.image_device;
        } else if (b->reqs[i]->host_direct) {
            it.desc.image_address = r.image_host;
        } else {
            it.desc.image_address = reinterpret_cast<uint64_t>(b->device) + off;
            off += align256((uint64_t)r.width * r.height * 4);
        }
    }
    e = cudaMemcpyAsync(b->device, staging, (size_t)n * kUniformSlot, cudaMemcpyHostToDevice, sv->stream);
    if (e != cudaSuccess) return RT_ERR_CUDA;
    int32_t st = rt_cmd_trace_rays_batched(sv->ctx, items.data(), n, nullptr, 0, sv->stream);
    if (st != RT_OK) return st;
    for (uint32_t i = 0; i < n; i++) {
        const RtServeRequest& r = b->reqs[i]->req;
        if (!r.image_host || b->reqs[i]->host_direct) continue;
        e = cudaMemcpyAsync(reinterpret_cast<void*>(r.image_host), reinterpret_cast<void*>(items[i].desc.image_address),
                            (size_t)r.width * r.height * 4, cudaMemcpyDeviceToHost, sv->stream);
        if (e != cudaSuccess) return RT_ERR_CUDA;
    }
    e = cudaLaunchHostFunc(sv->stream, batch_done, b);
    return e == cudaSuccess ? RT_OK : RT_ERR_CUDA;
}

void worker_loop(rt_server* sv) {
    cudaSetDevice(sv->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    for (;;) {
        std::vector<Batch*> finished = take_finished(sv);
        if (!finished.empty()) {
            lk.unlock();
            free_batches(sv, finished);
            lk.lock();
            continue;
        }
        if (sv->stop && sv->queue.empty() && sv->in_flight.empty()) break;
        if (sv->queue.empty() || sv->in_flight.size() >= sv->cfg.max_in_flight) {
            sv->cv.wait(lk);
            continue;
        }
        // form a batch: arrival order, within the request / ray-slot / shadow-ray limits and the budget
        // (a request beyond a limit on its own still forms a batch alone)
        Batch* b = new Batch();
        b->server = sv;
        uint64_t slots = 0, shadow = 0;
        while (!sv->queue.empty() && b->reqs.size() < sv->cfg.max_batch_requests) {
            Request* q = sv->queue.front();
            const uint64_t sl = slots_of(q->req);
            const uint64_t sh = (uint64_t)q->req.width * q->req.height * q->req.shadow_ray_count;
            if (!b->reqs.empty() && sv->cfg.max_batch_pixels && slots + sl > sv->cfg.max_batch_pixels) break;
            if (!b->reqs.empty() && sv->cfg.max_batch_shadow_rays && shadow + sh > sv->cfg.max_batch_shadow_rays)
                break;
            b->reqs.push_back(q);
            const uint64_t ws = std::max(sv->workspace, batch_workspace(sv, b->reqs));
            if (sv->resident + sv->frames + b->bytes + q->frame_bytes + ws > sv->cfg.hbm_budget_bytes) {
                b->reqs.pop_back();
                break;
            }
            sv->queue.pop_front();
            b->bytes += q->frame_bytes;
            slots += sl;
            shadow += sh;
        }
        if (b->reqs.empty()) {  // the head request waits for memory to be released
            delete b;
            if (sv->in_flight.empty()) {
                // nothing will free memory: it cannot fit (submit checked it alone against the budget)
                Request* q = sv->queue.front();
                sv->queue.pop_front();
                q->result.state = RT_SERVE_REJECTED;
                q->result.status = RT_ERR_OOM;
                sv->stats.rejected++;
                sv->done_cv.notify_all();
                continue;
            }
            sv->cv.wait(lk);
            continue;
        }
        sv->workspace = std::max(sv->workspace, batch_workspace(sv, b->reqs));
        sv->frames += b->bytes;
        sv->note_peak();
        b->id = sv->next_batch++;
        b->slot = sv->free_slots.back();
        sv->free_slots.pop_back();
        sv->stats.batches++;
        const Clock::time_point now = Clock::now();
        for (Request* q : b->reqs) {
            q->t_launch = now;
            q->result.batch = b->id;
            q->result.batch_requests = (uint32_t)b->reqs.size();
            q->result.queue_ms = ms_between(q->t_submit, now);
        }
        sv->in_flight.push_back(b);
        lk.unlock();
        const int32_t st = launch(sv, b);
        lk.lock();
        if (st != RT_OK) {  // fail the batch's requests; its memory is released when the stream reaches here
            for (Request* q : b->reqs) q->result.status = (uint32_t)st;
            if (cudaLaunchHostFunc(sv->stream, batch_done, b) != cudaSuccess) {
                // no callback will come: finish the batch here, as batch_done would
                lk.unlock();
                batch_done(b);
                lk.lock();
            }
        }
    }
}

}  // namespace

extern "C" {

RTCORE_API int32_t rt_server_create(rt_ctx* ctx, const RtServerConfig* config, rt_server** out) {
    if (!ctx || !config || !out) return RT_ERR_INVALID;
    if (config->max_batch_requests == 0 || config->max_batch_requests > RT_MAX_BATCH_SCENES ||
        config->max_in_flight == 0 || config->max_in_flight > 64 || config->hbm_budget_bytes == 0)
        return RT_ERR_INVALID;
    if (!rt::ctx_is_threadsafe(ctx)) return RT_ERR_INVALID;  // the worker thread shares the context
    rt_server* sv = new rt_server();
    sv->ctx = ctx;
    sv->cfg = *config;
    cudaGetDevice(&sv->device);
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = sv->device;
    cudaError_t e = cudaStreamCreateWithFlags(&sv->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMemPoolCreate(&sv->pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = config->hbm_budget_bytes;  // keep freed frame buffers for reuse up to the budget
        e = cudaMemPoolSetAttribute(sv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess)
        e = cudaMallocHost(reinterpret_cast<void**>(&sv->staging),
                           (size_t)config->max_in_flight * config->max_batch_requests * kUniformSlot);
    if (e == cudaSuccess && config->max_batch_pixels && config->max_batch_shadow_rays) {
        // Size the wavefront workspace of the server's stream for the largest batch the limits allow,
        // and grow the frame-buffer pool by one full batch of images, so that steady-state batches
        // allocate nothing new; both count against the budget from here on.
        const uint64_t ws = rt::trace_workspace_bound(config->max_batch_requests, config->max_batch_pixels,
                                                      config->max_batch_pixels, config->max_batch_shadow_rays);
        const uint64_t frames = (uint64_t)config->max_batch_requests * kUniformSlot +
                                align256((uint64_t)config->max_batch_pixels * 4);
        if (ws + frames > config->hbm_budget_bytes) {
            e = cudaErrorMemoryAllocation;
        } else {
            e = rt::ctx_reserve_workspace(ctx, sv->stream, ws);
            void* warm = nullptr;
            if (e == cudaSuccess) e = cudaMallocFromPoolAsync(&warm, frames, sv->pool, sv->stream);
            if (e == cudaSuccess) e = cudaFreeAsync(warm, sv->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(sv->stream);
            if (e == cudaSuccess) {
                sv->workspace = ws;
                sv->note_peak();
            }
        }
    }
    if (e != cudaSuccess) {
        if (sv->staging) cudaFreeHost(sv->staging);
        if (sv->pool) cudaMemPoolDestroy(sv->pool);
        if (sv->stream) cudaStreamDestroy(sv->stream);
        delete sv;
        return e == cudaErrorMemoryAllocation ? RT_ERR_OOM : RT_ERR_CUDA;
    }
    for (uint32_t i = 0; i < config->max_in_flight; i++) sv->free_slots.push_back(i);
    sv->stats.budget_bytes = config->hbm_budget_bytes;
    sv->worker = std::thread(worker_loop, sv);
    *out = sv;
    return RT_OK;
}

RTCORE_API int32_t rt_server_destroy(rt_server* sv) {
    if (!sv) return RT_ERR_INVALID;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv.notify_all();
    sv->worker.join();  // returns once every admitted batch has finished and been freed
    cudaStreamSynchronize(sv->stream);
    for (auto& kv : sv->tickets) delete kv.second;
    sv->tickets.clear();
    cudaMemPoolDestroy(sv->pool);
    cudaFreeHost(sv->staging);
    cudaStreamDestroy(sv->stream);
    delete sv;
    return RT_OK;
}

RTCORE_API int32_t rt_server_add_scene(rt_server* sv, const RtServeScene* scene, uint32_t* id) {
    if (!sv || !scene || !id || !scene->acceleration_structure) return RT_ERR_INVALID;
    if (scene->texture_table && (scene->texture_count == 0 || scene->texture_count > RT_MAX_BOUND_IMAGES))
        return RT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(sv->mu);
    if (sv->used() + scene->resident_bytes > sv->cfg.hbm_budget_bytes) return RT_ERR_OOM;
    sv->scenes.push_back(*scene);
    sv->resident += scene->resident_bytes;
    sv->stats.resident_bytes = sv->resident;
    sv->note_peak();
    *id = (uint32_t)sv->scenes.size() - 1;
    return RT_OK;
}

RTCORE_API int32_t rt_server_submit(rt_server* sv, const RtServeRequest* r, uint64_t* ticket) {
    if (!sv || !r || !ticket) return RT_ERR_INVALID;
    if (r->width == 0 || r->height == 0 || (uint64_t)r->width * r->height > (1ull << 28) || r->max_trace_depth == 0 ||
        r->max_trace_depth > 64 || r->shadow_ray_count > 256 || (r->image_device & 3))
        return RT_ERR_INVALID;
    Request* q = new Request();
    q->req = *r;
    q->host_direct = !r->image_device && page_locked(r->image_host);
    q->frame_bytes = frame_bytes_of(*r, q->host_direct);
    q->t_submit = Clock::now();
    memset(&q->result, 0, sizeof q->result);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (r->scene >= sv->scenes.size()) {
            delete q;
            return RT_ERR_INVALID;
        }
        const uint64_t alone = q->frame_bytes + std::max(sv->workspace, batch_workspace(sv, {q}));
        if (sv->resident + alone > sv->cfg.hbm_budget_bytes) {
            delete q;
            sv->stats.rejected++;
            return RT_ERR_TOO_LARGE;
        }
        q->ticket = sv->next_ticket++;
        sv->tickets[q->ticket] = q;
        sv->queue.push_back(q);
        sv->stats.submitted++;
    }
    sv->cv.notify_all();
    *ticket = q->ticket;
    return RT_OK;
}

RTCORE_API int32_t rt_server_wait(rt_server* sv, uint64_t ticket, uint32_t timeout_ms, RtServeResult* out) {
    if (!sv || !out) return RT_ERR_INVALID;
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->tickets.find(ticket);
    if (it == sv->tickets.end()) return RT_ERR_INVALID;
    Request* q = it->second;
    const bool ok = sv->done_cv.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                                         [&] { return q->result.state != RT_SERVE_PENDING; });
    if (!ok) return RT_ERR_TIMEOUT;
    *out = q->result;
    sv->tickets.erase(it);
    delete q;
    return RT_OK;
}

RTCORE_API int32_t rt_server_stats(rt_server* sv, RtServeStats* out) {
    if (!sv || !out) return RT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(sv->mu);
    *out = sv->stats;
    out->resident_bytes = sv->resident;
    out->peak_bytes = sv->peak;
    out->budget_bytes = sv->cfg.hbm_budget_bytes;
    return RT_OK;
}

}  // extern "C"
