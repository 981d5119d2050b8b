// serve.cpp — request loop over a resident scene with continuous batching.
//
// The reference renders one frame at a time on one thread (src/Core/blitzenEntry.cpp:121-144) and
// updates dynamic objects by copying their transforms before each frame
// (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:46-60). The server turns that into a request loop:
//  - each request is one view to cull over the resident scene, with its own rotation of the
//    dynamic objects [0, rotateCount) applied into a private transform slab (the cull reads that
//    slab instead of the scene's rows), so a request's result depends only on the request;
//  - a worker thread admits waiting requests in arrival order while their worst-case output
//    (count * stride bytes, plus the slab) fits in the device output pool and an in-flight slot
//    is free, packs them into one batch launch, and keeps up to maxInFlight batches on the
//    device at once (one stream and one sub-context per slot, so their work overlaps);
//  - completion is observed with CUDA events; a request's output stays in the pool until the
//    client releases it, which is what frees memory for the next admissions.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/blz_cull.h"

namespace {

double now_seconds() {
    using clock = std::chrono::steady_clock;
    return std::chrono::duration<double>(clock::now().time_since_epoch()).count();
}

// First-fit allocator over one device region (offsets aligned to 256 bytes).
class Pool {
public:
    void reset(size_t bytes) {
        free_.clear();
        free_[0] = bytes;
        used_ = 0;
        peak_ = 0;
    }
    bool alloc(size_t bytes, size_t* off) {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, at = it->first + bytes;
                free_.erase(it);
                if (rest) free_[at] = rest;
                used_ += bytes;
                peak_ = std::max(peak_, used_);
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t peak() const { return peak_; }

private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0, peak_ = 0;
};

enum class ReqState { Pending, Running, Done };

struct Request {
    BlzServeRequest r{};
    std::vector<float> axes;
    BlzPyramid pyramid{};
    bool hasPyramid = false;
    ReqState state = ReqState::Pending;
    double arrival = 0, complete = 0;
    size_t off = 0, bytes = 0;       // pool range: records | count | slab | axes
    uint32_t status = BLZ_OK;
    uint32_t drawCount = 0;
    uint32_t objects = 0;
    std::vector<uint8_t> host;
    bool hostReady = false;
};

struct Slot {
    blz_ctx* ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t done = nullptr;
    bool busy = false;
    std::vector<uint64_t> tickets;
    uint32_t* hostCounts = nullptr;  // pinned, one per batched request
    float* hostAxes = nullptr;       // pinned staging for rotation axes
};

}  // namespace

struct blz_server {
    blz_ctx* main = nullptr;
    BlzServeConfig cfg{};
    BlzSceneDesc tables{};
    uint8_t* poolDev = nullptr;
    Pool pool;
    uint32_t* idsDev = nullptr;  // 0..dynamicCount-1
    std::vector<Slot> slots;
    std::mutex mu;
    std::condition_variable cvWork, cvDone;
    std::deque<uint64_t> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    uint64_t nextTicket = 1;
    bool stop = false;
    std::thread worker;
    // stats
    std::vector<double> latencies;
    uint64_t submitted = 0, completed = 0, batches = 0, objects = 0;
    uint32_t maxConcurrent = 0, maxBatch = 0;
    int device = 0;

    size_t request_bytes(const Request& q) const {
        const size_t rec = (size_t)q.objects * cfg.stride;
        const size_t slab = (size_t)q.r.rotateCount * sizeof(BlzMeshTransform);
        const size_t axes = (size_t)q.r.rotateCount * 3 * sizeof(float);
        return ((rec + 255) & ~size_t(255)) + 256 + ((slab + 255) & ~size_t(255)) + axes;
    }
    uint32_t* count_ptr(const Request& q) const {
        const size_t rec = (size_t)q.objects * cfg.stride;
        return reinterpret_cast<uint32_t*>(poolDev + q.off + ((rec + 255) & ~size_t(255)));
    }
    BlzMeshTransform* slab_ptr(const Request& q) const {
        return reinterpret_cast<BlzMeshTransform*>(reinterpret_cast<uint8_t*>(count_ptr(q)) + 256);
    }
    float* axes_ptr(const Request& q) const {
        const size_t slab = (size_t)q.r.rotateCount * sizeof(BlzMeshTransform);
        return reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(slab_ptr(q)) + ((slab + 255) & ~size_t(255)));
    }

    void finish_slot(Slot& s) {
        const double t = now_seconds();
        for (size_t k = 0; k < s.tickets.size(); ++k) {
            Request& q = *reqs[s.tickets[k]];
            q.drawCount = s.hostCounts[k];
            q.complete = t;
            q.state = ReqState::Done;
            if (q.drawCount > q.objects) q.status = BLZ_ERR_CAPACITY;
            latencies.push_back((q.complete - q.arrival) * 1e3);
            ++completed;
        }
        s.tickets.clear();
        s.busy = false;
        cvDone.notify_all();
    }

    // Launches one batch from the head of the queue on a free slot; returns false if nothing ran.
    bool launch_batch(Slot& s, std::unique_lock<std::mutex>& lk) {
        std::vector<uint64_t> take;
        while (!pending.empty() && take.size() < cfg.maxBatchViews) {
            Request& q = *reqs[pending.front()];
            if (!pool.alloc(q.bytes, &q.off)) break;  // admission by free output memory, in order
            take.push_back(pending.front());
            pending.pop_front();
        }
        if (take.empty()) return false;
        // the requests themselves, looked up while the lock is held: submissions may insert into
        // (and rehash) the map once it is released; running requests are never erased
        std::vector<Request*> reqOf(take.size());
        for (size_t k = 0; k < take.size(); ++k) reqOf[k] = reqs[take[k]].get();
        std::vector<BlzBatchView> views(take.size());
        for (size_t k = 0; k < take.size(); ++k) {
            Request& q = *reqOf[k];
            q.state = ReqState::Running;
            BlzBatchView& v = views[k];
            memset(&v, 0, sizeof v);
            v.view = q.r.view;
            v.list = q.r.list;
            v.mode = q.r.mode;
            v.pyramid = q.hasPyramid ? &q.pyramid : nullptr;
            v.target.commands = poolDev + q.off;
            v.target.stride = cfg.stride;
            v.target.capacity = q.objects;
            v.target.drawCount = count_ptr(q);
            v.dynamicTransforms = q.r.rotateCount ? slab_ptr(q) : nullptr;
            v.dynamicCount = q.r.rotateCount;
        }
        s.tickets = take;
        s.busy = true;
        ++batches;
        maxBatch = std::max<uint32_t>(maxBatch, (uint32_t)take.size());
        uint32_t running = 0;
        for (auto& o : slots) running += o.busy ? 1u : 0u;
        maxConcurrent = std::max(maxConcurrent, running);
        lk.unlock();
        // rotations of the dynamic objects into each request's slab
        size_t axesAt = 0;
        for (size_t k = 0; k < take.size(); ++k) {
            Request& q = *reqOf[k];
            if (!q.r.rotateCount) continue;
            memcpy(s.hostAxes + axesAt, q.axes.data(), q.axes.size() * sizeof(float));
            cudaMemcpyAsync(axes_ptr(q), s.hostAxes + axesAt, q.axes.size() * sizeof(float), cudaMemcpyHostToDevice, s.stream);
            blz_transforms_rotate(s.ctx, idsDev, axes_ptr(q), q.r.rotateAngle, q.r.rotateCount, slab_ptr(q),
                                  reinterpret_cast<blz_stream_t>(s.stream));
            axesAt += q.axes.size();
        }
        int rc = blz_cull_batch(s.ctx, views.data(), (uint32_t)views.size(), reinterpret_cast<blz_stream_t>(s.stream));
        for (size_t k = 0; k < take.size(); ++k) {
            Request& q = *reqOf[k];
            cudaMemcpyAsync(&s.hostCounts[k], count_ptr(q), sizeof(uint32_t), cudaMemcpyDeviceToHost, s.stream);
            if (rc != BLZ_OK) q.status = (uint32_t)rc;
        }
        cudaEventRecord(s.done, s.stream);
        lk.lock();
        return true;
    }

    void run() {
        cudaSetDevice(device);
        std::unique_lock<std::mutex> lk(mu);
        while (true) {
            bool progressed = false;
            for (auto& s : slots) {
                if (s.busy && cudaEventQuery(s.done) == cudaSuccess) {
                    finish_slot(s);
                    progressed = true;
                }
            }
            for (auto& s : slots) {
                if (!s.busy && !pending.empty()) progressed |= launch_batch(s, lk);
            }
            bool anyBusy = false;
            for (auto& s : slots) anyBusy |= s.busy;
            if (stop && !anyBusy) break;
            if (!progressed) {
                if (anyBusy) {
                    lk.unlock();
                    std::this_thread::sleep_for(std::chrono::microseconds(10));
                    lk.lock();
                } else {
                    cvWork.wait_for(lk, std::chrono::milliseconds(5));
                }
            }
        }
    }
};

extern "C" {

int blz_serve_create(blz_ctx* ctx, const BlzServeConfig* config, blz_server** out) {
    if (!ctx || !config || !out) return BLZ_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    BlzServeConfig cfg = *config;
    if (cfg.maxInFlight == 0) cfg.maxInFlight = 4;
    if (cfg.maxBatchViews == 0) cfg.maxBatchViews = 64;
    if (cfg.stride == 0) cfg.stride = BLZ_STRIDE_VULKAN;
    if (cfg.stride != BLZ_STRIDE_VULKAN && cfg.stride != BLZ_STRIDE_D3D12) return BLZ_ERR_INVALID_ARGUMENT;
    if (cfg.maxInFlight > 16 || cfg.maxBatchViews > 1024) return BLZ_ERR_INVALID_ARGUMENT;
    auto s = std::make_unique<blz_server>();
    s->main = ctx;
    int rc = blz_scene_device_tables(ctx, &s->tables);
    if (rc != BLZ_OK) return rc;
    if (cfg.dynamicCount > s->tables.transformCount) return BLZ_ERR_INVALID_ARGUMENT;
    cudaGetDevice(&s->device);
    if (cfg.outputPoolBytes == 0) {
        size_t fr = 0, tot = 0;
        cudaMemGetInfo(&fr, &tot);
        cfg.outputPoolBytes = fr / 4;
    }
    s->cfg = cfg;
    if (cudaMalloc(&s->poolDev, cfg.outputPoolBytes) != cudaSuccess) return BLZ_ERR_OUT_OF_MEMORY;
    s->pool.reset(cfg.outputPoolBytes);
    if (cfg.dynamicCount) {
        std::vector<uint32_t> ids(cfg.dynamicCount);
        for (uint32_t i = 0; i < cfg.dynamicCount; ++i) ids[i] = i;
        if (cudaMalloc(&s->idsDev, ids.size() * sizeof(uint32_t)) != cudaSuccess) {
            cudaFree(s->poolDev);
            return BLZ_ERR_OUT_OF_MEMORY;
        }
        cudaMemcpy(s->idsDev, ids.data(), ids.size() * sizeof(uint32_t), cudaMemcpyHostToDevice);
    }
    s->slots.resize(cfg.maxInFlight);
    for (auto& sl : s->slots) {
        rc = blz_ctx_create(s->device, &sl.ctx);
        if (rc == BLZ_OK) rc = blz_scene_upload(sl.ctx, &s->tables, BLZ_SCENE_BORROW_DEVICE, nullptr);
        if (rc == BLZ_OK) {
            BlzLaunchShape shape;
            blz_get_launch_shape(ctx, &shape);
            blz_set_launch_shape(sl.ctx, &shape);
        }
        if (rc == BLZ_OK && cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking) != cudaSuccess) rc = BLZ_ERR_CUDA;
        if (rc == BLZ_OK && cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess) rc = BLZ_ERR_CUDA;
        if (rc == BLZ_OK && cudaMallocHost(&sl.hostCounts, sizeof(uint32_t) * cfg.maxBatchViews) != cudaSuccess) rc = BLZ_ERR_OUT_OF_MEMORY;
        if (rc == BLZ_OK && cudaMallocHost(&sl.hostAxes, sizeof(float) * 3 * (size_t)(cfg.dynamicCount ? cfg.dynamicCount : 1) * cfg.maxBatchViews) != cudaSuccess)
            rc = BLZ_ERR_OUT_OF_MEMORY;
        if (rc != BLZ_OK) {
            blz_server* raw = s.release();
            raw->stop = true;
            blz_serve_destroy(raw);
            return rc;
        }
    }
    blz_server* raw = s.release();
    raw->worker = std::thread([raw] { raw->run(); });
    *out = raw;
    return BLZ_OK;
}

int blz_serve_submit(blz_server* s, const BlzServeRequest* r, uint64_t* ticketOut) {
    if (!s || !r) return BLZ_ERR_INVALID_ARGUMENT;
    if (r->mode != BLZ_MODE_FRUSTUM && r->mode != BLZ_MODE_TEMPORAL) return BLZ_ERR_INVALID_ARGUMENT;
    if (r->mode == BLZ_MODE_TEMPORAL && !r->pyramid) return BLZ_ERR_INVALID_ARGUMENT;
    if (r->rotateCount > s->cfg.dynamicCount || (r->rotateCount && !r->rotateAxes)) return BLZ_ERR_INVALID_ARGUMENT;
    auto q = std::make_unique<Request>();
    q->r = *r;
    q->arrival = now_seconds();
    q->objects = r->list.objects ? r->list.count : (r->list.count ? r->list.count : s->tables.renderObjectCount);
    if (!r->list.objects && q->objects > s->tables.renderObjectCount) return BLZ_ERR_INVALID_ARGUMENT;
    if (r->pyramid) {
        q->pyramid = *r->pyramid;
        q->hasPyramid = true;
        q->r.pyramid = nullptr;
    }
    if (r->rotateCount) q->axes.assign(r->rotateAxes, r->rotateAxes + 3 * (size_t)r->rotateCount);
    q->r.rotateAxes = nullptr;
    q->bytes = s->request_bytes(*q);
    if (q->bytes > s->cfg.outputPoolBytes) return BLZ_ERR_CAPACITY;
    std::lock_guard<std::mutex> lk(s->mu);
    const uint64_t t = s->nextTicket++;
    s->reqs[t] = std::move(q);
    s->pending.push_back(t);
    ++s->submitted;
    if (ticketOut) *ticketOut = t;
    s->cvWork.notify_one();
    return BLZ_OK;
}

int blz_serve_wait(blz_server* s, uint64_t ticket, uint32_t timeoutMs, BlzServeResult* out) {
    if (!s || !out) return BLZ_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return BLZ_ERR_INVALID_ARGUMENT;
    Request& q = *it->second;
    const bool ok = s->cvDone.wait_for(lk, std::chrono::milliseconds(timeoutMs), [&] { return q.state == ReqState::Done; });
    if (!ok) return timeoutMs ? BLZ_ERR_TIMEOUT : BLZ_ERR_NOT_READY;
    if (q.r.copyToHost && !q.hostReady) {
        const size_t n = (size_t)std::min(q.drawCount, q.objects) * s->cfg.stride;
        q.host.resize(n);
        if (n) cudaMemcpy(q.host.data(), s->poolDev + q.off, n, cudaMemcpyDeviceToHost);
        q.hostReady = true;
    }
    out->status = q.status;
    out->drawCount = q.drawCount;
    out->deviceRecords = s->poolDev + q.off;
    out->hostRecords = q.hostReady ? q.host.data() : nullptr;
    out->arrivalSeconds = q.arrival;
    out->completeSeconds = q.complete;
    return BLZ_OK;
}

int blz_serve_release(blz_server* s, uint64_t ticket) {
    if (!s) return BLZ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return BLZ_ERR_INVALID_ARGUMENT;
    if (it->second->state != ReqState::Done) return BLZ_ERR_NOT_READY;
    s->objects += it->second->objects;
    s->pool.release(it->second->off, it->second->bytes);
    s->reqs.erase(it);
    s->cvWork.notify_one();
    return BLZ_OK;
}

int blz_serve_stats(blz_server* s, BlzServeStats* out) {
    if (!s || !out) return BLZ_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    memset(out, 0, sizeof *out);
    out->submitted = s->submitted;
    out->completed = s->completed;
    out->batches = s->batches;
    out->objects = s->objects;
    out->peakOutputBytes = s->pool.peak();
    out->maxConcurrentBatches = s->maxConcurrent;
    out->maxBatchSize = s->maxBatch;
    if (!s->latencies.empty()) {
        std::vector<double> v = s->latencies;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (double)(v.size() - 1) + 0.5))]; };
        out->p50Ms = pct(0.50);
        out->p99Ms = pct(0.99);
        double sum = 0;
        for (double x : v) sum += x;
        out->meanMs = sum / (double)v.size();
        out->maxMs = v.back();
    }
    return BLZ_OK;
}

int blz_serve_destroy(blz_server* s) {
    if (!s) return BLZ_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->pending.clear();
        s->cvWork.notify_all();
    }
    if (s->worker.joinable()) s->worker.join();
    for (auto& sl : s->slots) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);
        if (sl.done) cudaEventDestroy(sl.done);
        if (sl.stream) cudaStreamDestroy(sl.stream);
        if (sl.hostCounts) cudaFreeHost(sl.hostCounts);
        if (sl.hostAxes) cudaFreeHost(sl.hostAxes);
        if (sl.ctx) blz_ctx_destroy(sl.ctx);
    }
    if (s->idsDev) cudaFree(s->idsDev);
    if (s->poolDev) cudaFree(s->poolDev);
    delete s;
    return BLZ_OK;
}

}  // extern "C"
