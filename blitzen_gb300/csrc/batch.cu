// batch.cu — many views in one launch, its per-view baseline, CUDA-graph replay, recorded frames
// and the launch-shape autotuner.
//
// The reference culls one camera per pass with one dispatch each (src/Core/blitzenEngine.h:49,
// src/Renderer/BlitzenVulkan/vulkanDraw.cpp:107-226). Here every (view, chunk) pair is an item of
// one decide launch (chunks of 256, 512 or 1024 objects, the launch shape's chunk size): warps start on the chunk of their index and take further chunks
// from a work counter, and the scatter launch turns the per-chunk counts into per-view offsets and
// draw counts, so views of 1k and 2M objects share the machine without a launch or a tail per view.
#include <algorithm>
#include <cstddef>
#include <cstring>
#include <vector>

#include "api_internal.h"

namespace blz {

// Objects per chunk of a batch launch shape (0: the default).
static uint32_t batch_chunk(const BlzLaunchShape& s) { return s.chunkObjects ? s.chunkObjects : object_tile_size(); }

static bool chunk_supported(uint32_t chunk) { return chunk == 0 || chunk == 256 || chunk == 512 || chunk == 1024; }

const TunedShape* find_tuned(const blz_ctx* c, uint64_t objects, uint32_t views, uint32_t mode) {
    for (const TunedShape& t : c->tuned)
        if (t.objects == objects && t.views == views && t.mode == mode) return &t;
    return nullptr;
}

void remember_tuned(blz_ctx* c, const TunedShape& t) {
    for (TunedShape& u : c->tuned)
        if (u.objects == t.objects && u.views == t.views && u.mode == t.mode) {
            u = t;
            return;
        }
    c->tuned.push_back(t);
}

// Total objects of a batch (each view's list, or the scene's when the list is NULL).
static uint64_t batch_objects(const blz_ctx* c, const BlzBatchView* views, uint32_t n) {
    uint64_t total = 0;
    for (uint32_t i = 0; i < n; ++i) total += views[i].list.objects ? views[i].list.count : c->defaultCount;
    return total;
}

// The shape a batch of these views runs with: the autotuner's choice for its size, else the context's.
static BlzLaunchShape batch_shape(const blz_ctx* c, const BlzBatchView* views, uint32_t n) {
    const TunedShape* t = find_tuned(c, batch_objects(c, views, n), n, kTunedBatch);
    return t ? t->shape : c->shape;
}

static int build_views(blz_ctx* c, const BlzBatchView* views, uint32_t n, uint32_t tile, std::vector<BatchViewDev>& out,
                       std::vector<uint32_t>& tileStart) {
    out.resize(n);
    tileStart.resize(n + 1);
    uint64_t at = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const BlzBatchView& v = views[i];
        if (v.mode > BLZ_MODE_TEMPORAL) return fail(BLZ_ERR_INVALID_ARGUMENT, "view %u: unknown mode %u", i, v.mode);
        int rc = check_target(&v.target);
        if (rc != BLZ_OK) return rc;
        const BlzRenderObject* objs = nullptr;
        uint32_t count = 0;
        rc = resolve_list(c, v.list, &objs, &count);
        if (rc != BLZ_OK) return rc;
        if ((v.mode == BLZ_MODE_FIRST || v.mode == BLZ_MODE_LATE) && count && !v.visibility)
            return fail(BLZ_ERR_INVALID_ARGUMENT, "view %u: visibility buffer is NULL", i);
        if (v.mode == BLZ_MODE_LATE || v.mode == BLZ_MODE_TEMPORAL) {
            rc = check_pyramid(v.pyramid, true);
            if (rc != BLZ_OK) return rc;
        }
        if (v.dynamicCount && !v.dynamicTransforms) return fail(BLZ_ERR_INVALID_ARGUMENT, "view %u: dynamic transforms are NULL", i);
        if (reinterpret_cast<uintptr_t>(v.dynamicTransforms) % 32)
            return fail(BLZ_ERR_INVALID_ARGUMENT, "view %u: dynamic transforms must be 32-byte aligned", i);
        BatchViewDev d{};
        d.view = v.view;
        d.objects = objs;
        d.count = count;
        d.mode = v.mode;
        d.vis = v.visibility;
        d.pyr = pyramid_view(v.pyramid);
        d.cmds = static_cast<uint8_t*>(v.target.commands);
        d.stride = v.target.stride;
        d.capacity = v.target.capacity;
        d.drawCount = v.target.drawCount;
        d.dynT = v.dynamicTransforms;
        d.dynCount = v.dynamicCount;
        out[i] = d;
        tileStart[i] = static_cast<uint32_t>(at);
        uint64_t tiles = (count + tile - 1) / tile;
        if (tiles == 0) tiles = 1;  // an empty view still gets one item that writes drawCount = 0
        at += tiles;
    }
    if (at >= (1ull << 32)) return fail(BLZ_ERR_CAPACITY, "batch has too many tiles");
    tileStart[n] = static_cast<uint32_t>(at);
    return BLZ_OK;
}

static size_t batch_bytes(uint32_t n) { return sizeof(BatchViewDev) * n + sizeof(uint32_t) * (n + 1) + 256; }

static int upload_views(blz_ctx* c, const std::vector<BatchViewDev>& d, const std::vector<uint32_t>& ts, void* dst,
                        cudaStream_t st, uint32_t tile, PipeParams& p) {
    const uint32_t n = static_cast<uint32_t>(d.size());
    const size_t viewsBytes = sizeof(BatchViewDev) * n;
    const size_t tsOff = (viewsBytes + 255) & ~size_t(255);
    const size_t total = tsOff + sizeof(uint32_t) * (n + 1);
    if (total > kPinnedBytes) return fail(BLZ_ERR_CAPACITY, "%u views exceed the staging buffer", n);
    cudaEventSynchronize(c->pinnedDone);
    char* h = static_cast<char*>(c->pinned);
    memcpy(h, d.data(), viewsBytes);
    memcpy(h + tsOff, ts.data(), sizeof(uint32_t) * (n + 1));
    cudaError_t e = cudaMemcpyAsync(dst, h, total, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaEventRecord(c->pinnedDone, st);
    if (e != cudaSuccess) return cuda_fail(e, "batch view upload");
    p = PipeParams{};
    p.sc = c->scene;
    p.views = static_cast<const BatchViewDev*>(dst);
    p.tileStart = reinterpret_cast<const uint32_t*>(static_cast<char*>(dst) + tsOff);
    p.viewCount = n;
    p.totalTiles = ts[n];
    p.chunkSize = tile;
    p.scratch = c->scratch;
    return BLZ_OK;
}

static int ensure_batch_dev(blz_ctx* c, size_t bytes) {
    if (bytes <= c->batchBytes) return BLZ_OK;
    if (c->batchDev) {
        cudaDeviceSynchronize();
        cudaFree(c->batchDev);
        c->batchDev = nullptr;
        c->batchBytes = 0;
    }
    size_t want = bytes < (size_t(1) << 20) ? (size_t(1) << 20) : bytes;
    if (cudaMalloc(&c->batchDev, want) != cudaSuccess) return fail(BLZ_ERR_OUT_OF_MEMORY, "batch workspace allocation failed");
    c->batchBytes = want;
    return BLZ_OK;
}

// The pass all views run, or -1 when they differ.
static int uniform_mode(const BlzBatchView* views, uint32_t n) {
    for (uint32_t i = 1; i < n; ++i)
        if (views[i].mode != views[0].mode) return -1;
    return n ? static_cast<int>(views[0].mode) : -1;
}

static int run_batch_shape(blz_ctx* c, const BlzBatchView* views, uint32_t n, cudaStream_t st, const BlzLaunchShape& sh) {
    const uint32_t tile = batch_chunk(sh);
    std::vector<BatchViewDev> d;
    std::vector<uint32_t> ts;
    int rc = build_views(c, views, n, tile, d, ts);
    if (rc != BLZ_OK) return rc;
    rc = ensure_batch_dev(c, batch_bytes(n));
    if (rc != BLZ_OK) return rc;
    rc = ensure_chunk_scratch(c, ts[n], tile);
    if (rc != BLZ_OK) return rc;
    PipeParams p{};
    rc = upload_views(c, d, ts, c->batchDev, st, tile, p);
    if (rc != BLZ_OK) return rc;
    bind_chunk_scratch(c, p);
    cudaError_t e = launch_batch_cull(p, sh.threadsPerBlock, sh.objectsPerThread, sh.blocksPerSm, c->smCount, st,
                                      uniform_mode(views, n));
    if (e != cudaSuccess) return cuda_fail(e, "batch launch");
    c->launches += 2;  // decide + scatter
    return BLZ_OK;
}

int run_batch(blz_ctx* c, const BlzBatchView* views, uint32_t n, cudaStream_t st) {
    if (!c || (n && !views)) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or views is NULL");
    if (n == 0) return BLZ_OK;
    return run_batch_shape(c, views, n, st, batch_shape(c, views, n));
}

}  // namespace blz

using namespace blz;

struct blz_batch_graph {
    blz_ctx* ctx = nullptr;
    void* viewsDev = nullptr;
    void* chunkMem = nullptr;  // the graph's own staging scratch (a context's may be reallocated)
    uint32_t viewCount = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct blz_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    uint32_t kernels = 0;
    blz_ctx* ctx = nullptr;
};

extern "C" {

int blz_capture_begin(blz_ctx* c, blz_stream_t stream) {
    if (!c || !stream) return fail(BLZ_ERR_INVALID_ARGUMENT, "capture needs a context and a non-default stream");
    if (c->capturing) return fail(BLZ_ERR_INVALID_ARGUMENT, "a capture is already open on this context");
    cudaError_t e = cudaStreamBeginCapture(reinterpret_cast<cudaStream_t>(stream), cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamBeginCapture");
    c->capturing = true;
    c->launchesAtCapture = c->launches.load();
    return BLZ_OK;
}

int blz_capture_end(blz_ctx* c, blz_stream_t stream, blz_graph** out, uint32_t* kernelsOut) {
    if (!c || !out) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or out is NULL");
    *out = nullptr;
    if (!c->capturing) return fail(BLZ_ERR_INVALID_ARGUMENT, "no capture is open on this context");
    c->capturing = false;
    blz_graph* g = new blz_graph();
    g->ctx = c;
    g->kernels = static_cast<uint32_t>(c->launches.load() - c->launchesAtCapture);
    cudaError_t e = cudaStreamEndCapture(reinterpret_cast<cudaStream_t>(stream), &g->graph);
    if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
    if (e != cudaSuccess) {
        blz_graph_destroy(g);
        return cuda_fail(e, "capture end");
    }
    if (kernelsOut) *kernelsOut = g->kernels;
    *out = g;
    return BLZ_OK;
}

int blz_graph_launch(blz_graph* g, blz_stream_t stream) {
    if (!g || !g->exec) return fail(BLZ_ERR_INVALID_ARGUMENT, "graph is NULL");
    cudaError_t e = cudaGraphLaunch(g->exec, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    g->ctx->launches += g->kernels;
    return BLZ_OK;
}

int blz_graph_destroy(blz_graph* g) {
    if (!g) return BLZ_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return BLZ_OK;
}

int blz_cull_batch(blz_ctx* c, const BlzBatchView* views, uint32_t n, blz_stream_t stream) {
    return run_batch(c, views, n, reinterpret_cast<cudaStream_t>(stream));
}

int blz_cull_batch_per_view(blz_ctx* c, const BlzBatchView* views, uint32_t n, blz_stream_t stream) {
    if (!c || (n && !views)) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or views is NULL");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    std::vector<BatchViewDev> d;
    std::vector<uint32_t> ts;
    const uint32_t tile = batch_chunk(batch_shape(c, views, n));
    int rc = build_views(c, views, n, tile, d, ts);
    if (rc != BLZ_OK) return rc;
    uint32_t maxTiles = 1;
    for (uint32_t i = 0; i < n; ++i) maxTiles = std::max(maxTiles, ts[i + 1] - ts[i]);
    rc = ensure_chunk_scratch(c, maxTiles, tile);
    if (rc != BLZ_OK) return rc;
    for (uint32_t i = 0; i < n; ++i) {
        PipeParams p{};
        p.sc = c->scene;
        p.single = d[i];
        p.views = nullptr;
        p.tileStart = nullptr;
        p.viewCount = 1;
        p.totalTiles = ts[i + 1] - ts[i];
        p.chunkSize = tile;
        bind_chunk_scratch(c, p);
        cudaError_t e = launch_object_cull(d[i].mode, p, c->singleThreads, c->singleOpt, c->smCount, st);
        if (e != cudaSuccess) return cuda_fail(e, "per-view cull launch");
        c->launches += 2;
    }
    return BLZ_OK;
}

int blz_get_launch_shape(const blz_ctx* c, BlzLaunchShape* out) {
    if (!c || !out) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or out is NULL");
    *out = c->shape;
    return BLZ_OK;
}

int blz_set_launch_shape(blz_ctx* c, const BlzLaunchShape* s) {
    if (!c || !s) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or shape is NULL");
    if (!batch_shape_supported(s->threadsPerBlock, s->objectsPerThread))
        return fail(BLZ_ERR_INVALID_ARGUMENT, "unsupported launch shape %u x %u", s->threadsPerBlock, s->objectsPerThread);
    if (!chunk_supported(s->chunkObjects))
        return fail(BLZ_ERR_INVALID_ARGUMENT, "unsupported chunk size %u (256, 512, 1024 or 0)", s->chunkObjects);
    c->shape = *s;
    c->tuned.clear();  // an explicit shape wins over every cached choice
    if (single_shape_supported(s->threadsPerBlock, s->objectsPerThread)) {
        c->singleThreads = s->threadsPerBlock;
        c->singleOpt = s->objectsPerThread;
    }
    return BLZ_OK;
}

int blz_autotune_batch(blz_ctx* c, const BlzBatchView* views, uint32_t n, uint32_t repeats, blz_stream_t stream,
                       BlzLaunchShape* best, float* bestUs) {
    if (!c || !views || n == 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or views is NULL");
    if (c->capturing) return fail(BLZ_ERR_INVALID_ARGUMENT, "the autotuner cannot run inside a capture");
    const uint64_t objects = batch_objects(c, views, n);
    if (const TunedShape* t = find_tuned(c, objects, n, kTunedBatch)) {
        c->shape = t->shape;
        if (best) *best = t->shape;
        if (bestUs) *bestUs = t->us;
        return BLZ_OK;
    }
    if (repeats == 0) repeats = 5;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const uint32_t threads[] = {128, 256, 512};
    const uint32_t opts[] = {1, 2, 4, 8};
    const uint32_t perSm[] = {0, 1, 2, 4};
    const uint32_t chunks[] = {256, 512, 1024};
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    BlzLaunchShape top = c->shape;
    float topUs = 1e30f;
    for (uint32_t t : threads)
        for (uint32_t o : opts)
            for (uint32_t s : perSm)
                for (uint32_t k : chunks) {
                    if (s && s * t > 2048) continue;
                    if (!batch_shape_supported(t, o)) continue;
                    const BlzLaunchShape sh{t, o, s, k};
                    if (run_batch_shape(c, views, n, st, sh) != BLZ_OK) continue;  // warm-up
                    cudaEventRecord(a, st);
                    int rc = BLZ_OK;
                    for (uint32_t r = 0; r < repeats && rc == BLZ_OK; ++r) rc = run_batch_shape(c, views, n, st, sh);
                    cudaEventRecord(b, st);
                    cudaEventSynchronize(b);
                    if (rc != BLZ_OK) continue;
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, a, b);
                    const float us = ms * 1000.f / static_cast<float>(repeats);
                    if (us < topUs) {
                        topUs = us;
                        top = sh;
                    }
                }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (!(topUs < 1e30f)) return fail(BLZ_ERR_CUDA, "no launch shape ran");
    c->shape = top;
    remember_tuned(c, TunedShape{objects, n, kTunedBatch, top, topUs});
    if (best) *best = top;
    if (bestUs) *bestUs = topUs;
    return BLZ_OK;
}

int blz_batch_graph_create(blz_ctx* c, const BlzBatchView* views, uint32_t n, blz_stream_t stream, blz_batch_graph** outGraph) {
    if (!c || !views || n == 0 || !outGraph) return fail(BLZ_ERR_INVALID_ARGUMENT, "bad batch graph arguments");
    *outGraph = nullptr;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const BlzLaunchShape sh = batch_shape(c, views, n);
    const uint32_t tile = batch_chunk(sh);
    std::vector<BatchViewDev> d;
    std::vector<uint32_t> ts;
    int rc = build_views(c, views, n, tile, d, ts);
    if (rc != BLZ_OK) return rc;
    blz_batch_graph* g = new blz_batch_graph();
    g->ctx = c;
    g->viewCount = n;
    if (cudaMalloc(&g->viewsDev, batch_bytes(n)) != cudaSuccess) {
        delete g;
        return fail(BLZ_ERR_OUT_OF_MEMORY, "batch graph workspace allocation failed");
    }
    PipeParams p{};
    rc = upload_views(c, d, ts, g->viewsDev, st, tile, p);
    if (rc == BLZ_OK && cudaStreamSynchronize(st) != cudaSuccess) rc = fail(BLZ_ERR_CUDA, "batch graph upload failed");
    if (rc == BLZ_OK) {
        const size_t chunks = ts[n], objects = chunks * tile;
        const size_t bytes = objects * sizeof(uint2) + chunks * sizeof(uint32_t) + 256;
        if (cudaMalloc(&g->chunkMem, bytes) != cudaSuccess || cudaMemset(g->chunkMem, 0, bytes) != cudaSuccess) {
            rc = fail(BLZ_ERR_OUT_OF_MEMORY, "batch graph scratch allocation failed");
        } else {
            char* m = static_cast<char*>(g->chunkMem);
            p.staged = reinterpret_cast<uint2*>(m);
            p.chunkCount = reinterpret_cast<uint32_t*>(m + objects * sizeof(uint2));
            p.workCounter = reinterpret_cast<unsigned int*>(p.chunkCount + chunks);  // zeroed above
            p.scratch = c->scratch;
        }
    }
    cudaStream_t cap = nullptr;
    if (rc == BLZ_OK) {
        cudaError_t e = cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking);
        if (e == cudaSuccess) e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
        if (e == cudaSuccess) {
            cudaError_t le = launch_batch_cull(p, sh.threadsPerBlock, sh.objectsPerThread, sh.blocksPerSm, c->smCount, cap,
                                               uniform_mode(views, n));
            e = cudaStreamEndCapture(cap, &g->graph);
            if (le != cudaSuccess) e = le;
        }
        if (e == cudaSuccess) e = cudaGraphInstantiate(&g->exec, g->graph, 0);
        if (cap) cudaStreamDestroy(cap);
        if (e != cudaSuccess) rc = cuda_fail(e, "batch graph capture");
    }
    if (rc != BLZ_OK) {
        blz_batch_graph_destroy(g);
        return rc;
    }
    *outGraph = g;
    return BLZ_OK;
}

int blz_batch_graph_set_view(blz_batch_graph* g, uint32_t i, const BlzCameraViewData* view) {
    if (!g || !view || i >= g->viewCount) return fail(BLZ_ERR_INVALID_ARGUMENT, "bad batch graph view update");
    char* dst = static_cast<char*>(g->viewsDev) + sizeof(BatchViewDev) * i + offsetof(BatchViewDev, view);
    cudaError_t e = cudaMemcpy(dst, view, sizeof(BlzCameraViewData), cudaMemcpyHostToDevice);
    return e == cudaSuccess ? BLZ_OK : cuda_fail(e, "batch graph view update");
}

int blz_batch_graph_launch(blz_batch_graph* g, blz_stream_t stream) {
    if (!g || !g->exec) return fail(BLZ_ERR_INVALID_ARGUMENT, "graph is NULL");
    cudaError_t e = cudaGraphLaunch(g->exec, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "graph launch");
    g->ctx->launches += 2;
    return BLZ_OK;
}

int blz_batch_graph_destroy(blz_batch_graph* g) {
    if (!g) return BLZ_OK;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    if (g->viewsDev || g->chunkMem) cudaDeviceSynchronize();
    if (g->viewsDev) cudaFree(g->viewsDev);
    if (g->chunkMem) cudaFree(g->chunkMem);
    delete g;
    return BLZ_OK;
}

}  // extern "C"
