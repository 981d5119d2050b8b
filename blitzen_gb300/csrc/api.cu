// api.cu — the C ABI of libblz_cull.so: context, scene residency, pyramid, culls, batches.
//
// Host-side counterpart of the reference's cull dispatch code: the renderer members and static
// dispatch helpers of src/Renderer/BlitzenVulkan/vulkanDraw.cpp:107-622 and
// src/Renderer/BlitzenDX12/dx12Draw.cpp:114-415, without the graphics API around them.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "api_internal.h"

namespace blz {

thread_local std::string g_lastError;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_lastError = buf;
    return code;
}

int cuda_fail(cudaError_t e, const char* what) {
    return fail(BLZ_ERR_CUDA, "%s: %s (%s)", what, cudaGetErrorName(e), cudaGetErrorString(e));
}

static void release_scene(blz_ctx* c) {
    for (void* p : c->ownedScene) cudaFree(p);
    c->ownedScene.clear();
    c->scene = SceneT{};
    c->defaultObjects = nullptr;
    c->defaultCount = 0;
    c->hasScene = false;
}

SceneT scene_tables(const blz_ctx* c) { return c->scene; }

PyramidT pyramid_view(const BlzPyramid* p) {
    PyramidT v{};
    if (!p) return v;
    v.data = p->data;
    v.width = p->width;
    v.height = p->height;
    v.mipCount = p->mipCount;
    v.mode = p->mode;
    for (uint32_t i = 0; i < BLZ_PYRAMID_MAX_MIPS; ++i) v.mipOffset[i] = p->mipOffset[i];
    return v;
}

int check_pyramid(const BlzPyramid* p, bool required) {
    if (!p) return required ? fail(BLZ_ERR_INVALID_ARGUMENT, "a pyramid is required for this pass") : BLZ_OK;
    if (!p->data) return fail(BLZ_ERR_INVALID_ARGUMENT, "pyramid has no storage");
    if (p->mipCount == 0 || p->mipCount > BLZ_PYRAMID_MAX_MIPS) return fail(BLZ_ERR_INVALID_ARGUMENT, "pyramid mipCount %u out of range", p->mipCount);
    if (p->mode > BLZ_HIZ_VULKAN) return fail(BLZ_ERR_INVALID_ARGUMENT, "unknown pyramid mode %u", p->mode);
    if (p->width == 0 || p->height == 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "pyramid extent is zero");
    return BLZ_OK;
}

int check_target(const BlzCullTarget* t) {
    if (!t) return fail(BLZ_ERR_INVALID_ARGUMENT, "target is NULL");
    if (t->stride != BLZ_STRIDE_VULKAN && t->stride != BLZ_STRIDE_D3D12)
        return fail(BLZ_ERR_INVALID_ARGUMENT, "record stride must be 24 or 32, got %u", t->stride);
    if (!t->drawCount) return fail(BLZ_ERR_INVALID_ARGUMENT, "target drawCount is NULL");
    if (t->capacity > 0 && !t->commands) return fail(BLZ_ERR_INVALID_ARGUMENT, "target commands is NULL");
    if (reinterpret_cast<uintptr_t>(t->commands) % 16 != 0)
        return fail(BLZ_ERR_INVALID_ARGUMENT, "target commands must be 16-byte aligned");
    return BLZ_OK;
}

int resolve_list(const blz_ctx* c, BlzRenderList list, const BlzRenderObject** objs, uint32_t* count) {
    if (!c->hasScene) return fail(BLZ_ERR_NO_SCENE, "no scene uploaded");
    if (list.objects) {
        *objs = list.objects;
        *count = list.count;
    } else {
        *objs = c->defaultObjects;
        *count = list.count ? list.count : c->defaultCount;
        if (*count > c->defaultCount) return fail(BLZ_ERR_INVALID_ARGUMENT, "render list count %u exceeds the scene's %u", *count, c->defaultCount);
    }
    if (*count > 0 && !*objs) return fail(BLZ_ERR_INVALID_ARGUMENT, "render list has no objects");
    if (reinterpret_cast<uintptr_t>(*objs) % 8 != 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "render list must be 8-byte aligned");
    if (*count >= (1u << 30)) return fail(BLZ_ERR_INVALID_ARGUMENT, "render list count %u exceeds 2^30", *count);
    return BLZ_OK;
}

int ensure_chunk_scratch(blz_ctx* c, size_t chunks, size_t chunkSize) {
    const size_t objects = chunks * chunkSize;
    if (objects <= c->chunkObjects && chunks <= c->chunkSlots) return BLZ_OK;
    if (c->capturing) return fail(BLZ_ERR_CAPACITY, "scratch must grow, which a capture cannot record: run the calls once before capturing");
    size_t wantObj = objects > c->chunkObjects ? objects + objects / 4 : c->chunkObjects;
    size_t wantSlots = chunks > c->chunkSlots ? chunks + chunks / 4 + 64 : c->chunkSlots;
    if (c->chunkMem) {
        cudaDeviceSynchronize();
        cudaFree(c->chunkMem);
        c->chunkMem = nullptr;
        c->chunkObjects = c->chunkSlots = 0;
    }
    const size_t bytes = wantObj * sizeof(uint2) + wantSlots * sizeof(uint32_t) + 256;
    if (cudaMalloc(&c->chunkMem, bytes) != cudaSuccess) return fail(BLZ_ERR_OUT_OF_MEMORY, "object-cull scratch of %zu bytes", bytes);
    c->chunkObjects = wantObj;
    c->chunkSlots = wantSlots;
    return BLZ_OK;
}

// Cluster-cull scratch for `tiles` tiles. First the work list's item count (zero between launches:
// zeroed when allocated, rewound by the emit launch) and the frame's totals. Then, laid out for this
// call's tile count: counts per tile (uint2), candidates per tile, the objects' cluster ranges, transforms and survivor counts, the
// work list, and the visibility bits (bitWords per tile). Grown on demand like the object-cull
// scratch.
int bind_cluster_scratch(blz_ctx* c, uint32_t tiles, ClusterParams& p) {
    const size_t objs = static_cast<size_t>(tiles) * cluster_tile_objects();
    const uint32_t bitWords = std::max<uint32_t>(c->lodClusterMax, 1u);  // 32 objects x max clusters / 32 bits
    auto r256 = [](size_t b) { return (b + 255) & ~size_t(255); };
    const size_t headBytes = 256;
    const size_t countBytes = r256(static_cast<size_t>(tiles) * sizeof(uint2));
    const size_t superBytes = r256(static_cast<size_t>(cluster_tile_groups(tiles)) * sizeof(uint2));
    const size_t tileBytes = r256(static_cast<size_t>(tiles) * sizeof(uint32_t));
    const size_t infoBytes = r256(objs * sizeof(uint2));
    const size_t xfBytes = r256(objs * 2 * sizeof(float4));
    const size_t survBytes = r256(objs * sizeof(uint32_t));
    const size_t itemBytes = r256(static_cast<size_t>(cluster_max_items(tiles, bitWords)) * sizeof(uint4));
    const size_t bitBytes = static_cast<size_t>(tiles) * bitWords * sizeof(uint32_t);
    const size_t need = headBytes + countBytes + superBytes + tileBytes + infoBytes + xfBytes + survBytes + itemBytes + bitBytes;
    if (need > c->clusterBytes) {
        if (c->capturing) return fail(BLZ_ERR_CAPACITY, "scratch must grow, which a capture cannot record: run the call once before capturing");
        if (c->clusterMem) {
            cudaDeviceSynchronize();
            cudaFree(c->clusterMem);
            c->clusterMem = nullptr;
            c->clusterBytes = 0;
        }
        const size_t want = need + need / 4;
        if (cudaMalloc(&c->clusterMem, want) != cudaSuccess)
            return fail(BLZ_ERR_OUT_OF_MEMORY, "cluster-cull scratch of %zu bytes", want);
        const cudaError_t e = cudaMemset(c->clusterMem, 0, headBytes);  // the work list's counts start at zero
        if (e != cudaSuccess) {
            cudaFree(c->clusterMem);
            c->clusterMem = nullptr;
            return cuda_fail(e, "zeroing the cluster-cull scratch");
        }
        c->clusterBytes = want;
    }
    char* m = static_cast<char*>(c->clusterMem);
    p.itemCount = reinterpret_cast<uint32_t*>(m);
    p.totals = reinterpret_cast<uint2*>(m + 8);
    m += headBytes;
    p.tileCount = reinterpret_cast<uint32_t*>(m);
    m += countBytes;
    p.superCount = reinterpret_cast<uint2*>(m);
    m += superBytes;
    p.tileSlots = reinterpret_cast<uint32_t*>(m);
    m += tileBytes;
    p.objInfo = reinterpret_cast<uint2*>(m);
    m += infoBytes;
    p.objXf = reinterpret_cast<float4*>(m);
    m += xfBytes;
    p.objSurv = reinterpret_cast<uint32_t*>(m);
    m += survBytes;
    p.items = reinterpret_cast<uint4*>(m);
    p.itemCapacity = static_cast<uint32_t>(std::min<uint64_t>(cluster_max_items(tiles, bitWords), 0xFFFFFFFFu));
    m += itemBytes;
    p.bits = reinterpret_cast<uint32_t*>(m);
    p.bitWords = bitWords;
    p.tiles = tiles;
    p.smCount = static_cast<uint32_t>(c->smCount);
    return BLZ_OK;
}

// The cluster test kernel's resident blocks per SM for the records (tasks false) or task form, found
// on the context's first call of that form (which allocates the cluster scratch, so it never runs
// inside a capture) and kept in the context.
int cluster_test_occupancy(blz_ctx* c, bool tasks, ClusterParams& p) {
    int& n = c->clusterTestBlocksPerSm[tasks ? 1 : 0];
    if (n == 0) {
        const cudaError_t e = cluster_test_blocks_per_sm(tasks, &n);
        if (e != cudaSuccess) {
            n = 0;
            return cuda_fail(e, "cluster test kernel occupancy");
        }
    }
    p.testBlocksPerSm = static_cast<uint32_t>(n);
    return BLZ_OK;
}

void bind_chunk_scratch(blz_ctx* c, PipeParams& p) {
    char* m = static_cast<char*>(c->chunkMem);
    p.staged = reinterpret_cast<uint2*>(m);
    p.chunkCount = reinterpret_cast<uint32_t*>(m + c->chunkObjects * sizeof(uint2));
    p.workCounter = c->workCounter;
    p.scratch = c->scratch;
}

int ensure_states(blz_ctx* c, size_t states) {
    if (states <= c->stateCapacity) return BLZ_OK;
    return fail(BLZ_ERR_CAPACITY, "%zu tile states needed, the context holds %zu", states, c->stateCapacity);
}

}  // namespace blz

using namespace blz;

extern "C" {

const char* blz_last_error(void) { return g_lastError.c_str(); }

const char* blz_version(void) { return "blz_cull 0.1 (sm_103a)"; }

int blz_ctx_create(int device, blz_ctx** out) {
    if (!out) return fail(BLZ_ERR_INVALID_ARGUMENT, "outCtx is NULL");
    *out = nullptr;
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    blz_ctx* c = new blz_ctx();
    c->device = device;
    cudaDeviceGetAttribute(&c->smCount, cudaDevAttrMultiProcessorCount, device);
    c->stateCapacity = kDefaultStateCapacity;
    const size_t bytes = kScratchHeaderBytes + c->stateCapacity * sizeof(unsigned long long);
    e = cudaMalloc(&c->scratchMem, bytes);
    if (e != cudaSuccess) { delete c; return e == cudaErrorMemoryAllocation ? fail(BLZ_ERR_OUT_OF_MEMORY, "scratch allocation failed") : cuda_fail(e, "cudaMalloc scratch"); }
    e = cudaMemset(c->scratchMem, 0, bytes);
    if (e == cudaSuccess) {
        // epoch starts at 1 so zeroed tile states never read as published
        const unsigned int one = 1u;
        e = cudaMemcpy(static_cast<char*>(c->scratchMem) + 4, &one, sizeof one, cudaMemcpyHostToDevice);
    }
    // word 0: the batch decide kernel's work counter; word 1: where blz_ctx_check takes the status
    if (e == cudaSuccess) e = cudaMalloc(&c->workCounter, 2 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMemset(c->workCounter, 0, 2 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMallocHost(&c->pinned, kPinnedBytes);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->pinnedDone, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        int rc = cuda_fail(e, "context setup");
        blz_ctx_destroy(c);
        return rc;
    }
    c->scratch = static_cast<Scratch*>(c->scratchMem);
    *out = c;
    return BLZ_OK;
}

int blz_ctx_destroy(blz_ctx* c) {
    if (!c) return BLZ_OK;
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    release_scene(c);
    if (c->scratchMem) cudaFree(c->scratchMem);
    if (c->workCounter) cudaFree(c->workCounter);
    if (c->pinned) cudaFreeHost(c->pinned);
    if (c->pinnedDone) cudaEventDestroy(c->pinnedDone);
    if (c->batchDev) cudaFree(c->batchDev);
    if (c->chunkMem) cudaFree(c->chunkMem);
    if (c->instScratch) cudaFree(c->instScratch);
    if (c->clusterMem) cudaFree(c->clusterMem);
    if (c->frameMem) cudaFree(c->frameMem);
    delete c;
    return BLZ_OK;
}

uint64_t blz_ctx_launch_count(const blz_ctx* c) { return c ? c->launches.load() : 0; }

int blz_ctx_set_wait_limit(blz_ctx* c, uint32_t polls) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    c->waitLimit = polls ? polls : static_cast<uint32_t>(kSpinLimitDefault);
    return BLZ_OK;
}

int blz_ctx_debug_advance_ticket(blz_ctx* c, uint32_t n, blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (n == 0 || n > 1024) return fail(BLZ_ERR_INVALID_ARGUMENT, "ticket advance %u outside [1, 1024]", n);
    cudaError_t e = launch_add_word(&c->scratch->ticket, n, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "ticket advance");
    return BLZ_OK;
}

int blz_ctx_debug_skip_frame_tiles(blz_ctx* c, uint32_t n, blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (n == 0 || n > 1024) return fail(BLZ_ERR_INVALID_ARGUMENT, "tile skip %u outside [1, 1024]", n);
    cudaError_t e = launch_add_word(&c->scratch->frameTicket, n, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "frame ticket advance");
    return BLZ_OK;
}

int blz_ctx_check(blz_ctx* c, blz_stream_t stream, uint32_t* flagsOut) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaError_t e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamSynchronize");
    // the status word is taken and cleared in one atomic exchange on the device, so a flag that
    // work on another stream of this context raises meanwhile is kept for the next check
    e = launch_take_status(&c->scratch->status, c->workCounter + 1, st);
    unsigned int hdr[2];
    uint32_t flags = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flags, c->workCounter + 1, sizeof flags, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hdr, c->scratchMem, sizeof hdr, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_fail(e, "status read");
    if (flags & BLZ_FLAG_TIMEOUT) {
        // a timed-out launch may have left the ticket mid-way: restart the protocol on a new epoch
        unsigned int fresh[3] = {0u, hdr[1] + 2u, 0u};
        cudaMemcpy(c->scratchMem, fresh, sizeof fresh, cudaMemcpyHostToDevice);
        cudaMemset(c->workCounter, 0, sizeof(unsigned int));
    }
    if (flagsOut) *flagsOut = flags;
    if (flags & BLZ_FLAG_TIMEOUT) return fail(BLZ_ERR_TIMEOUT, "a device-side wait timed out (flags 0x%x)", flags);
    if (flags & BLZ_FLAG_BAD_INDEX) return fail(BLZ_ERR_BAD_INDEX, "a scene id was out of range (flags 0x%x)", flags);
    if (flags & (BLZ_FLAG_COMMAND_OVERFLOW | BLZ_FLAG_INSTANCE_OVERFLOW))
        return fail(BLZ_ERR_CAPACITY, "an output buffer overflowed (flags 0x%x)", flags);
    return BLZ_OK;
}

// ------------------------------------------------------------------ scene

int blz_scene_upload(blz_ctx* c, const BlzSceneDesc* s, uint32_t flags, blz_stream_t stream) {
    if (!c || !s) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or scene is NULL");
    if (flags > BLZ_SCENE_BORROW_DEVICE) return fail(BLZ_ERR_INVALID_ARGUMENT, "unknown scene flags 0x%x", flags);
    if ((s->transformCount && !s->transforms) || (s->surfaceCount && !s->surfaces) || (s->lodCount && !s->lods) ||
        (s->clusterCount && !s->clusters) || (s->renderObjectCount && !s->renderObjects))
        return fail(BLZ_ERR_INVALID_ARGUMENT, "a scene table has a count but no pointer");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    cudaSetDevice(c->device);
    release_scene(c);
    SceneT t{};
    t.transformCount = s->transformCount;
    t.surfaceCount = s->surfaceCount;
    t.lodCount = s->lodCount;
    t.clusterCount = s->clusterCount;
    if (flags == BLZ_SCENE_BORROW_DEVICE) {
        t.objects = s->renderObjects;
        t.transforms = s->transforms;
        t.surfaces = s->surfaces;
        t.lods = s->lods;
        t.clusters = s->clusters;
    } else {
        auto up = [&](const void* src, size_t bytes, const void** dst) -> cudaError_t {
            *dst = nullptr;
            if (!bytes) return cudaSuccess;
            void* d = nullptr;
            cudaError_t e = cudaMalloc(&d, bytes);
            if (e != cudaSuccess) return e;
            c->ownedScene.push_back(d);
            *dst = d;
            return cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, st);
        };
        cudaError_t e = up(s->renderObjects, sizeof(BlzRenderObject) * (size_t)s->renderObjectCount, reinterpret_cast<const void**>(&t.objects));
        if (e == cudaSuccess) e = up(s->transforms, sizeof(BlzMeshTransform) * (size_t)s->transformCount, reinterpret_cast<const void**>(&t.transforms));
        if (e == cudaSuccess) e = up(s->surfaces, sizeof(BlzPrimitiveSurface) * (size_t)s->surfaceCount, reinterpret_cast<const void**>(&t.surfaces));
        if (e == cudaSuccess) e = up(s->lods, sizeof(BlzLodData) * (size_t)s->lodCount, reinterpret_cast<const void**>(&t.lods));
        if (e == cudaSuccess) e = up(s->clusters, sizeof(BlzCluster) * (size_t)s->clusterCount, reinterpret_cast<const void**>(&t.clusters));
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            release_scene(c);
            return e == cudaErrorMemoryAllocation ? fail(BLZ_ERR_OUT_OF_MEMORY, "scene allocation failed") : cuda_fail(e, "scene upload");
        }
    }
    if (reinterpret_cast<uintptr_t>(t.transforms) % 32 || reinterpret_cast<uintptr_t>(t.surfaces) % 16 ||
        reinterpret_cast<uintptr_t>(t.lods) % 16 || reinterpret_cast<uintptr_t>(t.clusters) % 16 ||
        reinterpret_cast<uintptr_t>(t.objects) % 8) {
        release_scene(c);
        return fail(BLZ_ERR_INVALID_ARGUMENT,
                    "scene tables must be aligned: transforms 32 bytes, surfaces/LODs/clusters 16, render objects 8");
    }
    // the largest cluster range a LOD can select bounds the candidates of a tile of objects
    uint32_t lodClusterMax = 0;
    if (s->lodCount) {
        std::vector<BlzLodData> lods(s->lodCount);
        cudaError_t e = cudaMemcpy(lods.data(), s->lods, sizeof(BlzLodData) * lods.size(), cudaMemcpyDefault);
        if (e != cudaSuccess) {
            release_scene(c);
            return cuda_fail(e, "reading the LOD table");
        }
        for (const BlzLodData& l : lods) lodClusterMax = std::max(lodClusterMax, std::min(l.clusterCount, s->clusterCount));
    }
    c->lodClusterMax = lodClusterMax;
    c->scene = t;
    c->defaultObjects = t.objects;
    c->defaultCount = s->renderObjectCount;
    c->hasScene = true;
    return BLZ_OK;
}

int blz_scene_bind_dynamic(blz_ctx* c, const BlzMeshTransform* rows, uint32_t count) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!c->hasScene) return fail(BLZ_ERR_NO_SCENE, "no scene uploaded");
    if (count > c->scene.transformCount)
        return fail(BLZ_ERR_INVALID_ARGUMENT, "%u dynamic rows but the scene has %u transforms", count, c->scene.transformCount);
    if (count > 0 && !rows) return fail(BLZ_ERR_INVALID_ARGUMENT, "rows is NULL");
    if (reinterpret_cast<uintptr_t>(rows) % 32 != 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "rows must be 32-byte aligned");
    c->scene.dynRows = count > 0 ? rows : nullptr;
    c->scene.dynCount = count;
    return BLZ_OK;
}

int blz_scene_device_tables(const blz_ctx* c, BlzSceneDesc* out) {
    if (!c || !out) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or out is NULL");
    if (!c->hasScene) return fail(BLZ_ERR_NO_SCENE, "no scene uploaded");
    out->renderObjects = c->defaultObjects;
    out->renderObjectCount = c->defaultCount;
    out->transforms = c->scene.transforms;
    out->transformCount = c->scene.transformCount;
    out->surfaces = c->scene.surfaces;
    out->surfaceCount = c->scene.surfaceCount;
    out->lods = c->scene.lods;
    out->lodCount = c->scene.lodCount;
    out->clusters = c->scene.clusters;
    out->clusterCount = c->scene.clusterCount;
    return BLZ_OK;
}

int blz_transforms_update_device(blz_ctx* c, const uint32_t* ids, const BlzMeshTransform* in, uint32_t n, blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!c->hasScene) return fail(BLZ_ERR_NO_SCENE, "no scene uploaded");
    if (n && (!ids || !in)) return fail(BLZ_ERR_INVALID_ARGUMENT, "ids or transforms is NULL");
    cudaError_t e = launch_transforms_scatter(const_cast<BlzMeshTransform*>(c->scene.transforms), c->scene.transformCount, ids, in, n,
                                              &c->scratch->status, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "transforms scatter launch");
    if (n) c->launches++;
    return BLZ_OK;
}

int blz_transforms_update(blz_ctx* c, const uint32_t* ids, const BlzMeshTransform* in, uint32_t n, blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!c->hasScene) return fail(BLZ_ERR_NO_SCENE, "no scene uploaded");
    if (n == 0) return BLZ_OK;
    if (!ids || !in) return fail(BLZ_ERR_INVALID_ARGUMENT, "ids or transforms is NULL");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    const size_t need = (size_t)n * (sizeof(uint32_t) + sizeof(BlzMeshTransform)) + 64;
    if (need > kPinnedBytes) return fail(BLZ_ERR_CAPACITY, "%u transforms exceed the staging buffer", n);
    cudaEventSynchronize(c->pinnedDone);  // the previous update's kernel has read the pinned buffer
    char* h = static_cast<char*>(c->pinned);
    const size_t tOff = 0, iOff = ((size_t)n * sizeof(BlzMeshTransform) + 63) & ~size_t(63);
    memcpy(h + tOff, in, (size_t)n * sizeof(BlzMeshTransform));
    memcpy(h + iOff, ids, (size_t)n * sizeof(uint32_t));
    // the scatter kernel reads the rows straight from pinned host memory (no staging copy): over
    // the coherent CPU-GPU link of a Grace-Blackwell node that is one transfer instead of two
    int rc = blz_transforms_update_device(c, reinterpret_cast<const uint32_t*>(h + iOff),
                                          reinterpret_cast<const BlzMeshTransform*>(h + tOff), n, stream);
    if (rc != BLZ_OK) return rc;
    cudaError_t e = cudaEventRecord(c->pinnedDone, st);
    if (e != cudaSuccess) return cuda_fail(e, "transform update event");
    return BLZ_OK;
}

int blz_transforms_rotate(blz_ctx* c, const uint32_t* ids, const float* axes, float angle, uint32_t n, BlzMeshTransform* dst,
                          blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!c->hasScene) return fail(BLZ_ERR_NO_SCENE, "no scene uploaded");
    if (n && (!ids || !axes)) return fail(BLZ_ERR_INVALID_ARGUMENT, "ids or axes is NULL");
    BlzMeshTransform* out = dst;
    if (!out) {
        // in place: rotate into staging, then scatter back (a kernel may not read and write the same rows)
        return fail(BLZ_ERR_INVALID_ARGUMENT, "in-place rotation needs a destination buffer; pass dDst and scatter it");
    }
    cudaError_t e = launch_transforms_rotate(c->scene.transforms, c->scene.transformCount, c->scene.dynRows, c->scene.dynCount, ids, axes, angle, n, out, &c->scratch->status,
                                             reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "transforms rotate launch");
    if (n) c->launches++;
    return BLZ_OK;
}

// ------------------------------------------------------------------ pyramid

static uint32_t mip_levels(uint32_t w, uint32_t h) {  // blitML.h:95-107
    uint32_t n = 0;
    while (w > 1 || h > 1) {
        ++n;
        w /= 2;
        h /= 2;
    }
    return n;
}

static uint32_t previous_pow2(uint32_t v) {  // blitML.h:54-62
    uint32_t r = 1;
    while (r * 2 < v) r *= 2;
    return r;
}

uint64_t blz_pyramid_layout(uint32_t dw, uint32_t dh, uint32_t mode, BlzPyramid* out) {
    if (!out || dw == 0 || dh == 0 || mode > BLZ_HIZ_VULKAN) return 0;
    memset(out, 0, sizeof *out);
    out->mode = mode;
    out->depthWidth = dw;
    out->depthHeight = dh;
    if (mode == BLZ_HIZ_D3D12) {
        out->width = (dw >> 1) ? (dw >> 1) : 1u;
        out->height = (dh >> 1) ? (dh >> 1) : 1u;
    } else {
        out->width = previous_pow2(dw);
        out->height = previous_pow2(dh);
    }
    uint32_t n = mip_levels(out->width, out->height);
    if (n == 0) n = 1;
    if (n > BLZ_PYRAMID_MAX_MIPS) return 0;
    out->mipCount = n;
    uint64_t at = 0;
    for (uint32_t i = 0; i < n; ++i) {
        uint32_t w = out->width >> i, h = out->height >> i;
        w = w ? w : 1u;
        h = h ? h : 1u;
        out->mipOffset[i] = static_cast<uint32_t>(at);
        at += (uint64_t)w * h;
    }
    return at * sizeof(float);
}

namespace blz {

// The parameters of one pyramid build from `depth` (checked), for the pyramid kernel or the
// one-call frame kernel.
static int pyramid_build_params(blz_ctx* c, const BlzPyramid* p, const float* depth, PyramidBuildParams& bp) {
    int rc = check_pyramid(p, true);
    if (rc != BLZ_OK) return rc;
    if (!depth) return fail(BLZ_ERR_INVALID_ARGUMENT, "depth is NULL");
    if (p->depthWidth == 0 || p->depthHeight == 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "pyramid has no depth extent");
    bp = PyramidBuildParams{};
    bp.depth = depth;
    bp.depthWidth = p->depthWidth;
    bp.depthHeight = p->depthHeight;
    bp.data = p->data;
    bp.width = p->width;
    bp.height = p->height;
    bp.mipCount = p->mipCount;
    bp.mode = p->mode;
    for (uint32_t i = 0; i < BLZ_PYRAMID_MAX_MIPS; ++i) bp.mipOffset[i] = p->mipOffset[i];
    bp.done = &c->scratch->pyrDone;
    bp.vec4 = (p->mode == BLZ_HIZ_D3D12 && p->depthWidth % 4 == 0 && p->depthHeight >= 2 &&
               p->width == p->depthWidth / 2 && p->height <= p->depthHeight / 2 && p->mipOffset[0] == 0 &&
               reinterpret_cast<uintptr_t>(depth) % 16 == 0 && reinterpret_cast<uintptr_t>(p->data) % 8 == 0) ? 1u : 0u;
    bp.spinLimit = c->waitLimit ? c->waitLimit : kSpinLimitDefault;
    return BLZ_OK;
}

}  // namespace blz

int blz_pyramid_build(blz_ctx* c, const BlzPyramid* p, const float* depth, blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    PyramidBuildParams bp;
    int rc = pyramid_build_params(c, p, depth, bp);
    if (rc != BLZ_OK) return rc;
    uint32_t launches = 0;
    cudaError_t e = launch_pyramid_build(bp, reinterpret_cast<cudaStream_t>(stream), &launches);
    if (e != cudaSuccess) return cuda_fail(e, "pyramid launch");
    c->launches += launches;
    return BLZ_OK;
}

int blz_depth_raster_boxes(blz_ctx* c, const BlzCameraViewData* view, const float* boxes, uint32_t boxCount, float* depth,
                           uint32_t width, uint32_t height, blz_stream_t stream) {
    if (!c || !view || !depth) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx, view or depth is NULL");
    if (boxCount && !boxes) return fail(BLZ_ERR_INVALID_ARGUMENT, "boxes is NULL");
    if (width == 0 || height == 0 || (uint64_t)width * height >= (1ull << 31)) return fail(BLZ_ERR_INVALID_ARGUMENT, "bad depth extent");
    uint32_t launches = 0;
    cudaError_t e = launch_depth_raster(*view, boxes, boxCount, depth, width, height, reinterpret_cast<cudaStream_t>(stream), &launches);
    if (e != cudaSuccess) return cuda_fail(e, "depth raster launch");
    c->launches += launches;
    return BLZ_OK;
}

// ------------------------------------------------------------------ single-view culls

static int object_cull(blz_ctx* c, uint32_t mode, const BlzCameraViewData* view, BlzRenderList list, uint32_t* vis,
                       const BlzPyramid* pyr, const BlzCullTarget* target, blz_stream_t stream) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    int rc = check_target(target);
    if (rc != BLZ_OK) return rc;
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    if ((mode == BLZ_MODE_FIRST || mode == BLZ_MODE_LATE) && count && !vis) return fail(BLZ_ERR_INVALID_ARGUMENT, "visibility buffer is NULL");
    if (mode == BLZ_MODE_LATE || mode == BLZ_MODE_TEMPORAL) {
        rc = check_pyramid(pyr, true);
        if (rc != BLZ_OK) return rc;
    }
    // the single-view autotuner's choice for this size and pass, else the context's shape
    uint32_t threads = c->singleThreads, opt = c->singleOpt;
    if (const TunedShape* t = find_tuned(c, count, 1u, mode)) {
        threads = t->shape.threadsPerBlock;
        opt = t->shape.objectsPerThread;
    }
    const uint32_t tile = single_chunk_size(mode, threads, opt, count, c->smCount);
    uint32_t tiles = (count + tile - 1) / tile;
    if (tiles == 0) tiles = 1;  // an empty list still gets one chunk, and its draw count is written
    rc = ensure_chunk_scratch(c, tiles, tile);
    if (rc != BLZ_OK) return rc;
    PipeParams p{};
    p.sc = c->scene;
    p.single.view = *view;
    p.single.objects = objs;
    p.single.count = count;
    p.single.mode = mode;
    p.single.vis = vis;
    p.single.pyr = pyramid_view(pyr);
    p.single.cmds = static_cast<uint8_t*>(target->commands);
    p.single.stride = target->stride;
    p.single.capacity = target->capacity;
    p.single.drawCount = target->drawCount;
    p.single.dynT = nullptr;
    p.single.dynCount = 0;
    p.views = nullptr;
    p.tileStart = nullptr;
    p.viewCount = 1;
    p.totalTiles = tiles;
    p.chunkSize = tile;
    bind_chunk_scratch(c, p);
    p.workCounter = nullptr;  // one chunk per resident warp, assigned by warp index
    cudaError_t e = launch_object_cull(mode, p, threads, opt, c->smCount, reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "cull launch");
    c->launches += 2;  // decide + scatter
    return BLZ_OK;
}

// The single-view autotuner: every single-view shape timed on the caller's pass, each run on a copy
// of the visibility buffer (restored before every run, outside the timed events).
static int autotune_single(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, uint32_t mode, const uint32_t* vis,
                           const BlzPyramid* pyr, const BlzCullTarget* target, uint32_t repeats, blz_stream_t stream,
                           BlzLaunchShape* best, float* bestUs) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    if (mode > BLZ_MODE_TEMPORAL) return fail(BLZ_ERR_INVALID_ARGUMENT, "unknown mode %u", mode);
    if (c->capturing) return fail(BLZ_ERR_INVALID_ARGUMENT, "the autotuner cannot run inside a capture");
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    int rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    if (count == 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "nothing to tune on: the list is empty");
    if ((mode == BLZ_MODE_FIRST || mode == BLZ_MODE_LATE) && !vis) return fail(BLZ_ERR_INVALID_ARGUMENT, "visibility buffer is NULL");
    auto report = [&](const TunedShape& t) {
        if (best) {
            *best = t.shape;
            best->chunkObjects = single_chunk_size(mode, t.shape.threadsPerBlock, t.shape.objectsPerThread, count, c->smCount);
        }
        if (bestUs) *bestUs = t.us;
        return BLZ_OK;
    };
    if (const TunedShape* t = find_tuned(c, count, 1u, mode)) return report(*t);
    if (repeats == 0) repeats = 5;
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    uint32_t* work = nullptr;  // the pass's visibility buffer: a copy of the caller's
    if (vis && cudaMalloc(&work, sizeof(uint32_t) * count) != cudaSuccess) return fail(BLZ_ERR_OUT_OF_MEMORY, "autotune visibility copy");
    BlzRenderList own{objs, count};
    const uint32_t shapes[][2] = {{256, 1}, {256, 2}, {256, 4}, {128, 2}, {128, 4}, {512, 1}};
    const uint32_t savedT = c->singleThreads, savedO = c->singleOpt;
    cudaEvent_t a, b;
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    TunedShape top{count, 1u, mode, BlzLaunchShape{savedT, savedO, 0, 0}, 1e30f};
    for (const auto& sh : shapes) {
        c->singleThreads = sh[0];
        c->singleOpt = sh[1];
        float total = 0.f;
        rc = BLZ_OK;
        for (uint32_t r = 0; r <= repeats && rc == BLZ_OK; ++r) {  // run 0 is untimed
            if (work && cudaMemcpyAsync(work, vis, sizeof(uint32_t) * count, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
                rc = fail(BLZ_ERR_CUDA, "autotune visibility copy");
                break;
            }
            cudaEventRecord(a, st);
            rc = object_cull(c, mode, view, own, work, pyr, target, stream);
            cudaEventRecord(b, st);
            cudaEventSynchronize(b);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, a, b);
            if (r > 0) total += ms;
        }
        if (rc != BLZ_OK) break;
        const float us = total * 1000.f / static_cast<float>(repeats);
        if (us < top.us) {
            top.us = us;
            top.shape = BlzLaunchShape{sh[0], sh[1], 0, 0};
        }
    }
    c->singleThreads = savedT;
    c->singleOpt = savedO;
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (work) {
        cudaStreamSynchronize(st);
        cudaFree(work);
    }
    if (rc != BLZ_OK) return rc;
    remember_tuned(c, top);
    return report(top);
}

int blz_cull_frustum(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, const BlzCullTarget* target, blz_stream_t s) {
    return object_cull(c, BLZ_MODE_FRUSTUM, view, list, nullptr, nullptr, target, s);
}

int blz_cull_first(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, const uint32_t* vis, const BlzCullTarget* target,
                   blz_stream_t s) {
    return object_cull(c, BLZ_MODE_FIRST, view, list, const_cast<uint32_t*>(vis), nullptr, target, s);
}

int blz_cull_late(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, uint32_t* vis, const BlzPyramid* pyr,
                  const BlzCullTarget* target, blz_stream_t s) {
    return object_cull(c, BLZ_MODE_LATE, view, list, vis, pyr, target, s);
}

int blz_cull_temporal(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, const BlzPyramid* pyr,
                      const BlzCullTarget* target, blz_stream_t s) {
    return object_cull(c, BLZ_MODE_TEMPORAL, view, list, nullptr, pyr, target, s);
}

int blz_autotune_single(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, uint32_t mode, const uint32_t* vis,
                        const BlzPyramid* pyr, const BlzCullTarget* target, uint32_t repeats, blz_stream_t stream,
                        BlzLaunchShape* best, float* bestUs) {
    return autotune_single(c, view, list, mode, vis, pyr, target, repeats, stream, best, bestUs);
}

// ------------------------------------------------------------------ kept frames

}  // extern "C"

namespace blz {

// Kept-frame memory for `chunks` chunks of `chunkSize` objects: staged records of pass 1 and of
// pass 2 (8 bytes per object each), the chunk counts of both passes and of the kept survivors, and
// the survivors themselves (32 bytes per object). Grown on demand; never inside a capture.
struct FrameBuffers {
    uint2 *staged1, *staged2;
    uint32_t *count1, *count2, *keepCount;
    void* keep;
};

static int ensure_frame_scratch(blz_ctx* c, size_t chunks, size_t chunkSize, FrameBuffers& fb) {
    const size_t objects = chunks * chunkSize;
    if (objects > c->frameObjects || chunks > c->frameChunks) {
        if (c->capturing) return fail(BLZ_ERR_CAPACITY, "scratch must grow, which a capture cannot record: run the call once before capturing");
        if (c->frameMem) {
            cudaDeviceSynchronize();
            cudaFree(c->frameMem);
            c->frameMem = nullptr;
            c->frameObjects = c->frameChunks = 0;
        }
        const size_t wantObj = objects + objects / 8 + 1024, wantChunks = chunks + chunks / 8 + 64;
        const size_t bytes = wantObj * (2 * sizeof(uint2) + 32) + wantChunks * 3 * sizeof(uint32_t) + 1024;
        if (cudaMalloc(&c->frameMem, bytes) != cudaSuccess) return fail(BLZ_ERR_OUT_OF_MEMORY, "kept-frame scratch of %zu bytes", bytes);
        c->frameObjects = wantObj;
        c->frameChunks = wantChunks;
        c->frameOpen = false;
    }
    char* m = static_cast<char*>(c->frameMem);
    fb.keep = m;  // 32-byte survivors first: 256-byte aligned
    m += c->frameObjects * 32;
    fb.staged1 = reinterpret_cast<uint2*>(m);
    m += c->frameObjects * sizeof(uint2);
    fb.staged2 = reinterpret_cast<uint2*>(m);
    m += c->frameObjects * sizeof(uint2);
    fb.count1 = reinterpret_cast<uint32_t*>(m);
    fb.count2 = fb.count1 + c->frameChunks;
    fb.keepCount = fb.count2 + c->frameChunks;
    return BLZ_OK;
}

static PipeParams frame_params(blz_ctx* c, const FrameBuffers& fb, const BlzCameraViewData& view, const BlzRenderObject* objs,
                               uint32_t count, uint32_t* vis, uint32_t chunkSize, uint32_t tiles) {
    PipeParams p{};
    p.sc = c->scene;
    p.single.view = view;
    p.single.objects = objs;
    p.single.count = count;
    p.single.vis = vis;
    p.viewCount = 1;
    p.totalTiles = tiles;
    p.chunkSize = chunkSize;
    p.scratch = c->scratch;
    p.workCounter = nullptr;
    p.keep = fb.keep;
    p.keepCount = fb.keepCount;
    return p;
}

static void set_target(PipeParams& p, const BlzCullTarget* t) {
    p.single.cmds = static_cast<uint8_t*>(t->commands);
    p.single.stride = t->stride;
    p.single.capacity = t->capacity;
    p.single.drawCount = t->drawCount;
}

// Validates a frame's pass-1 arguments and binds its memory; nothing is launched.
static int frame_begin(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, uint32_t* vis,
                       const BlzCullTarget* target, FrameBuffers& fb, PipeParams& p1, int mode = kModeFrame1) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    int rc = check_target(target);
    if (rc != BLZ_OK) return rc;
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    if (count && !vis) return fail(BLZ_ERR_INVALID_ARGUMENT, "visibility buffer is NULL");
    const uint32_t tile = single_chunk_size(static_cast<uint32_t>(mode), c->singleThreads, c->singleOpt, count, c->smCount);
    uint32_t tiles = (count + tile - 1) / tile;
    if (tiles == 0) tiles = 1;  // an empty list still gets one chunk, and its draw counts are written
    rc = ensure_frame_scratch(c, tiles, tile, fb);
    if (rc != BLZ_OK) return rc;
    p1 = frame_params(c, fb, *view, objs, count, vis, tile, tiles);
    p1.single.mode = BLZ_MODE_FIRST;
    p1.staged = fb.staged1;
    p1.chunkCount = fb.count1;
    set_target(p1, target);
    return BLZ_OK;
}

static void frame_keep(blz_ctx* c, const PipeParams& p1) {
    c->frameOpen = true;
    c->frameView = p1.single.view;
    c->frameObjs = p1.single.objects;
    c->frameCount = p1.single.count;
    c->frameVis = p1.single.vis;
    c->frameChunkSize = p1.chunkSize;
    c->frameTiles = p1.totalTiles;
}

// Pass-2 parameters of the context's open frame.
static int frame_late_params(blz_ctx* c, const BlzPyramid* pyr, const BlzCullTarget* target, PipeParams& p2) {
    int rc = check_target(target);
    if (rc != BLZ_OK) return rc;
    rc = check_pyramid(pyr, true);
    if (rc != BLZ_OK) return rc;
    FrameBuffers fb{};
    rc = ensure_frame_scratch(c, c->frameTiles, c->frameChunkSize, fb);  // binds only: the frame's chunks fit
    if (rc != BLZ_OK) return rc;
    p2 = frame_params(c, fb, c->frameView, c->frameObjs, c->frameCount, c->frameVis, c->frameChunkSize, c->frameTiles);
    p2.single.mode = BLZ_MODE_LATE;
    p2.single.pyr = pyramid_view(pyr);
    p2.staged = fb.staged2;
    p2.chunkCount = fb.count2;
    set_target(p2, target);
    return BLZ_OK;
}

}  // namespace blz

extern "C" {

int blz_frame_first(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, uint32_t* vis,
                    const BlzCullTarget* target, blz_stream_t stream) {
    FrameBuffers fb{};
    PipeParams p1{};
    int rc = frame_begin(c, view, list, vis, target, fb, p1);
    if (rc != BLZ_OK) return rc;
    cudaError_t e = launch_frame_first(p1, c->singleThreads, c->singleOpt, c->smCount, reinterpret_cast<cudaStream_t>(stream), true);
    if (e != cudaSuccess) return cuda_fail(e, "frame pass-1 launch");
    c->launches += 2;  // decide + scatter
    frame_keep(c, p1);
    return BLZ_OK;
}

int blz_frame_late(blz_ctx* c, const BlzPyramid* pyr, const BlzCullTarget* target, blz_stream_t stream) {
    if (!c) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx is NULL");
    if (!c->frameOpen) return fail(BLZ_ERR_INVALID_ARGUMENT, "blz_frame_late needs a blz_frame_first on this context first");
    PipeParams p2{};
    int rc = frame_late_params(c, pyr, target, p2);
    if (rc != BLZ_OK) return rc;
    cudaError_t e = launch_frame_late(p2, c->smCount, reinterpret_cast<cudaStream_t>(stream), true);
    if (e != cudaSuccess) return cuda_fail(e, "frame pass-2 launch");
    c->launches += 2;  // survivors' pyramid test + scatter
    return BLZ_OK;
}

int blz_cull_frame(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, uint32_t* vis, const float* depth,
                   const BlzPyramid* pyr, const BlzCullTarget* target1, const BlzCullTarget* target2, blz_stream_t stream) {
    FrameBuffers fb{};
    PipeParams p1{};
    int rc = frame_begin(c, view, list, vis, target1, fb, p1, kModeFrameFused);
    if (rc != BLZ_OK) return rc;
    rc = check_target(target2);
    if (rc != BLZ_OK) return rc;
    rc = check_pyramid(pyr, true);
    if (rc != BLZ_OK) return rc;
    PyramidBuildParams bp;
    if (depth) {
        rc = pyramid_build_params(c, pyr, depth, bp);
        if (rc != BLZ_OK) return rc;
    }
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);
    PipeParams p2 = p1;  // pass 2's records: staged / chunkCount, target 2
    p2.single.mode = BLZ_MODE_LATE;
    p2.single.pyr = pyramid_view(pyr);
    p2.staged = fb.staged1;
    p2.chunkCount = fb.count1;
    set_target(p2, target2);
    p2.staged2 = fb.staged2;  // pass 1's records
    p2.chunkCount2 = fb.count2;
    // one launch building the pyramid's tiles and then deciding both passes in one sweep (or the
    // sweep alone over the pyramid the caller built), then both record lists in one launch
    cudaError_t e = depth ? launch_frame_pyr(p2, bp, c->singleThreads, c->singleOpt, c->smCount, st)
                          : launch_frame_fused(p2, c->singleThreads, c->singleOpt, c->smCount, st);
    PipeParams q1 = p1;  // pass 1's list for the scatter
    q1.staged = fb.staged2;
    q1.chunkCount = fb.count2;
    if (e == cudaSuccess) e = launch_frame_scatter2(q1, p2, st);
    if (e != cudaSuccess) return cuda_fail(e, "frame launch");
    c->launches += 2;  // the sweep (with the pyramid) + both scatters
    c->frameOpen = false;  // the fused sweep keeps no survivors for blz_frame_late
    return BLZ_OK;
}

int blz_cull_instanced(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, BlzLodInstanceCounter* counters,
                       uint32_t* instances, uint32_t instanceCapacity, uint32_t slotsPerLod, const BlzCullTarget* target,
                       blz_stream_t s) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    int rc = check_target(target);
    if (rc != BLZ_OK) return rc;
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    if (!counters) return fail(BLZ_ERR_INVALID_ARGUMENT, "counters is NULL");
    if (instanceCapacity && !instances) return fail(BLZ_ERR_INVALID_ARGUMENT, "instances is NULL");
    const uint32_t nL = c->scene.lodCount;
    if (nL == 0) return fail(BLZ_ERR_INVALID_ARGUMENT, "the scene has no LODs");
    if (nL > kMaxInstancedLods) return fail(BLZ_ERR_INVALID_ARGUMENT, "instanced cull supports up to %u LODs, scene has %u", kMaxInstancedLods, nL);
    if (nL <= kInstStagedMaxLods) {
        // the FRUSTUM decide kernel stages (object, LOD) pairs; a counting sort turns them into lists
        const uint32_t tile = single_chunk_size(kModeInstanced, c->singleThreads, c->singleOpt, count, c->smCount);
        uint32_t chunks = (count + tile - 1) / tile;
        if (chunks == 0) chunks = 1;
        rc = ensure_chunk_scratch(c, chunks, tile);
        if (rc != BLZ_OK) return rc;
        const uint32_t groups = instanced_group_count(chunks);
        const size_t words = static_cast<size_t>(groups) * nL;  // the groups' LOD histograms
        if (words > c->instWords) {
            if (c->capturing) return fail(BLZ_ERR_CAPACITY, "scratch must grow, which a capture cannot record: run the call once before capturing");
            if (c->instScratch) {
                cudaDeviceSynchronize();
                cudaFree(c->instScratch);
                c->instScratch = nullptr;
                c->instWords = 0;
            }
            const size_t want = words + words / 4;
            if (cudaMalloc(&c->instScratch, want * sizeof(uint32_t)) != cudaSuccess)
                return fail(BLZ_ERR_OUT_OF_MEMORY, "instanced scratch of %zu bytes", want * sizeof(uint32_t));
            c->instWords = want;
        }
        PipeParams p{};
        p.sc = c->scene;
        p.single.view = *view;
        p.single.objects = objs;
        p.single.count = count;
        p.single.mode = BLZ_MODE_FRUSTUM;
        p.viewCount = 1;
        p.totalTiles = chunks;
        p.chunkSize = tile;
        bind_chunk_scratch(c, p);
        p.workCounter = nullptr;
        p.instHist = c->instScratch;
        p.instLods = nL;
        InstStagedParams q{};
        q.staged = p.staged;
        q.chunkCount = p.chunkCount;
        q.totalTiles = chunks;
        q.chunkSize = tile;
        q.groups = groups;
        q.nL = nL;
        q.hist = c->instScratch;
        q.lods = c->scene.lods;
        q.counters = counters;
        q.instances = instances;
        q.instanceCapacity = instanceCapacity;
        q.slotsPerLod = slotsPerLod;
        q.cmds = static_cast<uint8_t*>(target->commands);
        q.stride = target->stride;
        q.capacity = target->capacity;
        q.drawCount = target->drawCount;
        q.status = &c->scratch->status;
        cudaError_t e = launch_instanced_staged(p, q, c->singleThreads, c->singleOpt, c->smCount, reinterpret_cast<cudaStream_t>(s));
        if (e != cudaSuccess) return cuda_fail(e, "instanced cull launch");
        c->launches += 2;  // decide (with the group histograms), place
        return BLZ_OK;
    }
    const uint32_t tiles = (count + instanced_tile_size() - 1) / instanced_tile_size();
    rc = ensure_states(c, (size_t)(tiles ? tiles : 1) * nL);
    if (rc != BLZ_OK) return rc;
    InstancedParams p{};
    p.sc = c->scene;
    p.objects = objs;
    p.count = count;
    p.stride = target->stride;
    p.counters = counters;
    p.instances = instances;
    p.instanceCapacity = instanceCapacity;
    p.slotsPerLod = slotsPerLod;
    p.cmds = static_cast<uint8_t*>(target->commands);
    p.capacity = target->capacity;
    p.drawCount = target->drawCount;
    p.scratch = c->scratch;
    p.spinLimit = c->waitLimit;
    cudaError_t e = launch_instanced_cull(p, *view, reinterpret_cast<cudaStream_t>(s));
    if (e != cudaSuccess) return cuda_fail(e, "instanced cull launch");
    c->launches++;
    return BLZ_OK;
}

int blz_cull_clusters(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, const BlzPyramid* pyr,
                      const BlzCullTarget* target, uint32_t* clusterIds, blz_stream_t s) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    int rc = check_target(target);
    if (rc != BLZ_OK) return rc;
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    rc = check_pyramid(pyr, false);
    if (rc != BLZ_OK) return rc;
    if (!c->scene.clusters && c->scene.clusterCount) return fail(BLZ_ERR_INVALID_ARGUMENT, "scene has no cluster table");
    uint32_t tiles = (count + cluster_tile_objects() - 1) / cluster_tile_objects();
    if (tiles == 0) tiles = 1;
    ClusterParams p{};
    rc = bind_cluster_scratch(c, tiles, p);
    if (rc != BLZ_OK) return rc;
    rc = cluster_test_occupancy(c, false, p);
    if (rc != BLZ_OK) return rc;
    p.sc = c->scene;
    p.objects = objs;
    p.count = count;
    p.stride = target->stride;
    p.pyr = pyramid_view(pyr);
    p.hasPyramid = pyr ? 1u : 0u;
    p.capacity = target->capacity;
    p.cmds = static_cast<uint8_t*>(target->commands);
    p.clusterIds = clusterIds;
    p.drawCount = target->drawCount;
    p.scratch = c->scratch;
    cudaError_t e = launch_cluster_cull(p, *view, reinterpret_cast<cudaStream_t>(s));
    if (e != cudaSuccess) return cuda_fail(e, "cluster cull launch");
    c->launches += 3;  // objects, tests, emit
    return BLZ_OK;
}

int blz_cull_cluster_tasks(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list, const BlzPyramid* pyr,
                           const BlzTaskTarget* target, blz_stream_t s) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    if (!target) return fail(BLZ_ERR_INVALID_ARGUMENT, "target is NULL");
    if (!target->taskCount || !target->payloadCount)
        return fail(BLZ_ERR_INVALID_ARGUMENT, "target taskCount or payloadCount is NULL");
    if ((target->taskCapacity > 0 && !target->tasks) || (target->payloadCapacity > 0 && !target->payloads))
        return fail(BLZ_ERR_INVALID_ARGUMENT, "target tasks or payloads is NULL");
    if (reinterpret_cast<uintptr_t>(target->tasks) % 4 != 0 || reinterpret_cast<uintptr_t>(target->payloads) % 4 != 0)
        return fail(BLZ_ERR_INVALID_ARGUMENT, "target tasks and payloads must be 4-byte aligned");
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    int rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    rc = check_pyramid(pyr, false);
    if (rc != BLZ_OK) return rc;
    if (!c->scene.clusters && c->scene.clusterCount) return fail(BLZ_ERR_INVALID_ARGUMENT, "scene has no cluster table");
    uint32_t tiles = (count + cluster_tile_objects() - 1) / cluster_tile_objects();
    if (tiles == 0) tiles = 1;
    ClusterParams p{};
    rc = bind_cluster_scratch(c, tiles, p);
    if (rc != BLZ_OK) return rc;
    rc = cluster_test_occupancy(c, true, p);
    if (rc != BLZ_OK) return rc;
    p.sc = c->scene;
    p.objects = objs;
    p.count = count;
    p.pyr = pyramid_view(pyr);
    p.hasPyramid = pyr ? 1u : 0u;
    p.scratch = c->scratch;
    p.tasks = reinterpret_cast<uint32_t*>(target->tasks);
    p.payloads = reinterpret_cast<uint32_t*>(target->payloads);
    p.taskCapacity = target->taskCapacity;
    p.payloadCapacity = target->payloadCapacity;
    p.taskCount = target->taskCount;
    p.payloadCount = target->payloadCount;
    cudaError_t e = launch_cluster_tasks(p, *view, reinterpret_cast<cudaStream_t>(s));
    if (e != cudaSuccess) return cuda_fail(e, "cluster task cull launch");
    c->launches += 3;  // objects, tests, emit
    return BLZ_OK;
}

// ------------------------------------------------------------------ view constants

}  // extern "C"
