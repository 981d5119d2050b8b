// noalloc.cu — blz_cull_frustum_noalloc: the frustum + LOD cull with its per-call staging held in
// a fixed array of this library's own device memory, so the call allocates nothing.
//
// blz_cull_frustum stages each chunk's emitted (object, LOD) pairs and the chunk counts in context
// memory that grows on demand, and growing it means cudaFree + cudaMalloc. Some callers cannot take that: a frame loop that has reserved all of its
// device memory up front (another pool owns the rest, so a cudaMalloc would fail mid-frame), or
// one that must never stall, since cudaFree waits for the whole device. This entry point runs the
// same two kernels with that staging in `g_noallocScratch` below, a file-scope array sized for at
// most BLZ_NOALLOC_MAX_OBJECTS render objects, and rejects larger lists instead of growing.
//
// Set-up: the array's device address is fetched with cudaGetSymbolAddress by the first call made on
// each context (with the context's device current) and kept in the context. Make that first call
// before any stream capture: a first call inside a capture is refused with an error, since the
// address lookup can load this file's device code, which a capture cannot record. After set-up a
// call only validates its arguments and launches. Keeping the address per context, not per
// device for the process, means a context created after cudaDeviceReset fetches the address of
// the reloaded module instead of reusing a dead one.
//
// Nothing in the array has to start at zero: each call writes every word it later reads (each
// chunk's count and staged records are written by the decide kernel before the scatter kernel
// reads them).
//
// The array is one per device for the whole process, shared by every context on that device:
// two calls that overlap on the device (two streams, two threads, two contexts) race on it and
// both results are undefined. Order such calls on one stream, or with events.
#include <mutex>

#include "api_internal.h"

namespace {

using namespace blz;

constexpr uint32_t kNoAllocChunk = 512;  // objects per chunk (the kernels take any multiple of 32)
constexpr uint32_t kNoAllocChunks = BLZ_NOALLOC_MAX_OBJECTS / kNoAllocChunk;
static_assert(BLZ_NOALLOC_MAX_OBJECTS % kNoAllocChunk == 0, "the object bound must be whole chunks");

// layout: staged records | chunk counts
constexpr size_t kStagedBytes = size_t(BLZ_NOALLOC_MAX_OBJECTS) * sizeof(uint2);
constexpr size_t kCountsOffset = kStagedBytes;
constexpr size_t kNoAllocBytes = kCountsOffset + size_t(kNoAllocChunks) * sizeof(uint32_t);
static_assert(kCountsOffset % 256 == 0, "regions start on 256-byte lines");

static __device__ __align__(256) unsigned char g_noallocScratch[kNoAllocBytes];

std::mutex g_setupLock;

// The array's device address for context c (whose device is current), fetched on first use.
int scratch_base(blz_ctx* c, unsigned char** out) {
    std::lock_guard<std::mutex> guard(g_setupLock);
    if (!c->noallocBase) {
        if (c->capturing)
            return fail(BLZ_ERR_INVALID_ARGUMENT,
                        "blz_cull_frustum_noalloc's first call on a context must come before any capture: it looks up its staging array");
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noallocScratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress of the no-alloc scratch");
        if (reinterpret_cast<uintptr_t>(p) % 256 != 0) return fail(BLZ_ERR_CUDA, "no-alloc scratch is not 256-byte aligned");
        c->noallocBase = static_cast<unsigned char*>(p);
    }
    *out = c->noallocBase;
    return BLZ_OK;
}

}  // namespace

extern "C" int blz_cull_frustum_noalloc(blz_ctx* c, const BlzCameraViewData* view, BlzRenderList list,
                                        const BlzCullTarget* target, blz_stream_t stream) {
    if (!c || !view) return fail(BLZ_ERR_INVALID_ARGUMENT, "ctx or view is NULL");
    int rc = check_target(target);
    if (rc != BLZ_OK) return rc;
    const BlzRenderObject* objs = nullptr;
    uint32_t count = 0;
    rc = resolve_list(c, list, &objs, &count);
    if (rc != BLZ_OK) return rc;
    if (count > BLZ_NOALLOC_MAX_OBJECTS)
        return fail(BLZ_ERR_CAPACITY, "blz_cull_frustum_noalloc takes at most %u render objects, got %u",
                    BLZ_NOALLOC_MAX_OBJECTS, count);
    int device = -1;
    cudaError_t e = cudaGetDevice(&device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    if (device != c->device) return fail(BLZ_ERR_INVALID_ARGUMENT, "device %d is current, the context is on device %d", device, c->device);
    unsigned char* base = nullptr;
    rc = scratch_base(c, &base);
    if (rc != BLZ_OK) return rc;

    uint32_t chunks = (count + kNoAllocChunk - 1) / kNoAllocChunk;
    if (chunks == 0) chunks = 1;  // an empty list still gets one chunk, and its draw count is written
    PipeParams p{};
    p.sc = c->scene;
    p.single.view = *view;
    p.single.objects = objs;
    p.single.count = count;
    p.single.mode = BLZ_MODE_FRUSTUM;
    p.single.cmds = static_cast<uint8_t*>(target->commands);
    p.single.stride = target->stride;
    p.single.capacity = target->capacity;
    p.single.drawCount = target->drawCount;
    p.viewCount = 1;
    p.totalTiles = chunks;
    p.chunkSize = kNoAllocChunk;
    p.scratch = c->scratch;  // status flags stay in the context, read by blz_ctx_check
    p.staged = reinterpret_cast<uint2*>(base);
    p.chunkCount = reinterpret_cast<uint32_t*>(base + kCountsOffset);
    e = launch_object_cull(BLZ_MODE_FRUSTUM, p, c->singleThreads, c->singleOpt, c->smCount,
                           reinterpret_cast<cudaStream_t>(stream));
    if (e != cudaSuccess) return cuda_fail(e, "no-alloc cull launch");
    c->launches += 2;  // decide + scatter
    return BLZ_OK;
}
