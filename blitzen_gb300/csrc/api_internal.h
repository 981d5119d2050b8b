// api_internal.h — context layout and helpers shared by the C ABI translation units.
#pragma once

#include <atomic>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "kernels.h"

namespace blz {

constexpr size_t kDefaultStateCapacity = size_t(1) << 22;  // 4M tile states (32 MiB)
constexpr size_t kPinnedBytes = size_t(8) << 20;            // pinned host staging: transform rows, batch views
constexpr uint32_t kMaxInstancedLods = 4096;                // shared-memory bucket histograms

// An autotuner's choice for one workload size: batches keyed by (total objects, views), single-view
// passes by (objects, 1, pass).
constexpr uint32_t kTunedBatch = 0xFFFFFFFFu;
struct TunedShape {
    uint64_t objects;
    uint32_t views;
    uint32_t mode;  // the single-view pass, or kTunedBatch
    BlzLaunchShape shape;
    float us;
};

}  // namespace blz

struct blz_ctx {
    int device = 0;
    int smCount = 0;
    void* scratchMem = nullptr;        // Scratch header + tile states
    blz::Scratch* scratch = nullptr;
    size_t stateCapacity = 0;
    unsigned int* workCounter = nullptr;  // batch decide launches: next chunk (zero between launches)
    void* pinned = nullptr;            // pinned host staging
    cudaEvent_t pinnedDone = nullptr;  // last copy out of `pinned` has completed
    void* batchDev = nullptr;          // device BatchViewDev[] + tileStart[]
    size_t batchBytes = 0;
    void* chunkMem = nullptr;          // object-cull staging: records, chunk counts
    size_t chunkObjects = 0;           // staged-record capacity
    size_t chunkSlots = 0;             // chunk count capacity
    uint32_t* instScratch = nullptr;   // instanced cull: group x LOD counts, then LOD totals
    size_t instWords = 0;
    void* clusterMem = nullptr;        // cluster cull: tile counts, object ranges and survivors, visibility bits
    size_t clusterBytes = 0;
    int clusterTestBlocksPerSm[2] = {0, 0};  // records, task form: resident test blocks per SM (found on first use)
    uint32_t lodClusterMax = 0;        // largest clusterCount of the scene's LODs (clamped to the cluster table)
    bool hasScene = false;
    blz::SceneT scene{};
    const BlzRenderObject* defaultObjects = nullptr;
    uint32_t defaultCount = 0;
    std::vector<void*> ownedScene;
    std::atomic<uint64_t> launches{0};
    bool capturing = false;            // a blz_capture_begin is open
    uint64_t launchesAtCapture = 0;
    BlzLaunchShape shape{256, 2, 0, 0};   // batch launches
    std::vector<blz::TunedShape> tuned;  // the autotuners' cached choices (cleared by blz_set_launch_shape)
    uint32_t singleThreads = 256, singleOpt = 2;  // single-view launches
    uint32_t waitLimit = static_cast<uint32_t>(blz::kSpinLimitDefault);  // polls before a device-side wait gives up
    unsigned char* noallocBase = nullptr;  // device address of the no-alloc staging array, fetched by this context's first no-alloc call
    // kept frame (blz_frame_first / blz_frame_late): staged records of both passes, their chunk
    // counts, the survivors pass 1 keeps and their counts, and what pass 2 reuses of pass 1's call
    void* frameMem = nullptr;
    size_t frameObjects = 0, frameChunks = 0;
    bool frameOpen = false;
    BlzCameraViewData frameView{};
    const BlzRenderObject* frameObjs = nullptr;
    uint32_t frameCount = 0, frameChunkSize = 0, frameTiles = 0;
    uint32_t* frameVis = nullptr;
};

namespace blz {

int fail(int code, const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);
PyramidT pyramid_view(const BlzPyramid* p);
int check_pyramid(const BlzPyramid* p, bool required);
int check_target(const BlzCullTarget* t);
int resolve_list(const blz_ctx* c, BlzRenderList list, const BlzRenderObject** objs, uint32_t* count);
int ensure_states(blz_ctx* c, size_t states);

// Object-cull scratch for `chunks` chunks of `chunkSize` objects (grown on demand; a call that
// grows it synchronises the device first).
int ensure_chunk_scratch(blz_ctx* c, size_t chunks, size_t chunkSize);
void bind_chunk_scratch(blz_ctx* c, PipeParams& p);

// The cached autotuner choice for (objects, views, mode), or null.
const TunedShape* find_tuned(const blz_ctx* c, uint64_t objects, uint32_t views, uint32_t mode);
void remember_tuned(blz_ctx* c, const TunedShape& t);

}  // namespace blz
