// kernels.h — launch parameters and launchers shared by the kernel files and the C ABI layer.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/blz_cull.h"
#include "../../include/blz_types.h"

namespace blz {

struct Scratch;

#ifndef __CUDACC__
// Host-only translation units see the device structs as opaque layouts of the same size.
struct Vec3 { float x, y, z; };
#endif

struct SceneTablesHost {
    const BlzRenderObject* objects;
    const BlzMeshTransform* transforms;
    const BlzPrimitiveSurface* surfaces;
    const BlzLodData* lods;
    const BlzCluster* clusters;
    uint32_t transformCount, surfaceCount, lodCount, clusterCount;
    const BlzMeshTransform* dynRows;  // bound dynamic rows: transforms [0, dynCount) are read here
    uint32_t dynCount, pad0;
};

struct PyramidViewHost {
    const float* data;
    uint32_t width, height, mipCount, mode;
    uint32_t mipOffset[BLZ_PYRAMID_MAX_MIPS];
};

}  // namespace blz

#ifdef __CUDACC__
#include "blz_device.cuh"
#endif

namespace blz {

#ifdef __CUDACC__
using SceneT = SceneTables;
using PyramidT = PyramidView;
static_assert(sizeof(SceneTables) == sizeof(SceneTablesHost), "scene table layout");
static_assert(sizeof(PyramidView) == sizeof(PyramidViewHost), "pyramid layout");
#else
using SceneT = SceneTablesHost;
using PyramidT = PyramidViewHost;
#endif

// Pass 1 of a kept frame (blz_frame_first): every object of the list is frustum-tested once; the
// objects visible last frame that pass are emitted (pass 1's records), and every object that passes
// is kept, with its view-space sphere, for the frame's pass 2, which then tests only those against
// the pyramid (frame_late_kernel). An object outside the frustum gets its final visibility (0) here.
constexpr int kModeFrame1 = 4;
// Both passes of a frame in one sweep (blz_cull_frame, the pyramid built first): every object is
// frustum-tested once, the survivors are tested against the pyramid at once, and each object lands
// in pass 1's records (visible last frame and inside the frustum), in pass 2's (not visible last
// frame, inside the frustum and not occluded) or in neither; its visibility is rewritten as pass 2
// rewrites it. Pass 1's records are staged in staged2 / chunkCount2.
constexpr int kModeFrameFused = 5;
// kModeFrameFused with the pyramid built inside the same launch (blz_cull_frame given a depth
// buffer): the kernel's blocks first build the pyramid's tiles, taken by ticket, and a warp waits
// for the finished pyramid (a flag in the context's scratch) before its first Hi-Z test.
constexpr int kModeFramePyr = 6;
// The frustum + LOD pass of the instanced cull: BLZ_MODE_FRUSTUM, and every emitted record also
// counts towards its group's LOD histogram (PipeParams.instHist: [group][LOD], 32 chunks a group),
// which the place kernel turns into list offsets.
constexpr int kModeInstanced = 7;

constexpr int kObjThreads = 256;
constexpr int kObjOpt = 2;
constexpr uint32_t kMaxTiles = 1u << 20;             // tile states held by one scratch
constexpr unsigned long long kSpinLimitDefault = 1ull << 20;  // polls of one state before a device-side wait gives up
constexpr size_t kScratchHeaderBytes = 128;          // Scratch fields before the state array

// Device copy of one view of a cull launch (its uniform, render list, mode, buffers).
struct BatchViewDev {
    BlzCameraViewData view;
    const BlzRenderObject* objects;
    uint32_t count;
    uint32_t mode;
    uint32_t* vis;
    PyramidT pyr;
    uint8_t* cmds;
    uint32_t stride;
    uint32_t capacity;
    uint32_t* drawCount;
    const BlzMeshTransform* dynT;
    uint32_t dynCount;
    uint32_t pad;
};

// Parameters of the object-cull kernels: one view inline (single-view launches) or an array of
// views in device memory with the first chunk of each (viewCount + 1 entries), plus the scratch
// the decide kernel stages compacted records in (chunk c owns staged[c * chunkSize ...]) and the
// per-chunk record counts the scatter kernel turns into output offsets.
struct PipeParams {
    SceneT sc;
    BatchViewDev single;
    const BatchViewDev* views;
    const uint32_t* tileStart;
    uint32_t viewCount;
    uint32_t totalTiles;   // chunks over all views
    uint32_t chunkSize;    // objects per chunk, a multiple of 32
    uint32_t descending;   // single-view pass 2: chunks were walked and staged last object first
    Scratch* scratch;      // status word
    uint2* staged;         // [totalTiles * chunkSize] (objectId, lodId)
    uint32_t* chunkCount;  // [totalTiles]
    unsigned int* workCounter;  // next chunk to decide (zero between launches), or NULL: static chunks
    void* keep;            // kept frame: [totalTiles * chunkSize] survivors (32 bytes each) pass 1 keeps for pass 2
    uint32_t* keepCount;   // kept frame: [totalTiles] survivors per chunk
    uint2* staged2;        // fused frame: pass 1's staged records, [totalTiles * chunkSize]
    uint32_t* chunkCount2; // fused frame: [totalTiles]
    uint32_t* instHist;    // instanced pass: [groups][lodCount] record counts (zero before the launch)
    uint32_t instLods;     // instanced pass: the histogram's row length (the scene's LOD count)
    uint32_t pad2;
};

struct InstancedParams {
    SceneT sc;
    const BlzRenderObject* objects;
    uint32_t count;
    uint32_t stride;
    BlzLodInstanceCounter* counters;
    uint32_t* instances;
    uint32_t instanceCapacity;
    uint32_t slotsPerLod;
    uint8_t* cmds;
    uint32_t capacity;
    uint32_t pad;
    uint32_t* drawCount;
    uint32_t* lodBlockCounts;   // scratch: [tiles][lodCount] per-tile LOD histograms
    Scratch* scratch;
    uint32_t spinLimit;         // polls of a state before the look-back gives up (BLZ_FLAG_TIMEOUT)
    uint32_t pad1;
};

// The instanced cull's stages after the FRUSTUM decide kernel (see cull_objects.cu).
struct InstStagedParams {
    const uint2* staged;        // decide kernel output: [totalTiles * chunkSize] (objectId, lodId)
    const uint32_t* chunkCount; // [totalTiles]
    uint32_t totalTiles, chunkSize;
    uint32_t groups, nL;        // chunk groups of the counting sort, LOD count
    const uint32_t* hist;       // [groups][nL] record counts per group and LOD (the decide kernel's)
    const BlzLodData* lods;
    BlzLodInstanceCounter* counters;
    uint32_t* instances;
    uint32_t instanceCapacity, slotsPerLod;
    uint8_t* cmds;
    uint32_t stride, capacity;
    uint32_t* drawCount;
    unsigned int* status;
};

struct ClusterParams {
    SceneT sc;
    const BlzRenderObject* objects;
    uint32_t count;
    uint32_t stride;
    PyramidT pyr;
    uint32_t hasPyramid;
    uint32_t capacity;
    uint8_t* cmds;
    uint32_t* clusterIds;
    uint32_t* drawCount;
    Scratch* scratch;
    uint32_t* tileCount;  // scratch [tiles] uint2: {surviving clusters, 0} per tile (task form: {tasks, payloads})
    uint4* items;         // scratch: the test launch's work list, {object, first cluster, first slot, clusters}
    uint32_t* itemCount;  // scratch, one word: items in the list (zero between launches)
    uint32_t itemCapacity; // items the list holds: every item the call's tiles can make
    uint2* totals;        // scratch: the frame's records (task form: {tasks, payloads}), counted by the test launch
    uint2* superCount;    // scratch [cluster_tile_groups(tiles)]: the same counts per group of tiles
    // task form (blz_cull_cluster_tasks)
    uint32_t* tasks;         // BlzIndirectTask words, 4 per task
    uint32_t* payloads;      // BlzMeshTaskPayload words, 33 per payload
    uint32_t taskCapacity;
    uint32_t payloadCapacity;
    uint32_t* taskCount;
    uint32_t* payloadCount;
    uint32_t* objSurv;       // scratch [tiles * objects per tile]: surviving clusters per object
    uint2* objInfo;          // scratch [tiles * objects per tile]: {clusterOffset, clusterCount} of the chosen LOD
    float4* objXf;           // scratch [tiles * objects per tile * 2]: the object's transform {pos, scale}, {quat}
    uint32_t* bits;          // scratch [tiles * bitWords]: one visibility bit per candidate cluster, slot order
    uint32_t bitWords;       // words per tile: >= 32 objects x the largest LOD cluster count / 32
    uint32_t tiles;          // tiles of 32 objects
    uint32_t smCount;        // the device's SMs (the test launch is one wave of resident blocks)
    uint32_t testBlocksPerSm; // resident blocks of the test kernel per SM
    uint32_t* tileSlots;     // scratch [tiles]: candidate clusters of the tile
};

struct PyramidBuildParams {
    const float* depth;
    uint32_t depthWidth, depthHeight;
    float* data;
    uint32_t width, height, mipCount, mode;
    uint32_t mipOffset[BLZ_PYRAMID_MAX_MIPS];
    unsigned int* done;  // the context's finished-tile counter (zero between builds)
    uint32_t vec4;       // D3D12: depth rows read 16 bytes at a time (width % 4 == 0, height >= 2, aligned buffers)
    uint32_t spinLimit;  // one-call frame kernel: polls of the pyramid-ready flag before a warp gives up
};

// Launches a kernel with programmatic stream serialization: it may be scheduled while the kernel
// before it on the stream finishes, and waits in pdl_wait() before touching memory.
template <typename... Params, typename... Args>
inline cudaError_t launch_pdl(void (*kernel)(Params...), dim3 grid, dim3 block, size_t smem, cudaStream_t s,
                              Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, static_cast<Params>(args)...);
}

uint32_t object_tile_size();
// Chunk size of a single-view launch of `count` objects: one chunk per warp the launch holds
// resident, so every warp streams one contiguous run of objects and none waits for a second round.
// (Smaller chunks handed out by a counter measured slower: each chunk drains its survivor ring in
// a partial round, and thousands of warps contend for the counter.)
uint32_t single_chunk_size(uint32_t mode, uint32_t threads, uint32_t opt, uint32_t count, int smCount);
bool single_shape_supported(uint32_t threads, uint32_t opt);
cudaError_t launch_object_cull(uint32_t mode, const PipeParams& p, uint32_t threads, uint32_t opt, int smCount,
                               cudaStream_t s);
// A kept frame (blz_frame_first / blz_frame_late): pass 1 tests every object once and keeps the
// frustum survivors in p.keep; pass 2 runs the pyramid test over those alone. `scatter` false leaves
// the records staged.
cudaError_t launch_frame_first(const PipeParams& p, uint32_t threads, uint32_t opt, int smCount, cudaStream_t s,
                               bool scatter);
cudaError_t launch_frame_late(const PipeParams& p, int smCount, cudaStream_t s, bool scatter);
cudaError_t launch_frame_scatter2(const PipeParams& p1, const PipeParams& p2, cudaStream_t s);
// The fused sweep of blz_cull_frame (kModeFrameFused) after the pyramid: p stages pass 2's records in
// staged / chunkCount and pass 1's in staged2 / chunkCount2; no scatter.
cudaError_t launch_frame_fused(const PipeParams& p, uint32_t threads, uint32_t opt, int smCount, cudaStream_t s);
cudaError_t launch_frame_pyr(const PipeParams& p, const PyramidBuildParams& bp, uint32_t threads, uint32_t opt, int smCount,
                             cudaStream_t s);
bool batch_shape_supported(uint32_t threads, uint32_t opt);
// mode: the pass every view of the batch runs, or -1 when they differ (the kernel reads it per view)
cudaError_t launch_batch_cull(const PipeParams& p, uint32_t threads, uint32_t opt, uint32_t blocksPerSm, int smCount,
                              cudaStream_t s, int mode);
uint32_t instanced_tile_size();
constexpr uint32_t kInstStagedMaxLods = 1024;  // the staged instanced path keeps [36 to 39][LODs] words in shared memory
uint32_t instanced_group_count(uint32_t chunks);
cudaError_t launch_instanced_staged(const PipeParams& p, const InstStagedParams& q, uint32_t threads, uint32_t opt,
                                    int smCount, cudaStream_t s);
cudaError_t launch_instanced_cull(const InstancedParams& p, const BlzCameraViewData& view, cudaStream_t s);
uint32_t cluster_tile_objects();
// Groups of tiles whose counts the cluster test launch also sums, for `tiles` tiles.
uint32_t cluster_tile_groups(uint32_t tiles);
// Resident blocks per SM of the cluster test kernel (records or task form) on the current device.
cudaError_t cluster_test_blocks_per_sm(bool tasks, int* out);
// Upper bound of the cluster test launch's work items for `tiles` tiles.
uint64_t cluster_max_items(uint32_t tiles, uint32_t lodClusterMax);
cudaError_t launch_cluster_cull(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s);
cudaError_t launch_cluster_tasks(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s);
cudaError_t launch_pyramid_build(const PyramidBuildParams& p, cudaStream_t s, uint32_t* launches);
cudaError_t launch_transforms_scatter(BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                                      const BlzMeshTransform* in, uint32_t n, unsigned int* status, cudaStream_t s);
cudaError_t launch_transforms_rotate(const BlzMeshTransform* table, uint32_t tableCount, const BlzMeshTransform* dynRows,
                                     uint32_t dynCount, const uint32_t* ids, const float* axes, float angle, uint32_t n,
                                     BlzMeshTransform* dst, unsigned int* status, cudaStream_t s);
// *word += n on the stream (one thread).
cudaError_t launch_add_word(unsigned int* word, unsigned int n, cudaStream_t s);
// *out = atomicExch(status, 0) on the stream (one thread).
cudaError_t launch_take_status(unsigned int* status, unsigned int* out, cudaStream_t s);
cudaError_t launch_depth_raster(const BlzCameraViewData& view, const float* boxes, uint32_t boxCount, float* depth,
                                uint32_t width, uint32_t height, cudaStream_t s, uint32_t* launches);

}  // namespace blz
