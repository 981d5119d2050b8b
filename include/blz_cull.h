/*
 * blz_cull.h — C ABI of the GB300 culling library (libblz_cull.so).
 *
 * The library replaces the GPU-driven culling path of the Blitzen renderer: the cull compute
 * shaders, the depth-pyramid shader and the host code that binds and dispatches them. Every
 * entry point names the reference interface it stands in for (paths inside the Blitzen project).
 *
 * Conventions
 *  - Every function returns an int status: BLZ_OK (0) or one of the BLZ_ERR_* codes. The
 *    reference returns uint8_t 1/0 plus a log line; blz_last_error() gives the message of the
 *    last failing call on the calling thread.
 *  - Pointers documented as "device" are CUDA device pointers the caller owns; "host" pointers
 *    are read before the call returns (or copied to pinned staging first).
 *  - Work is enqueued on the caller's stream (a cudaStream_t passed as blz_stream_t; NULL is the
 *    legacy default stream) and runs asynchronously, exactly like a recorded dispatch.
 *  - Results are deterministic: records are written in ascending render-object order (clusters:
 *    object order, then cluster order), instance lists in ascending object order, instanced
 *    commands in ascending LOD order. The reference orders them by atomic arrival; any stable
 *    order is a valid output of the reference, and this is the one its serial execution gives.
 *  - Capacity overflow never writes out of bounds: records past the capacity are counted but
 *    not stored, and a device-side status flag is raised (read it with blz_ctx_check).
 *  - One context serves one stream at a time; two streams need two contexts (each context
 *    owns the scratch state of its single-pass kernels).
 */
#ifndef BLZ_CULL_H
#define BLZ_CULL_H

#include <stddef.h>
#include <stdint.h>
#include "blz_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CUstream_st* blz_stream_t; /* identical to cudaStream_t */
typedef struct blz_ctx blz_ctx;
typedef struct blz_server blz_server;
typedef struct blz_batch_graph blz_batch_graph;

/* ---------------------------------------------------------------- status codes */
enum {
    BLZ_OK = 0,
    BLZ_ERR_INVALID_ARGUMENT = 1,
    BLZ_ERR_CAPACITY = 2,      /* an output buffer was too small; extra records were dropped */
    BLZ_ERR_OUT_OF_MEMORY = 3,
    BLZ_ERR_TIMEOUT = 4,       /* a bounded wait expired (device or host side) */
    BLZ_ERR_CUDA = 5,          /* a CUDA runtime call failed; see blz_last_error() */
    BLZ_ERR_BAD_INDEX = 6,     /* a scene table referenced an id past the end of its table */
    BLZ_ERR_NOT_READY = 7,     /* asynchronous result not available yet */
    BLZ_ERR_NO_SCENE = 8       /* cull called before blz_scene_upload */
};

/* Device-side status flags, OR-ed by kernels and read (and cleared) by blz_ctx_check. */
enum {
    BLZ_FLAG_COMMAND_OVERFLOW = 1u,  /* more visible records than BlzCullTarget.capacity */
    BLZ_FLAG_INSTANCE_OVERFLOW = 2u, /* a LOD received more instances than its slot range */
    BLZ_FLAG_BAD_INDEX = 4u,         /* transformId / surfaceId / LOD range out of range */
    BLZ_FLAG_TIMEOUT = 8u            /* a bounded spin-wait in a single-pass kernel gave up */
};

/* Record strides: Vulkan IndirectDrawData (24 B) or D3D12 IndirectDrawCmd (32 B). */
#define BLZ_STRIDE_VULKAN 24u
#define BLZ_STRIDE_D3D12 32u

/* Hi-Z semantics. D3D12 (default): mip 0 = depth extent / 2, 2x2 integer-load min per level,
 * one-texel Load in the occlusion test (depthPyramid.cs.hlsl, hlslMath.hlsl:58-78).
 * VULKAN: mip 0 = previous power of two of the depth extent, min-reduction bilinear footprint
 * (DepthPyramidGeneration.comp.glsl, CullingShaderData.glsl:60-73). */
#define BLZ_HIZ_D3D12 0u
#define BLZ_HIZ_VULKAN 1u
#define BLZ_PYRAMID_MAX_MIPS 16u

/* ---------------------------------------------------------------- context */

/* Creates a context on a CUDA device: scratch for the single-pass kernels, the status word and
 * pinned staging. Replaces the renderer setup of the cull resources
 * (src/Renderer/BlitzenVulkan/vulkanRendererSetup.cpp:453-522, vulkanRenderer.h:20-40). */
int blz_ctx_create(int device, blz_ctx** outCtx);
int blz_ctx_destroy(blz_ctx* ctx);

/* Message of the last failing call made on this thread ("" if none). */
const char* blz_last_error(void);

/* Library version string (name, version, target architecture). */
const char* blz_version(void);

/* Synchronises the stream, returns the device status flags raised since the last check and
 * clears them. Returns BLZ_ERR_CAPACITY / BLZ_ERR_BAD_INDEX / BLZ_ERR_TIMEOUT when the matching
 * flag is set, else BLZ_OK. flagsOut may be NULL. Stands in for the reference's fence wait plus
 * the validation it never had (vulkanData.h:196-197). */
int blz_ctx_check(blz_ctx* ctx, blz_stream_t stream, uint32_t* flagsOut);

/* Bound of the device-side waits of this context's launches. Two kernels wait:
 *  - the single-kernel instanced cull (scenes of more than 1,024 LODs): a tile waits, per LOD, for
 *    the running totals of the tiles that started before it;
 *  - the one-call frame given a depth buffer (blz_cull_frame): a warp waits, before its first Hi-Z
 *    test, for the pyramid the launch's blocks build first.
 * Each polls one word at most `polls` times; then it gives up, raises BLZ_FLAG_TIMEOUT and finishes
 * without waiting (its results are then wrong; blz_ctx_check returns BLZ_ERR_TIMEOUT and resets the
 * instanced protocol). 0 restores the default (2^20 polls, about a second at worst). Stands in for
 * the bounded fence wait of the reference's frame loop (vulkanData.h:196-197, ce_fenceTimeout). */
int blz_ctx_set_wait_limit(blz_ctx* ctx, uint32_t polls);

/* Test hook for the timeout path only: advances the context's block-ticket counter by n (1..1024)
 * on the stream, so that the next launch that takes tickets starts its blocks past the first n
 * places. Its blocks then wait for places no block holds, give up after the wait limit and raise
 * BLZ_FLAG_TIMEOUT; the launch's last block rewinds the counter, so the launch after it is whole
 * again. No counterpart in the reference. */
int blz_ctx_debug_advance_ticket(blz_ctx* ctx, uint32_t n, blz_stream_t stream);

/* Test hook for the one-call frame's wait only: advances the context's pyramid-tile ticket by n
 * (1..1024) on the stream, so that the next blz_cull_frame given a depth buffer never builds the
 * pyramid's first n tiles. Its warps then wait for a pyramid that is never finished, give up after
 * the wait limit and raise BLZ_FLAG_TIMEOUT (their records are then wrong); the frame's last launch
 * rewinds the ticket, so the frame after it is whole again. No counterpart in the reference. */
int blz_ctx_debug_skip_frame_tiles(blz_ctx* ctx, uint32_t n, blz_stream_t stream);

/* Number of this library's kernel launches enqueued by the context so far. */
uint64_t blz_ctx_launch_count(const blz_ctx* ctx);

/* ---------------------------------------------------------------- scene residency */

typedef struct BlzSceneDesc {
    const BlzRenderObject* renderObjects;   /* default render list (may be NULL) */
    uint32_t renderObjectCount;
    const BlzMeshTransform* transforms;
    uint32_t transformCount;
    const BlzPrimitiveSurface* surfaces;
    uint32_t surfaceCount;
    const BlzLodData* lods;
    uint32_t lodCount;
    const BlzCluster* clusters;              /* may be NULL when no cluster culling is done */
    uint32_t clusterCount;
} BlzSceneDesc;

#define BLZ_SCENE_COPY_FROM_HOST 0u   /* pointers are host memory; the library copies */
#define BLZ_SCENE_BORROW_DEVICE 1u    /* pointers are device memory the caller keeps alive */

/* Makes a scene resident: render objects, transforms, surfaces, LODs, clusters in the reference
 * layouts. Replaces StaticBuffersInit / SetupForRendering
 * (src/Renderer/BlitzenVulkan/vulkanRendererSetup.cpp:453-522, dx12Renderer.h:22-43).
 * Borrowed device tables must be aligned: transforms to 32 bytes (one transform is read in a
 * single 32-byte load), surfaces, LODs and clusters to 16, render objects to 8.
 * The LOD table is read once here (a borrowed one too, synchronously) for its largest cluster
 * range, which sizes the cluster cull's visibility bits and work list: an object whose chosen LOD's
 * clusterCount was raised past that afterwards emits nothing from the cluster culls, which raise
 * BLZ_FLAG_BAD_INDEX. */
int blz_scene_upload(blz_ctx* ctx, const BlzSceneDesc* scene, uint32_t flags, blz_stream_t stream);

/* Device pointers of the resident tables (for callers that build render lists on the device). */
int blz_scene_device_tables(const blz_ctx* ctx, BlzSceneDesc* out);

/* Overwrites transforms[ids[i]] = transforms_in[i] for i < n. ids and transforms_in are host
 * arrays, copied into the context's pinned buffer, which the update kernel reads directly.
 * Replaces UpdateObjectTransform + UpdateBuffers (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:46-60,816-820). */
int blz_transforms_update(blz_ctx* ctx, const uint32_t* ids, const BlzMeshTransform* transformsIn,
                          uint32_t n, blz_stream_t stream);

/* Same, with ids and transforms in device-accessible memory (device memory, or pinned host memory
 * the kernel reads directly); recordable in a captured frame. */
int blz_transforms_update_device(blz_ctx* ctx, const uint32_t* dIds, const BlzMeshTransform* dTransforms,
                                 uint32_t n, blz_stream_t stream);

/* Device-side rotation of dynamic objects: for i < n, writes dDst[i] = transforms[dIds[i]] with its
 * orientation replaced by q_i (x) orientation (Hamilton product), q_i = (sin(a/2) axis_i, cos(a/2)),
 * axis_i = dAxes[3i..3i+2] (unit vectors), a = angle. dDst is a device buffer of n transforms (it
 * can be scattered back with blz_transforms_update_device, or used as a per-view override of the
 * dynamic rows in a batch). The dynamic-object rotation of src/Game/blitzenObject.cpp:30-46 as a
 * kernel. */
int blz_transforms_rotate(blz_ctx* ctx, const uint32_t* dIds, const float* dAxes, float angle,
                          uint32_t n, BlzMeshTransform* dDst, blz_stream_t stream);

/* Binds the scene's dynamic rows: from the next call on, every cull and blz_transforms_rotate of
 * this context reads transforms [0, count) from rows[] instead of the resident table (count 0
 * unbinds). rows is device-accessible memory, 32-byte aligned: device memory, or pinned host memory
 * that the kernels read over the CPU-GPU link, so the renderer's mapped staging buffer can serve
 * directly. The reference keeps its dynamic objects in transforms [0, 1000)
 * (src/Renderer/blitRender.h:10), rewrites them through that staging buffer
 * (UpdateObjectTransform, src/Renderer/BlitzenVulkan/vulkanDraw.cpp:46-60) and copies it to the
 * device table every frame (UpdateBuffers, vulkanDraw.cpp:816-820); bound rows replace that copy.
 * blz_transforms_update writes the resident table, which bound rows hide for ids < count. A recorded
 * frame keeps the binding it was recorded with; blz_scene_upload unbinds. Host-side only. */
int blz_scene_bind_dynamic(blz_ctx* ctx, const BlzMeshTransform* rows, uint32_t count);

/* ---------------------------------------------------------------- depth pyramid */

typedef struct BlzPyramid {
    float* data;                 /* device storage, mips back to back, each row-major */
    uint32_t width;              /* mip 0 extent = CameraViewData.pyramidWidth */
    uint32_t height;             /* mip 0 extent = CameraViewData.pyramidHeight */
    uint32_t mipCount;
    uint32_t mode;               /* BLZ_HIZ_D3D12 or BLZ_HIZ_VULKAN */
    uint32_t depthWidth;         /* source depth-buffer extent */
    uint32_t depthHeight;
    uint32_t mipOffset[BLZ_PYRAMID_MAX_MIPS]; /* offset of each mip in floats */
} BlzPyramid;

/* Fills every field but data for a depth buffer of depthWidth x depthHeight and returns the
 * bytes data must hold (0 on bad arguments). D3D12: mip 0 = max(1, W>>1) x max(1, H>>1)
 * (src/Renderer/BlitzenDX12/dx12RNDResources.cpp:96-118); Vulkan: PreviousPow2 of each
 * (src/Renderer/BlitzenVulkan/vulkanResources.cpp:87-95). Mip count per GetDepthPyramidMipLevels
 * (src/BlitzenMathLibrary/blitML.h:95-107). */
uint64_t blz_pyramid_layout(uint32_t depthWidth, uint32_t depthHeight, uint32_t mode, BlzPyramid* out);

/* Builds every mip from an fp32 reverse-Z depth buffer (row-major, depthWidth floats per row):
 * one launch for the 32x32 tiles and one for the top mips. Replaces GenerateDepthPyramid
 * (src/Renderer/BlitzenDX12/dx12Draw.cpp:224-288, src/Renderer/BlitzenVulkan/vulkanDraw.cpp:554-622)
 * and its per-mip dispatches of depthPyramid.cs.hlsl / DepthPyramidGeneration.comp.glsl.
 * dDepth is any device-accessible pointer: device memory, or pinned host memory that the kernel
 * then reads once over the CPU-GPU link (no separate upload). */
int blz_pyramid_build(blz_ctx* ctx, const BlzPyramid* pyramid, const float* dDepth, blz_stream_t stream);

/* Rasterises axis-aligned occluder boxes (world space, 6 floats each: min xyz, max xyz) into a
 * device fp32 reverse-Z depth buffer for one view: clears to 0, then every box writes
 * zNear / zFarthestCorner over its projected screen rectangle (max-depth test). A stand-in for
 * the reference's depth pre-pass, which is a graphics-API rasterisation. */
int blz_depth_raster_boxes(blz_ctx* ctx, const BlzCameraViewData* view, const float* dBoxes, uint32_t boxCount,
                           float* dDepth, uint32_t width, uint32_t height, blz_stream_t stream);

/* ---------------------------------------------------------------- single-view culls */

typedef struct BlzRenderList {
    const BlzRenderObject* objects;  /* device; NULL = the scene's default render list */
    uint32_t count;                  /* drawCount / objCount push constant */
} BlzRenderList;

typedef struct BlzCullTarget {
    void* commands;          /* device: records of `stride` bytes */
    uint32_t stride;         /* BLZ_STRIDE_VULKAN or BLZ_STRIDE_D3D12 */
    uint32_t capacity;       /* records the buffer can hold */
    uint32_t* drawCount;     /* device-accessible (device or pinned host memory): set to the number
                              * of visible records (not accumulated) */
} BlzCullTarget;

/* Frustum + LOD cull of every object, no occlusion, no visibility state.
 * Replaces TransparentDrawCull.comp.glsl:13-65 and drawCull.cs.hlsl:10-52 with their dispatch
 * (DrawCullPass, src/Renderer/BlitzenDX12/dx12Draw.cpp:150-184). view is a host pointer. */
int blz_cull_frustum(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                     const BlzCullTarget* target, blz_stream_t stream);

/* blz_cull_frustum without any device allocation. It has no counterpart in the reference: it
 * exists for callers that cannot allocate device memory once running (their memory is reserved
 * up front, or they must not wait on the device-wide synchronisation of cudaFree). Its per-call
 * staging is a fixed device array inside this library, for at most BLZ_NOALLOC_MAX_OBJECTS render
 * objects (8 MiB); longer lists return BLZ_ERR_CAPACITY. Results equal blz_cull_frustum's.
 * The first call on each context fetches that array's address (cudaGetSymbolAddress) and keeps it
 * in the context, so make it before any stream capture (a first call inside a capture returns
 * BLZ_ERR_INVALID_ARGUMENT). The array is shared by every context on the device: calls that
 * overlap on the device race on it and must be ordered. */
#define BLZ_NOALLOC_MAX_OBJECTS (1u << 20)
int blz_cull_frustum_noalloc(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                             const BlzCullTarget* target, blz_stream_t stream);

/* Occlusion pass 1: objects with visibility[i] != 0 are frustum-tested and, when visible, emitted.
 * visibility is a device uint32 per render object (read only here).
 * Replaces InitialDrawCull.comp.glsl:12-59 / drawOccFirst.cs.hlsl:13-58 and DrawCullFirstPass
 * (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:107-158). */
int blz_cull_first(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                   const uint32_t* dVisibility, const BlzCullTarget* target, blz_stream_t stream);

/* Occlusion pass 2: every object is frustum- and Hi-Z-tested against the pyramid; objects visible
 * now but not last frame are emitted; visibility[i] is rewritten to 1/0.
 * Replaces LateDrawCull.comp.glsl:13-72 / drawOccLate.cs.hlsl:13-67 and DrawCullOcclusionPass
 * (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:162-226). */
int blz_cull_late(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                  uint32_t* dVisibility, const BlzPyramid* pyramid, const BlzCullTarget* target,
                  blz_stream_t stream);

/* Kept frame: the two occlusion passes of one frame with the frustum work done once.
 * The reference's frame is UpdateBuffers, pass 1, the pass-1 draw, the depth pyramid, pass 2
 * (VulkanRenderer::DrawFrame, src/Renderer/BlitzenVulkan/vulkanDraw.cpp:830,1015-1031): both passes
 * see the same view, transforms and render list. blz_frame_first runs pass 1 over every object of the
 * list: it writes pass 1's records exactly as blz_cull_first does, and keeps every object inside the
 * frustum (with its view-space sphere, in context memory) for blz_frame_late, which tests only those
 * against the pyramid and writes pass 2's records exactly as blz_cull_late does. Together they leave
 * the same records, counts and visibility as blz_cull_first + blz_cull_late.
 * Contract: between the two calls the scene tables, bound dynamic rows, render list and visibility
 * buffer must not change (the renderer's own frame guarantees this). blz_frame_first already writes
 * the final visibility (0) of the objects it found outside the frustum; blz_frame_late rewrites the
 * rest. blz_frame_late uses the last blz_frame_first of the context (BLZ_ERR_INVALID_ARGUMENT if
 * there is none). Replaces DrawCullFirstPass / DrawCullOcclusionPass (vulkanDraw.cpp:107-226),
 * drawOccFirst.cs.hlsl:13-58 and drawOccLate.cs.hlsl:13-67. */
int blz_frame_first(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list, uint32_t* dVisibility,
                    const BlzCullTarget* pass1Target, blz_stream_t stream);
int blz_frame_late(blz_ctx* ctx, const BlzPyramid* pyramid, const BlzCullTarget* pass2Target, blz_stream_t stream);

/* The whole frame in one call for a caller whose depth buffer is ready before pass 1 (an occluder
 * depth pass, a reprojected previous depth): the pyramid is built from dDepth first, then one sweep
 * tests every object once against the frustum and its survivors against the pyramid, and sorts each
 * object into pass 1's records (visible last frame, inside the frustum), pass 2's (not visible last
 * frame, inside the frustum, not occluded) or neither, rewriting the visibility as pass 2 does; one
 * final launch writes both record lists. Same records, counts, pyramid and visibility as
 * blz_cull_first + blz_pyramid_build + blz_cull_late on the same inputs. It keeps nothing for
 * blz_frame_late. With dDepth, the launch's blocks build the pyramid's tiles before their share of
 * the sweep and each warp waits for the finished pyramid before its first Hi-Z test (a bounded
 * wait, see blz_ctx_set_wait_limit). dDepth NULL: the pyramid is used as it stands (a caller that
 * built it itself, with blz_pyramid_build earlier or from another frame's depth). Replaces the pass order of
 * VulkanRenderer::DrawFrame (vulkanDraw.cpp:1015-1031) and dx12Draw.cpp:590-641 minus the draws. */
int blz_cull_frame(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list, uint32_t* dVisibility,
                   const float* dDepth, const BlzPyramid* pyramid, const BlzCullTarget* pass1Target,
                   const BlzCullTarget* pass2Target, blz_stream_t stream);

/* Single-pass occlusion against a pyramid (last frame's), no visibility state.
 * Replaces drawOccTemporal.hlsl:13-64. */
int blz_cull_temporal(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                      const BlzPyramid* pyramid, const BlzCullTarget* target, blz_stream_t stream);

/* Instanced cull: resets counters[l].instanceCount for every LOD, writes each visible object's id
 * into instances[counters[l].instanceOffset + slot] for its chosen LOD l (slot < slotsPerLod),
 * then emits one command per LOD with a non-zero count: {objId = instanceOffset, indexCount,
 * instCount = count, indexOffset = firstIndex, 0, 0}. counters is a device array of the scene's
 * LOD count; instanceCapacity bounds every write into instances.
 * Replaces drawInstCountReset.cs.hlsl + drawInstCull.cs.hlsl + drawInstCmd.cs.hlsl and
 * DrawInstanceCullPass (src/Renderer/BlitzenDX12/dx12Draw.cpp:340-415). */
int blz_cull_instanced(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                       BlzLodInstanceCounter* dCounters, uint32_t* dInstances, uint32_t instanceCapacity,
                       uint32_t slotsPerLod, const BlzCullTarget* target, blz_stream_t stream);

/* Cluster cull: object frustum + LOD select, then for every cluster of the chosen LOD a sphere
 * frustum test, a Hi-Z test (when pyramid != NULL) and a normal-cone backface test. Each surviving
 * cluster emits {objectId, triangleCount*3, 1, dataOffset, 0, 0} and, when dClusterIds != NULL,
 * its global cluster index into dClusterIds (same slot). Replaces PreClusterDrawCull.comp.glsl
 * + InitialClusterCull.comp.glsl and the CPU read-back between them
 * (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:318-423,874-905). */
int blz_cull_clusters(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                      const BlzPyramid* pyramid, const BlzCullTarget* target, uint32_t* dClusterIds,
                      blz_stream_t stream);

typedef struct BlzTaskTarget {
    BlzIndirectTask* tasks;          /* device: one task per object with a surviving cluster */
    BlzMeshTaskPayload* payloads;    /* device: ceil(survivors / 32) payloads per such object */
    uint32_t taskCapacity;           /* tasks the buffer can hold */
    uint32_t payloadCapacity;        /* payloads the buffer can hold */
    uint32_t* taskCount;             /* device-accessible: set to the number of tasks (not accumulated) */
    uint32_t* payloadCount;          /* device-accessible: set to the number of payloads */
} BlzTaskTarget;

/* Cluster cull into the mesh-shader form: the same object and cluster tests as blz_cull_clusters,
 * with each object's surviving clusters packed 32 to a task payload instead of one draw per
 * cluster. For every object o (ascending render-list index) with s >= 1 surviving clusters:
 *   tasks[t]            = {taskId = p, groupCountX = ceil(s / 32), 1, 1}, t = objects before o
 *                         with a surviving cluster;
 *   payloads[p + g]     = {drawId = o, meshletIndices = surviving cluster indices 32g .. 32g+31 in
 *                         ascending order, BLZ_NO_MESHLET past the last}, p = payloads of the
 *                         objects before o.
 * A task shader launched with groupCountX workgroups reads payloads[tasks[drawID].taskId +
 * workGroupID.x] and emits one mesh workgroup per valid slot; the mesh shader reads the payload as
 * MeshShader.mesh.glsl:22-25 does. Records past a capacity are not written; the counts are the
 * full counts and an overflow sets BLZ_FLAG_COMMAND_OVERFLOW. The reference declares this format
 * (ShaderBuffers.glsl:86-92,203-206; consumers MeshShader.task.glsl, MeshShader.mesh.glsl) but
 * its writer is disabled (vulkanDraw.cpp:425-436). */
int blz_cull_cluster_tasks(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list,
                           const BlzPyramid* pyramid, const BlzTaskTarget* target, blz_stream_t stream);

/* ---------------------------------------------------------------- batched views */

#define BLZ_MODE_FRUSTUM 0u
#define BLZ_MODE_FIRST 1u
#define BLZ_MODE_LATE 2u
#define BLZ_MODE_TEMPORAL 3u

typedef struct BlzBatchView {
    BlzCameraViewData view;          /* the view's cull uniform */
    BlzRenderList list;              /* its render objects */
    uint32_t mode;                   /* BLZ_MODE_* */
    uint32_t reserved0;
    uint32_t* visibility;            /* device; FIRST and LATE */
    const BlzPyramid* pyramid;       /* host descriptor; LATE and TEMPORAL */
    BlzCullTarget target;
    const BlzMeshTransform* dynamicTransforms; /* device, 32-byte aligned; overrides transforms[0, dynamicCount) */
    uint32_t dynamicCount;
    uint32_t reserved1;
} BlzBatchView;

/* Culls many views of uneven size in one persistent launch: a device work queue of
 * (view, object tile) items, per-view stable compaction. The reference has one camera and one
 * dispatch per pass (src/Core/blitzenEngine.h:49); this is the many-view form of the same passes. */
int blz_cull_batch(blz_ctx* ctx, const BlzBatchView* views, uint32_t viewCount, blz_stream_t stream);

/* Same work as blz_cull_batch, as one dispatch per view (the baseline the batch is compared to). */
int blz_cull_batch_per_view(blz_ctx* ctx, const BlzBatchView* views, uint32_t viewCount, blz_stream_t stream);

/* Captures blz_cull_batch for a fixed set of views into a CUDA graph and replays it. The views'
 * buffers must stay valid for the life of the graph; view data may be changed between replays
 * with blz_batch_graph_set_view, which writes the graph's copy of the view at once (a synchronous
 * copy): call it only when no replay of the graph is still running, as for any buffer a recorded
 * command reads. */
int blz_batch_graph_create(blz_ctx* ctx, const BlzBatchView* views, uint32_t viewCount,
                           blz_stream_t stream, blz_batch_graph** outGraph);
int blz_batch_graph_set_view(blz_batch_graph* g, uint32_t viewIndex, const BlzCameraViewData* view);
int blz_batch_graph_launch(blz_batch_graph* g, blz_stream_t stream);
int blz_batch_graph_destroy(blz_batch_graph* g);

/* Launch shape used by the batch kernel: threads per block, objects per thread, blocks per SM and
 * objects per chunk (the compaction unit: each chunk's records are staged and counted together;
 * 256, 512 or 1024, 0 = 512). blz_set_launch_shape also sets the single-view kernels' threads and
 * objects per thread when they have that shape (256 x 1, 2 or 4; 128 x 2 or 4; 512 x 1), and
 * forgets every choice the autotuners cached. A batch whose views all run the same pass uses a
 * kernel compiled for that pass for 256 x 1 and 512 x 1.
 *
 * blz_autotune_batch times every batch shape (threads x objects per thread x blocks per SM x chunk
 * size) on the given batch, keeps the fastest as the context's shape and caches it for the batch's
 * size (total objects, view count): later batches of that size use it, whatever the context's
 * shape, and a later call for that size returns the cached choice without timing again. The
 * reference has one fixed shape, N/64 + 1 groups of 64 threads (blitML.h:64-67). */
typedef struct BlzLaunchShape {
    uint32_t threadsPerBlock;
    uint32_t objectsPerThread;
    uint32_t blocksPerSm;
    uint32_t chunkObjects;
} BlzLaunchShape;
int blz_get_launch_shape(const blz_ctx* ctx, BlzLaunchShape* out);
int blz_set_launch_shape(blz_ctx* ctx, const BlzLaunchShape* shape);
int blz_autotune_batch(blz_ctx* ctx, const BlzBatchView* views, uint32_t viewCount, uint32_t repeats,
                       blz_stream_t stream, BlzLaunchShape* best, float* bestMicroseconds);

/* Times the single-view pass `mode` (BLZ_MODE_FRUSTUM, FIRST, LATE or TEMPORAL) on the given view,
 * list, pyramid and target under every single-view shape (256 x 1, 2, 4; 128 x 2, 4; 512 x 1), each
 * `repeats` times (0: 5) after one untimed run, and caches the fastest for (list size, pass): later
 * single-view culls of that size and pass use it. The visibility buffer is read but never changed:
 * each run works on a copy. The target's records and count are overwritten. best gets the shape,
 * with chunkObjects = the chunk the single-view kernels use for it (one chunk per resident warp);
 * a second call for the same size and pass returns the cached choice. Refused inside a capture. */
int blz_autotune_single(blz_ctx* ctx, const BlzCameraViewData* view, BlzRenderList list, uint32_t mode,
                        const uint32_t* dVisibility, const BlzPyramid* pyramid, const BlzCullTarget* target,
                        uint32_t repeats, blz_stream_t stream, BlzLaunchShape* best, float* bestMicroseconds);

/* ---------------------------------------------------------------- recorded frames */

typedef struct blz_graph blz_graph;

/* Records every library call enqueued on `stream` between begin and end into a CUDA graph (stream
 * capture, thread-local mode) and instantiates it; blz_graph_launch replays the whole sequence with
 * one launch. Buffers, views and counts are the ones of the recorded calls. A first, unrecorded
 * run of the same calls sizes the library's scratch, so nothing is allocated while recording.
 * The reference records the same passes into a command buffer once per frame
 * (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:822-1122). kernelsOut (may be NULL) receives the
 * number of this library's kernels in the graph. */
int blz_capture_begin(blz_ctx* ctx, blz_stream_t stream);
int blz_capture_end(blz_ctx* ctx, blz_stream_t stream, blz_graph** outGraph, uint32_t* kernelsOut);
int blz_graph_launch(blz_graph* graph, blz_stream_t stream);
int blz_graph_destroy(blz_graph* graph);

/* ---------------------------------------------------------------- serving loop */

typedef struct BlzServeConfig {
    uint64_t outputPoolBytes;   /* device memory for request outputs; 0 = a quarter of free memory */
    uint32_t maxInFlight;       /* batches on the device at once (streams) */
    uint32_t maxBatchViews;     /* requests per batch */
    uint32_t dynamicCount;      /* transforms [0, dynamicCount) are per-request */
    uint32_t stride;            /* record stride for request outputs */
} BlzServeConfig;

typedef struct BlzServeRequest {
    BlzCameraViewData view;
    BlzRenderList list;             /* device render list (resident scene) */
    uint32_t mode;                  /* BLZ_MODE_FRUSTUM or BLZ_MODE_TEMPORAL */
    uint32_t rotateCount;           /* dynamic objects to rotate for this request (<= dynamicCount) */
    const BlzPyramid* pyramid;      /* host descriptor, TEMPORAL only */
    const float* rotateAxes;        /* host, rotateCount unit vectors */
    float rotateAngle;
    uint32_t copyToHost;            /* copy records back to host memory on completion */
} BlzServeRequest;

typedef struct BlzServeResult {
    uint32_t status;
    uint32_t drawCount;
    const void* deviceRecords;      /* device; valid until blz_serve_release */
    const void* hostRecords;        /* valid until blz_serve_release (copyToHost != 0) */
    double arrivalSeconds;          /* host monotonic clock */
    double completeSeconds;
} BlzServeResult;

typedef struct BlzServeStats {
    uint64_t submitted, completed, batches, objects;
    double p50Ms, p99Ms, meanMs, maxMs;
    uint64_t peakOutputBytes;
    uint32_t maxConcurrentBatches;
    uint32_t maxBatchSize;
} BlzServeStats;

/* A request loop over the resident scene: admits requests as output memory and in-flight slots
 * free up, batches what is waiting into one batch launch, overlaps batches on several streams. */
int blz_serve_create(blz_ctx* ctx, const BlzServeConfig* config, blz_server** outServer);
int blz_serve_submit(blz_server* s, const BlzServeRequest* request, uint64_t* ticketOut);
int blz_serve_wait(blz_server* s, uint64_t ticket, uint32_t timeoutMs, BlzServeResult* out);
int blz_serve_release(blz_server* s, uint64_t ticket);
int blz_serve_stats(blz_server* s, BlzServeStats* out);
int blz_serve_destroy(blz_server* s);

/* ---------------------------------------------------------------- view constants (host) */

/* Builds the cull uniform the way the reference camera does: view = inverse(T(position) *
 * R(yaw about -Y) * R(pitch about +X)), infinite reverse-Z projection, symmetric frustum planes,
 * proj0/proj5, lodTarget = (2 / proj5) / windowHeight.
 * Restates SetupCamera + UpdateProjection (src/Game/blitzenCamera.cpp:14-41,93-126). fovRadians
 * is the vertical field of view. */
int blz_view_setup(BlzCameraViewData* out, float fovRadians, float windowWidth, float windowHeight,
                   float zNear, float zFar, const float position[3], float yawRadians, float pitchRadians,
                   float pyramidWidth, float pyramidHeight);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* BLZ_CULL_H */
