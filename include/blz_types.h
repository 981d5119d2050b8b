/*
 * blz_types.h — byte-exact mirrors of the Blitzen GPU-driven culling buffer layouts.
 *
 * Every struct here has the size, field order and alignment of the reference struct it
 * mirrors, so a scene uploaded from the reference's own CPU-side arrays needs no repacking.
 * The static size checks at the end of this file hold the layouts in place.
 *
 * Reference structs (paths inside the Blitzen project):
 *   BlzRenderObject        src/Renderer/Resources/renderingResourcesTypes.h:155-159  (RenderObject, 8 B)
 *   BlzMeshTransform       src/Renderer/Resources/renderingResourcesTypes.h:124-129  (MeshTransform, 32 B)
 *   BlzPrimitiveSurface    src/Renderer/Resources/renderingResourcesTypes.h:104-116  (PrimitiveSurface, 32 B)
 *   BlzLodData             src/Renderer/Resources/renderingResourcesTypes.h:73-96    (LodData, 32 B)
 *   BlzLodInstanceCounter  src/Renderer/Resources/renderingResourcesTypes.h:98-102   (LodInstanceCounter, 8 B)
 *   BlzCluster             src/Renderer/Resources/renderingResourcesTypes.h:27-47    (Cluster, 32 B)
 *   BlzIndirectDraw        src/Renderer/VulkanShaderHeaders/ShaderBuffers.glsl:73-84,
 *                          src/Renderer/BlitzenVulkan/vulkanData.h:429-433           (IndirectDrawData, 24 B)
 *   BlzDrawCmd             src/Renderer/HlslShaders/Headers/cullBuffers.hlsl:1-15,
 *                          src/Renderer/BlitzenDX12/dx12Data.h:284-296               (IndirectDrawCmd, 32 B)
 *   BlzClusterDispatchData src/Renderer/BlitzenVulkan/vulkanData.h:442-447           (ClusterDispatchData, 12 B)
 *   BlzCameraViewData      src/Game/blitCamera.h:38-64                                (CameraViewData, 256 B)
 *
 * Plain C: usable from C, C++ and CUDA translation units alike.
 */
#ifndef BLZ_TYPES_H
#define BLZ_TYPES_H

#include <stdint.h>

#if defined(__cplusplus)
#define BLZ_ALIGN(n) alignas(n)
#else
#define BLZ_ALIGN(n) _Alignas(n)
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* One drawable instance: which transform and which surface (mesh primitive) it uses. */
typedef struct BlzRenderObject {
    uint32_t transformId;   /* index into the MeshTransform table */
    uint32_t surfaceId;     /* index into the PrimitiveSurface table */
} BlzRenderObject;

/* World transform of one instance: position, uniform scale, orientation quaternion (x,y,z,w). */
typedef struct BlzMeshTransform {
    BLZ_ALIGN(16) float pos[3];
    float scale;
    float orientation[4];
} BlzMeshTransform;

/* Mesh primitive: model-space bounding sphere and its range of LODs in the LodData table. */
typedef struct BlzPrimitiveSurface {
    BLZ_ALIGN(16) float center[3];
    float radius;
    uint32_t materialId;
    uint32_t lodOffset;
    uint32_t lodCount;
    uint32_t vertexOffset;
} BlzPrimitiveSurface;

/* One level of detail: index range for the plain draw path, cluster range for the cluster path,
 * and the simplification error used by LOD selection. */
typedef struct BlzLodData {
    BLZ_ALIGN(16) uint32_t indexCount;
    uint32_t firstIndex;
    uint32_t clusterOffset;
    uint32_t clusterCount;
    float error;
    uint32_t padding0;
    uint32_t padding1;
    uint32_t padding2;
} BlzLodData;

/* Per-LOD instance list descriptor for the instanced path: where the LOD's instance ids start
 * in the instance buffer and how many were written this frame. */
typedef struct BlzLodInstanceCounter {
    uint32_t instanceOffset;
    uint32_t instanceCount;
} BlzLodInstanceCounter;

/* Meshlet: bounding sphere, int8-snorm normal cone (axis xyz, cutoff), index data offset. */
typedef struct BlzCluster {
    BLZ_ALIGN(16) float center[3];
    float radius;
    int8_t coneAxisX;
    int8_t coneAxisY;
    int8_t coneAxisZ;
    int8_t coneCutoff;
    uint32_t dataOffset;
    uint8_t vertexCount;
    uint8_t triangleCount;
    uint8_t padding0;
    uint8_t padding1;
} BlzCluster;

/* Vulkan indirect record: object id followed by VkDrawIndexedIndirectCommand (stride 24). */
typedef struct BlzIndirectDraw {
    uint32_t objectId;
    uint32_t indexCount;
    uint32_t instanceCount;
    uint32_t firstIndex;
    int32_t  vertexOffset;
    uint32_t firstInstance;
} BlzIndirectDraw;

/* D3D12 indirect record: object id, D3D12_DRAW_INDEXED_ARGUMENTS, two pad words (stride 32).
 * The cull kernels write the first six words and leave the pad words untouched, as the
 * reference shaders do. */
typedef struct BlzDrawCmd {
    uint32_t objId;
    uint32_t indexCount;
    uint32_t instCount;
    uint32_t indexOffset;
    int32_t  vertOffset;
    uint32_t insOffset;
    uint32_t padding0;
    uint32_t padding1;
} BlzDrawCmd;

/* The reference's materialised cluster work item (the CUDA path never materialises it; it is
 * kept for callers that still consume the two-stage Vulkan format). */
typedef struct BlzClusterDispatchData {
    uint32_t objectId;
    uint32_t lodIndex;
    uint32_t clusterId;
} BlzClusterDispatchData;

/* Mesh-shader draw record: the task id the task shader reads, followed by
 * VkDrawMeshTasksIndirectCommandEXT (IndirectTask, VulkanShaderHeaders/ShaderBuffers.glsl:86-92;
 * IndirectTaskData, src/Renderer/BlitzenVulkan/vulkanData.h:435-439). Stride 16; the indirect
 * draw reads the group counts at offset 4. */
typedef struct BlzIndirectTask {
    uint32_t taskId;
    uint32_t groupCountX;
    uint32_t groupCountY;
    uint32_t groupCountZ;
} BlzIndirectTask;

/* Task-to-mesh amplification payload: the draw and up to 32 meshlets, one mesh workgroup per
 * meshlet (MeshTaskPayload, VulkanShaderHeaders/ShaderBuffers.glsl:203-206). 132 bytes. Slots
 * past the last meshlet of a payload hold BLZ_NO_MESHLET. */
typedef struct BlzMeshTaskPayload {
    uint32_t drawId;
    uint32_t meshletIndices[32];
} BlzMeshTaskPayload;

#define BLZ_NO_MESHLET 0xFFFFFFFFu

/* The 256-byte cull uniform. Matrices are column-major: element (row r, column c) is
 * data[c * 4 + r], translation in data[12..14]. */
typedef struct BlzCameraViewData {
    BLZ_ALIGN(256) float viewMatrix[16];
    float projectionViewMatrix[16];
    float position[3];
    float frustumRight;
    float frustumLeft;
    float frustumTop;
    float frustumBottom;
    float proj0;
    float proj5;
    float zNear;
    float zFar;
    float pyramidWidth;
    float pyramidHeight;
    float lodTarget;
} BlzCameraViewData;

#ifdef __cplusplus
} /* extern "C" */
#define BLZ_STATIC_ASSERT(c, m) static_assert(c, m)
#else
#define BLZ_STATIC_ASSERT(c, m) _Static_assert(c, m)
#endif

BLZ_STATIC_ASSERT(sizeof(BlzRenderObject) == 8, "RenderObject is 8 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzMeshTransform) == 32, "MeshTransform is 32 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzPrimitiveSurface) == 32, "PrimitiveSurface is 32 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzLodData) == 32, "LodData is 32 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzLodInstanceCounter) == 8, "LodInstanceCounter is 8 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzCluster) == 32, "Cluster is 32 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzIndirectDraw) == 24, "IndirectDrawData is 24 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzDrawCmd) == 32, "IndirectDrawCmd is 32 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzClusterDispatchData) == 12, "ClusterDispatchData is 12 bytes");
BLZ_STATIC_ASSERT(sizeof(BlzCameraViewData) == 256, "CameraViewData is 256 bytes");

#endif /* BLZ_TYPES_H */
