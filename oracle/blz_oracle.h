/*
 * blz_oracle.h — CPU oracle for the Blitzen culling path. TEST INFRASTRUCTURE ONLY.
 *
 * A plain-C restatement of the reference's cull shaders, used by the tests to check the CUDA
 * kernels and by the benchmark's CPU-baseline leg. The product library never links or calls it.
 *
 * Pinning: the reference ships no tests, golden vectors or fixtures for this path, and its
 * shaders cannot run here (no graphics stack). The restatement is therefore pinned against the
 * reference's own HLSL shader source compiled as C++ through a small HLSL shim
 * (oracle/ref_hlsl.py builds it into oracle/_ref/ from the reference tree), and its view-constant
 * code against the reference's own camera code compiled from source (oracle/ref_camera.cpp).
 * Arithmetic the shaders leave to the GPU is fixed the same way in all three places:
 *   - every FP32 operation is one IEEE-754 round-to-nearest operation in source order; nothing
 *     is contracted into an FMA (build with -ffp-contract=off);
 *   - sqrt and division are correctly rounded;
 *   - floor(log2(x)) is exact: the unbiased exponent for finite x >= 1, 0 when x < 1 or NaN,
 *     UINT32_MAX for +inf (which lands past the last mip);
 *   - float -> uint is the D3D conversion: NaN and x <= 0 give 0, x >= 2^32 gives UINT32_MAX,
 *     else truncation;
 *   - min/max of floats ignore a NaN operand (IEEE minNum/maxNum), and min(a,b) keeps a on ties;
 *   - an out-of-range texel or mip Load returns 0 (D3D rule);
 *   - atomic arrival order is replaced by the order a serial run of the dispatch produces:
 *     ascending object index.
 */
#ifndef BLZ_ORACLE_H
#define BLZ_ORACLE_H

#include <stdint.h>
#include "../include/blz_types.h"
#include "../include/blz_cull.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Mirrors of the library modes. */
enum { BO_FRUSTUM = 0, BO_FIRST = 1, BO_LATE = 2, BO_TEMPORAL = 3 };

/* View constants: SetupCamera + UpdateProjection (src/Game/blitzenCamera.cpp:14-41,93-126). */
void bo_view_setup(BlzCameraViewData* out, float fovRadians, float windowWidth, float windowHeight,
                   float zNear, float zFar, const float position[3], float yawRadians, float pitchRadians,
                   float pyramidWidth, float pyramidHeight);

/* Pyramid layout and build (host memory in pyramid->data). */
uint64_t bo_pyramid_layout(uint32_t depthWidth, uint32_t depthHeight, uint32_t mode, BlzPyramid* out);
void bo_pyramid_build(const BlzPyramid* pyramid, const float* depth);

/* Object culls. Returns the number of visible records (uncapped); records past `capacity` are not
 * written. vis is read by FIRST, read and rewritten by LATE. *flags gets BLZ_FLAG_* bits OR-ed in.
 * threads > 1 splits the objects into contiguous ranges and concatenates results in order. */
uint32_t bo_cull(int mode, const BlzCameraViewData* view, const BlzSceneDesc* scene,
                 const BlzRenderObject* objects, uint32_t count, uint32_t* vis, const BlzPyramid* pyramid,
                 void* cmds, uint32_t stride, uint32_t capacity, uint32_t* flags, int threads);

/* Instanced cull. counters has scene->lodCount entries (instanceOffset is input, instanceCount is
 * output). Returns the number of commands. */
uint32_t bo_cull_instanced(const BlzCameraViewData* view, const BlzSceneDesc* scene,
                           const BlzRenderObject* objects, uint32_t count, BlzLodInstanceCounter* counters,
                           uint32_t* instances, uint32_t instanceCapacity, uint32_t slotsPerLod,
                           void* cmds, uint32_t stride, uint32_t capacity, uint32_t* flags, int threads);

/* Cluster cull. pyramid may be NULL (no Hi-Z). clusterIds may be NULL. */
uint32_t bo_cull_clusters(const BlzCameraViewData* view, const BlzSceneDesc* scene,
                          const BlzRenderObject* objects, uint32_t count, const BlzPyramid* pyramid,
                          void* cmds, uint32_t stride, uint32_t capacity, uint32_t* clusterIds,
                          uint32_t* flags, int threads);

/* Transform scatter (UpdateObjectTransform) and dynamic rotation. */
void bo_transforms_update(BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                          const BlzMeshTransform* in, uint32_t n, uint32_t* flags);
void bo_transforms_rotate(const BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                          const float* axes, float angle, uint32_t n, BlzMeshTransform* dst, uint32_t* flags);

/* Occluder-box depth raster (the library's blz_depth_raster_boxes semantics). */
void bo_depth_raster_boxes(const BlzCameraViewData* view, const float* boxes, uint32_t boxCount,
                           float* depth, uint32_t width, uint32_t height);

/* Scalar helpers exported for known-answer tests. */
uint32_t bo_ftou(float x);
uint32_t bo_floor_log2_u(float x);
int bo_object_test(int mode, const BlzCameraViewData* view, const BlzSceneDesc* scene,
                   BlzRenderObject obj, const BlzPyramid* pyramid, uint32_t* lodIdOut);

#ifdef __cplusplus
}
#endif
#endif
