// ref_glsl_runner.cpp — TEST INFRASTRUCTURE. Runs the reference's own Vulkan cull, depth-pyramid
// and cluster compute shaders on the CPU.
//
// oracle/ref_build.py copies nothing into the repository: it reads the GLSL from the reference tree,
// rewrites what only a GLSL compiler understands (layout-qualified buffer, uniform and push-constant
// blocks become structs, unsized arrays pointers, anonymous blocks plain globals, `out` parameters
// references, multi-component swizzles calls, #version/#extension lines and local-size layouts are
// dropped) into the git-ignored oracle/_ref/glsl/, and compiles this runner against those files and
// glsl_shim.h. Each shader lands in its own namespace with its own bindings; the runner binds the
// buffers and calls main() serially over the dispatch the reference host code issues
// (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:107-226 for the culls, 554-622 for the pyramid,
// 318-423 and 874-905 for the cluster path).
#include "glsl_shim.h"

#include "../../include/blz_cull.h"

uvec3 gl_GlobalInvocationID;

namespace vk_transparent {
#include "VulkanShaders/TransparentDrawCull.comp.glsl"
}
#undef COMPUTE_PIPELINE
#undef CULL
#undef LOD_ENABLED
#undef OCCLUSION_ENABLED
namespace vk_initial {
#include "VulkanShaders/InitialDrawCull.comp.glsl"
}
#undef COMPUTE_PIPELINE
#undef CULL
#undef LOD_ENABLED
#undef OCCLUSION_ENABLED
namespace vk_late {
#include "VulkanShaders/LateDrawCull.comp.glsl"
}
#undef COMPUTE_PIPELINE
#undef CULL
#undef LOD_ENABLED
#undef OCCLUSION_ENABLED
namespace vk_pyramid {
#include "VulkanShaders/DepthPyramidGeneration.comp.glsl"
}
namespace vk_precluster {
#include "VulkanShaders/PreClusterDrawCull.comp.glsl"
}
#undef COMPUTE_PIPELINE
#undef CLUSTER_CULLING
#undef PRE_CLUSTER
#undef LOD_ENABLED
#undef OCCLUSION_ENABLED
namespace vk_cluster {
#include "VulkanShaders/InitialClusterCull.comp.glsl"
}

static_assert(sizeof(vk_late::Transform) == sizeof(BlzMeshTransform), "Transform layout");
static_assert(sizeof(vk_late::Surface) == sizeof(BlzPrimitiveSurface), "Surface layout");
static_assert(sizeof(vk_late::Lod) == sizeof(BlzLodData), "Lod layout");
static_assert(sizeof(vk_late::RenderObject) == sizeof(BlzRenderObject), "RenderObject layout");
static_assert(sizeof(vk_late::IndirectDraw) == sizeof(BlzIndirectDraw), "IndirectDraw layout");
static_assert(sizeof(vk_cluster::Cluster) == sizeof(BlzCluster), "Cluster layout");
static_assert(sizeof(vk_cluster::ClusterDispatchData) == sizeof(BlzClusterDispatchData), "dispatch layout");
static_assert(sizeof(vk_late::ViewData) <= sizeof(BlzCameraViewData), "ViewData layout");

namespace {

sampler2D chain_of(const BlzPyramid* p) {
    sampler2D s;
    if (!p) return s;
    s.data = p->data;
    s.width = p->width;
    s.height = p->height;
    s.levels = p->mipCount;
    for (int i = 0; i < 16; ++i) s.offset[i] = p->mipOffset[i];
    return s;
}

// The uniform ViewData block (ShaderBuffers.glsl:173-196) has the members of CameraViewData in the
// same order: the first sizeof(ViewData) bytes are copied as they are.
#define BIND_VIEW(NS, V) memcpy(&NS::viewData, (V), sizeof NS::viewData)

#define BIND_SCENE(NS, S, OBJS, N)                                                                     \
    do {                                                                                               \
        NS::pushConstant.renderObjectBuffer.objects = (NS::RenderObject*)(OBJS);                      \
        NS::pushConstant.drawCount = (N);                                                              \
        NS::transformBuffer.instances = (NS::Transform*)(S)->transforms;                              \
        NS::surfaceBuffer.surfaces = (NS::Surface*)(S)->surfaces;                                     \
        NS::lodBuffer.levels = (NS::Lod*)(S)->lods;                                                    \
        NS::clusterBuffer.clusters = (NS::Cluster*)(S)->clusters;                                      \
    } while (0)

#define DISPATCH_1D(NS, N, THREADS)                                                  \
    do {                                                                             \
        const uint32_t groups = group_count((N), (THREADS));                         \
        for (uint32_t g = 0; g < groups; ++g)                                        \
            for (uint32_t t = 0; t < (THREADS); ++t) {                               \
                gl_GlobalInvocationID = uvec3{g * (THREADS) + t, 0u, 0u};            \
                NS::main();                                                          \
            }                                                                        \
    } while (0)

}  // namespace

extern "C" {

// kind 0 TransparentDrawCull (frustum + LOD), 1 InitialDrawCull (pass 1), 2 LateDrawCull (pass 2,
// pyramid = a Vulkan-form chain). Commands are Vulkan IndirectDraw records (24 bytes); the caller
// sizes them for n records. Returns the draw count after the pass.
uint32_t ref_glsl_cull(int kind, const BlzCameraViewData* v, const BlzSceneDesc* s, const BlzRenderObject* objs,
                       uint32_t n, uint32_t* vis, const BlzPyramid* pyr, BlzIndirectDraw* cmds)
{
    switch (kind) {
        case 0:
            BIND_VIEW(vk_transparent, v);
            BIND_SCENE(vk_transparent, s, objs, n);
            vk_transparent::indirectDrawBuffer.draws = (vk_transparent::IndirectDraw*)cmds;
            vk_transparent::indirectDrawCountBuffer.drawCount = 0;
            DISPATCH_1D(vk_transparent, n, 64u);
            return vk_transparent::indirectDrawCountBuffer.drawCount;
        case 1:
            BIND_VIEW(vk_initial, v);
            BIND_SCENE(vk_initial, s, objs, n);
            vk_initial::indirectDrawBuffer.draws = (vk_initial::IndirectDraw*)cmds;
            vk_initial::indirectDrawCountBuffer.drawCount = 0;
            vk_initial::visibilityBuffer.visibilities = vis;
            DISPATCH_1D(vk_initial, n, 64u);
            return vk_initial::indirectDrawCountBuffer.drawCount;
        case 2:
            BIND_VIEW(vk_late, v);
            BIND_SCENE(vk_late, s, objs, n);
            vk_late::indirectDrawBuffer.draws = (vk_late::IndirectDraw*)cmds;
            vk_late::indirectDrawCountBuffer.drawCount = 0;
            vk_late::visibilityBuffer.visibilities = vis;
            vk_late::depthPyramid = chain_of(pyr);
            DISPATCH_1D(vk_late, n, 64u);
            return vk_late::indirectDrawCountBuffer.drawCount;
        default:
            return 0;
    }
}

// GenerateDepthPyramid (vulkanDraw.cpp:554-622): level i samples the depth buffer (i = 0) or level
// i - 1 with the MIN sampler at (pos + 0.5) / levelExtent, over (w / 32 + 1) x (h / 32 + 1) groups
// of 32 x 32. pyr describes the Vulkan-form chain (extent PreviousPow2 of the depth's) and holds the
// output storage.
void ref_glsl_pyramid(const float* depth, uint32_t dw, uint32_t dh, const BlzPyramid* pyr)
{
    for (uint32_t i = 0; i < pyr->mipCount; ++i) {
        sampler2D in;
        if (i == 0) {
            in.data = depth;
            in.width = dw;
            in.height = dh;
        } else {
            in.data = pyr->data + pyr->mipOffset[i - 1];
            in.width = level_dim(pyr->width, i - 1);
            in.height = level_dim(pyr->height, i - 1);
        }
        in.levels = 1;
        const uint32_t lw = level_dim(pyr->width, i), lh = level_dim(pyr->height, i);
        vk_pyramid::inImage = in;
        vk_pyramid::outImage.data = pyr->data + pyr->mipOffset[i];
        vk_pyramid::outImage.width = lw;
        vk_pyramid::outImage.height = lh;
        vk_pyramid::imageSize = vec2((float)lw, (float)lh);
        const uint32_t gx = lw / 32 + 1, gy = lh / 32 + 1;
        for (uint32_t by = 0; by < gy; ++by)
            for (uint32_t bx = 0; bx < gx; ++bx)
                for (uint32_t ty = 0; ty < 32; ++ty)
                    for (uint32_t tx = 0; tx < 32; ++tx) {
                        gl_GlobalInvocationID = uvec3{bx * 32 + tx, by * 32 + ty, 0u};
                        vk_pyramid::main();
                    }
    }
}

// The cluster path (vulkanDraw.cpp:318-423, 874-905): PreClusterDrawCull expands every object that
// passes the frustum into the clusters of its LOD (dispatch entries, `dispatch` holds room for all),
// the host reads the entry count back, and InitialClusterCull turns each entry into an IndirectDraw
// record. Returns the draw count; *entries gets the number of dispatch entries.
uint32_t ref_glsl_clusters(const BlzCameraViewData* v, const BlzSceneDesc* s, const BlzRenderObject* objs, uint32_t n,
                           BlzClusterDispatchData* dispatch, uint32_t* entries, BlzIndirectDraw* cmds)
{
    BIND_VIEW(vk_precluster, v);
    BIND_SCENE(vk_precluster, s, objs, n);
    vk_precluster::pushConstant.clusterDispatchBuffer.data = (vk_precluster::ClusterDispatchData*)dispatch;
    vk_precluster::pushConstant.clusterCountBuffer.count = 0;
    DISPATCH_1D(vk_precluster, n, 64u);
    const uint32_t count = vk_precluster::pushConstant.clusterCountBuffer.count;
    *entries = count;

    BIND_VIEW(vk_cluster, v);
    BIND_SCENE(vk_cluster, s, objs, count);
    vk_cluster::pushConstant.clusterDispatchBuffer.data = (vk_cluster::ClusterDispatchData*)dispatch;
    vk_cluster::indirectDrawBuffer.draws = (vk_cluster::IndirectDraw*)cmds;
    vk_cluster::indirectDrawCountBuffer.drawCount = 0;
    DISPATCH_1D(vk_cluster, count, 64u);
    return vk_cluster::indirectDrawCountBuffer.drawCount;
}

}  // extern "C"
