// ref_hlsl_runner.cpp — TEST INFRASTRUCTURE. Runs the reference's own D3D12 cull shaders on the CPU.
//
// oracle/ref_build.py copies nothing into the repository: it reads the shaders from the reference
// tree, strips what only the D3D compiler understands (register bindings, system-value semantics,
// [numthreads], cbuffer wrappers, `out` parameters) into the git-ignored oracle/_ref/hlsl/, and
// compiles this runner against those files and hlsl_shim.h. Each shader lands in its own namespace
// with its own resource bindings; the runner binds buffers and dispatches csMain serially over the
// dispatch the reference host code issues (src/Renderer/BlitzenDX12/dx12Draw.cpp:114-415).
#include "hlsl_shim.h"

#include "../../include/blz_cull.h"

namespace cs_drawCull {
#include "CS/drawCull.cs.hlsl"
}
namespace cs_drawOccFirst {
#include "CS/drawOccFirst.cs.hlsl"
}
#undef DRAW_CULL_OCCLUSION
namespace cs_drawOccLate {
#include "CS/drawOccLate.cs.hlsl"
}
#undef DRAW_CULL_OCCLUSION
#undef HI_Z_MAP_DRAW_OCCLUSION
namespace cs_drawOccTemporal {
#include "CS/drawOccTemporal.hlsl"
}
#undef DRAW_OCCLUSION_TEMPORAL
#undef HI_Z_MAP_DRAW_OCCLUSION
namespace cs_drawCountReset {
#include "CS/drawCountReset.cs.hlsl"
}
namespace cs_drawInstCountReset {
#include "CS/drawInstCountReset.cs.hlsl"
}
#undef DRAW_INSTANCING
namespace cs_drawInstCull {
#include "CS/drawInstCull.cs.hlsl"
}
#undef DRAW_INSTANCING
namespace cs_drawInstCmd {
#include "CS/drawInstCmd.cs.hlsl"
}
#undef DRAW_INSTANCING
namespace cs_depthPyramid {
#include "CS/depthPyramid.cs.hlsl"
}
#undef DRAW_CULL_OCCLUSION
#undef DRAW_CULL_OCCLUSION_LATE

namespace {

MipChain chain_of(const BlzPyramid* p) {
    MipChain c;
    if (!p) return c;
    c.data = p->data;
    c.width = p->width;
    c.height = p->height;
    c.mips = p->mipCount;
    for (int i = 0; i < 16; ++i) c.offset[i] = p->mipOffset[i];
    return c;
}

// cbuffer ViewData (sharedBuffers.hlsl:40-61) members, one namespace at a time.
#define BIND_VIEW(NS, V)                                                           \
    do {                                                                           \
        memcpy(NS::viewMatrix.m, (V)->viewMatrix, 64);                             \
        memcpy(NS::projectionView.m, (V)->projectionViewMatrix, 64);               \
        NS::position = float3((V)->position[0], (V)->position[1], (V)->position[2]); \
        NS::frustumRight = (V)->frustumRight;                                      \
        NS::frustumLeft = (V)->frustumLeft;                                        \
        NS::frustumTop = (V)->frustumTop;                                          \
        NS::frustumBottom = (V)->frustumBottom;                                    \
        NS::proj0 = (V)->proj0;                                                    \
        NS::proj5 = (V)->proj5;                                                    \
        NS::zNear = (V)->zNear;                                                    \
        NS::zFar = (V)->zFar;                                                      \
        NS::pyramidWidth = (V)->pyramidWidth;                                      \
        NS::pyramidHeight = (V)->pyramidHeight;                                    \
        NS::lodTarget = (V)->lodTarget;                                            \
    } while (0)

#define BIND_SCENE(NS, S, OBJS, N)                                   \
    do {                                                             \
        NS::ssbo_Renders.bind(OBJS, N);                              \
        NS::ssbo_Surfaces.bind((S)->surfaces, (S)->surfaceCount);    \
        NS::ssbo_Transforms.bind((S)->transforms, (S)->transformCount); \
        NS::ssbo_LODs.bind((S)->lods, (S)->lodCount);                \
    } while (0)

#define DISPATCH_1D(NS, N, THREADS)                                           \
    do {                                                                      \
        const uint32_t groups = group_count(N, THREADS);                      \
        for (uint32_t g = 0; g < groups; ++g)                                 \
            for (uint32_t t = 0; t < (THREADS); ++t)                          \
                NS::csMain(uint3(uint(g * (THREADS) + t), uint(0), uint(0)), uint3(uint(g), uint(0), uint(0))); \
    } while (0)

// Shaders whose csMain takes only SV_DispatchThreadID.
#define DISPATCH_1D_TID(NS, N, THREADS)                                       \
    do {                                                                      \
        const uint32_t groups = group_count(N, THREADS);                      \
        for (uint32_t g = 0; g < groups; ++g)                                 \
            for (uint32_t t = 0; t < (THREADS); ++t)                          \
                NS::csMain(uint3(uint(g * (THREADS) + t), uint(0), uint(0))); \
    } while (0)

}  // namespace

extern "C" {

// kind 0 drawCull, 1 drawOccFirst, 2 drawOccLate, 3 drawOccTemporal. Commands are D3D12 DrawCmd
// records (32 bytes). Returns the draw counter after the pass.
uint32_t ref_hlsl_cull(int kind, const BlzCameraViewData* v, const BlzSceneDesc* s, const BlzRenderObject* objs,
                       uint32_t n, uint32_t* vis, const BlzPyramid* pyr, BlzDrawCmd* cmds, uint32_t capacity)
{
    uint32_t counter = 0;
    switch (kind) {
        case 0:
            BIND_VIEW(cs_drawCull, v);
            BIND_SCENE(cs_drawCull, s, objs, n);
            cs_drawCull::ssbo_DrawCmd.bind(cmds, capacity);
            cs_drawCull::rwb_DrawCmdCounter.bind(&counter, 1);
            cs_drawCull::objCount = n;
            DISPATCH_1D(cs_drawCull, n, 64);
            break;
        case 1:
            BIND_VIEW(cs_drawOccFirst, v);
            BIND_SCENE(cs_drawOccFirst, s, objs, n);
            cs_drawOccFirst::ssbo_DrawCmd.bind(cmds, capacity);
            cs_drawOccFirst::rwb_DrawCmdCounter.bind(&counter, 1);
            cs_drawOccFirst::rwssbo_DrawVisibilityBuffer.bind(vis, n);
            cs_drawOccFirst::objCount = n;
            DISPATCH_1D(cs_drawOccFirst, n, 64);
            break;
        case 2:
            BIND_VIEW(cs_drawOccLate, v);
            BIND_SCENE(cs_drawOccLate, s, objs, n);
            cs_drawOccLate::ssbo_DrawCmd.bind(cmds, capacity);
            cs_drawOccLate::rwb_DrawCmdCounter.bind(&counter, 1);
            cs_drawOccLate::rwssbo_DrawVisibilityBuffer.bind(vis, n);
            cs_drawOccLate::tex_HiZMap.c = chain_of(pyr);
            cs_drawOccLate::objCount = n;
            DISPATCH_1D(cs_drawOccLate, n, 64);
            break;
        case 3:
            BIND_VIEW(cs_drawOccTemporal, v);
            BIND_SCENE(cs_drawOccTemporal, s, objs, n);
            cs_drawOccTemporal::ssbo_DrawCmd.bind(cmds, capacity);
            cs_drawOccTemporal::rwb_DrawCmdCounter.bind(&counter, 1);
            cs_drawOccTemporal::tex_HiZMap.c = chain_of(pyr);
            cs_drawOccTemporal::objCount = n;
            DISPATCH_1D(cs_drawOccTemporal, n, 64);
            break;
        default:
            return 0xFFFFFFFFu;
    }
    return counter;
}

// DrawInstanceCullPass (dx12Draw.cpp:340-415): count reset, per-LOD counter reset, instance cull,
// command generation. counters has s->lodCount entries. Returns the draw counter.
uint32_t ref_hlsl_instanced(const BlzCameraViewData* v, const BlzSceneDesc* s, const BlzRenderObject* objs, uint32_t n,
                            BlzLodInstanceCounter* counters, uint32_t* instances, uint32_t instanceCapacity,
                            BlzDrawCmd* cmds, uint32_t capacity)
{
    uint32_t counter = 12345u;
    cs_drawCountReset::rwb_drawCmdCounter.bind(&counter, 1);
    cs_drawCountReset::csMain(uint3(uint(0), uint(0), uint(0)));

    const uint32_t nl = s->lodCount;
    cs_drawInstCountReset::rwssbo_InstCounter.bind(counters, nl);
    cs_drawInstCountReset::lodCount = nl;
    DISPATCH_1D_TID(cs_drawInstCountReset, nl, 64);

    BIND_VIEW(cs_drawInstCull, v);
    BIND_SCENE(cs_drawInstCull, s, objs, n);
    cs_drawInstCull::rwssbo_InstCounter.bind(counters, nl);
    cs_drawInstCull::rwssbo_instIndices.bind(instances, instanceCapacity);
    cs_drawInstCull::objCount = n;
    DISPATCH_1D(cs_drawInstCull, n, 64);

    cs_drawInstCmd::rwssbo_InstCounter.bind(counters, nl);
    cs_drawInstCmd::ssbo_LODs.bind(s->lods, nl);
    cs_drawInstCmd::ssbo_DrawCmd.bind(cmds, capacity);
    cs_drawInstCmd::rwb_DrawCmdCounter.bind(&counter, 1);
    cs_drawInstCmd::lodCount = nl;
    DISPATCH_1D_TID(cs_drawInstCmd, nl, 64);
    return counter;
}

// GenerateDepthPyramid (dx12Draw.cpp:248-277) over depthPyramid.cs.hlsl: level 0 reads the depth
// target, level i reads the pyramid at the mip the root constant names, which the loop sets before
// it advances (so level i reads mip i - 1).
void ref_hlsl_pyramid(const float* depth, uint32_t W, uint32_t H, const BlzPyramid* p)
{
    uint32_t mipLevel = 0;
    for (uint32_t i = 0; i < p->mipCount; ++i) {
        uint32_t levelWidth = p->width >> i, levelHeight = p->height >> i;
        levelWidth = levelWidth ? levelWidth : 1u;
        levelHeight = levelHeight ? levelHeight : 1u;
        cs_depthPyramid::mipLevel = mipLevel;
        if (i == 0) {
            MipChain c;
            c.data = depth;
            c.width = W;
            c.height = H;
            c.mips = 1;
            cs_depthPyramid::tex_depthIn.c = c;
        } else {
            cs_depthPyramid::tex_depthIn.c = chain_of(p);
            mipLevel++;
        }
        cs_depthPyramid::rwtex_depthOut.data = p->data + p->mipOffset[i];
        cs_depthPyramid::rwtex_depthOut.width = levelWidth;
        cs_depthPyramid::rwtex_depthOut.height = levelHeight;
        const uint32_t gx = group_count(levelWidth, 32), gy = group_count(levelHeight, 32);
        for (uint32_t by = 0; by < gy; ++by)
            for (uint32_t bx = 0; bx < gx; ++bx)
                for (uint32_t ty = 0; ty < 32; ++ty)
                    for (uint32_t tx = 0; tx < 32; ++tx)
                        cs_depthPyramid::csMain(uint3(uint(bx * 32 + tx), uint(by * 32 + ty), uint(0)));
    }
}

}  // extern "C"
