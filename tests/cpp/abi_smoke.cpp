// abi_smoke.cpp — the C ABI driven from C++ with no Python in the process: a renderer-side caller
// (as the reference's Vulkan/D3D12 renderer would be) builds a small scene in the reference
// layouts, uploads it, sets up the camera, runs the frustum + LOD cull and the two occlusion passes
// on the GPU, reads the draw counts and records back and prints a line of checksums that the test
// compares with the same calls made through ctypes.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "blz_cull.h"

#define CHECK(x)                                                          \
    do {                                                                  \
        int rc_ = (x);                                                    \
        if (rc_ != BLZ_OK) {                                              \
            std::fprintf(stderr, "%s: %d %s\n", #x, rc_, blz_last_error()); \
            return 1;                                                     \
        }                                                                 \
    } while (0)

static uint32_t lcg(uint32_t& s) { return s = s * 1664525u + 1013904223u; }
static float unit(uint32_t& s) { return (lcg(s) >> 8) * (1.0f / 16777216.0f); }

static uint64_t fnv(const void* p, size_t n, uint64_t h = 1469598103934665603ull) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) h = (h ^ b[i]) * 1099511628211ull;
    return h;
}

int main() {
    const uint32_t N = 50000, M = 8, L = 4;
    std::vector<BlzRenderObject> objs(N);
    std::vector<BlzMeshTransform> tr(N);
    std::vector<BlzPrimitiveSurface> surf(M);
    std::vector<BlzLodData> lods(M * L);
    uint32_t s = 12345u;
    for (uint32_t m = 0; m < M; ++m) {
        std::memset(&surf[m], 0, sizeof surf[m]);
        surf[m].center[0] = unit(s) - 0.5f;
        surf[m].center[1] = unit(s) - 0.5f;
        surf[m].center[2] = unit(s) - 0.5f;
        surf[m].radius = 0.5f + 2.0f * unit(s);
        surf[m].lodOffset = m * L;
        surf[m].lodCount = L;
        for (uint32_t l = 0; l < L; ++l) {
            BlzLodData& d = lods[m * L + l];
            std::memset(&d, 0, sizeof d);
            d.indexCount = 30000u >> l;
            d.firstIndex = 1000u * (m * L + l);
            d.error = l == 0 ? 0.0f : 0.01f * float(1u << (2 * (l - 1)));
        }
    }
    for (uint32_t i = 0; i < N; ++i) {
        tr[i].pos[0] = 2000.0f * unit(s) - 1000.0f;
        tr[i].pos[1] = 2000.0f * unit(s) - 1000.0f;
        tr[i].pos[2] = 2000.0f * unit(s) - 1000.0f;
        tr[i].scale = 0.5f + 1.5f * unit(s);
        tr[i].orientation[0] = 0.0f;
        tr[i].orientation[1] = 0.0f;
        tr[i].orientation[2] = 0.0f;
        tr[i].orientation[3] = 1.0f;
        objs[i].transformId = i;
        objs[i].surfaceId = lcg(s) % M;
    }

    blz_ctx* ctx = nullptr;
    CHECK(blz_ctx_create(0, &ctx));
    BlzSceneDesc desc{};
    desc.renderObjects = objs.data();
    desc.renderObjectCount = N;
    desc.transforms = tr.data();
    desc.transformCount = N;
    desc.surfaces = surf.data();
    desc.surfaceCount = M;
    desc.lods = lods.data();
    desc.lodCount = M * L;
    CHECK(blz_scene_upload(ctx, &desc, BLZ_SCENE_COPY_FROM_HOST, nullptr));

    BlzCameraViewData view;
    const float pos[3] = {0.0f, 0.0f, 0.0f};
    CHECK(blz_view_setup(&view, 1.2217305f, 1920.0f, 1080.0f, 0.1f, 1e4f, pos, 0.3f, 0.1f, 960.0f, 540.0f));

    // frustum + LOD
    void* cmds = nullptr;
    uint32_t* count = nullptr;
    if (cudaMalloc(&cmds, size_t(N) * BLZ_STRIDE_VULKAN) != cudaSuccess || cudaMalloc(&count, 4) != cudaSuccess) return 2;
    BlzCullTarget t{cmds, BLZ_STRIDE_VULKAN, N, count};
    BlzRenderList all{nullptr, 0};
    CHECK(blz_cull_frustum(ctx, &view, all, &t, nullptr));
    uint32_t flags = 0;
    CHECK(blz_ctx_check(ctx, nullptr, &flags));
    uint32_t n = 0;
    cudaMemcpy(&n, count, 4, cudaMemcpyDeviceToHost);
    std::vector<uint32_t> recs(size_t(n) * 6);
    cudaMemcpy(recs.data(), cmds, recs.size() * 4, cudaMemcpyDeviceToHost);
    const uint64_t hFrustum = fnv(recs.data(), recs.size() * 4);

    // pass 1 with every other object visible last frame, a flat depth, the pyramid, pass 2
    std::vector<uint32_t> visHost(N);
    for (uint32_t i = 0; i < N; ++i) visHost[i] = i & 1u;
    uint32_t* vis = nullptr;
    float* depth = nullptr;
    BlzPyramid pyr{};
    const uint64_t pyrBytes = blz_pyramid_layout(1920, 1080, BLZ_HIZ_D3D12, &pyr);
    if (cudaMalloc(&vis, size_t(N) * 4) != cudaSuccess || cudaMalloc(&depth, 1920ull * 1080 * 4) != cudaSuccess ||
        cudaMalloc(&pyr.data, pyrBytes) != cudaSuccess)
        return 2;
    cudaMemcpy(vis, visHost.data(), size_t(N) * 4, cudaMemcpyHostToDevice);
    std::vector<float> depthHost(1920ull * 1080, 0.0f);
    for (size_t i = 0; i < depthHost.size(); ++i) depthHost[i] = (i % 1920) < 960 ? 0.001f : 0.0f;  // left half occluding
    cudaMemcpy(depth, depthHost.data(), depthHost.size() * 4, cudaMemcpyHostToDevice);
    CHECK(blz_cull_first(ctx, &view, all, vis, &t, nullptr));
    CHECK(blz_ctx_check(ctx, nullptr, &flags));
    uint32_t n1 = 0;
    cudaMemcpy(&n1, count, 4, cudaMemcpyDeviceToHost);
    CHECK(blz_pyramid_build(ctx, &pyr, depth, nullptr));
    CHECK(blz_cull_late(ctx, &view, all, vis, &pyr, &t, nullptr));
    CHECK(blz_ctx_check(ctx, nullptr, &flags));
    uint32_t n2 = 0;
    cudaMemcpy(&n2, count, 4, cudaMemcpyDeviceToHost);
    std::vector<uint32_t> recs2(size_t(n2) * 6);
    cudaMemcpy(recs2.data(), cmds, recs2.size() * 4, cudaMemcpyDeviceToHost);
    cudaMemcpy(visHost.data(), vis, size_t(N) * 4, cudaMemcpyDeviceToHost);
    const uint64_t hLate = fnv(recs2.data(), recs2.size() * 4);
    const uint64_t hVis = fnv(visHost.data(), visHost.size() * 4);

    // the first 4,096 transforms moved 150 units along x, bound from pinned host memory
    const uint32_t K = 4096;
    BlzMeshTransform* rows = nullptr;
    if (cudaHostAlloc(reinterpret_cast<void**>(&rows), K * sizeof(BlzMeshTransform), cudaHostAllocDefault) != cudaSuccess) return 2;
    for (uint32_t i = 0; i < K; ++i) {
        rows[i] = tr[i];
        rows[i].pos[0] = tr[i].pos[0] + 150.0f;
    }
    CHECK(blz_scene_bind_dynamic(ctx, rows, K));
    CHECK(blz_cull_frustum(ctx, &view, all, &t, nullptr));
    CHECK(blz_ctx_check(ctx, nullptr, &flags));
    CHECK(blz_scene_bind_dynamic(ctx, nullptr, 0));
    uint32_t nb = 0;
    cudaMemcpy(&nb, count, 4, cudaMemcpyDeviceToHost);
    std::vector<uint32_t> recsB(size_t(nb) * 6);
    cudaMemcpy(recsB.data(), cmds, recsB.size() * 4, cudaMemcpyDeviceToHost);
    const uint64_t hBound = fnv(recsB.data(), recsB.size() * 4);
    cudaFreeHost(rows);

    std::printf("frustum %u %016llx first %u late %u %016llx vis %016llx bound %u %016llx\n", n,
                (unsigned long long)hFrustum, n1, n2, (unsigned long long)hLate, (unsigned long long)hVis, nb,
                (unsigned long long)hBound);
    cudaFree(cmds);
    cudaFree(count);
    cudaFree(vis);
    cudaFree(depth);
    cudaFree(pyr.data);
    blz_ctx_destroy(ctx);
    return 0;
}
