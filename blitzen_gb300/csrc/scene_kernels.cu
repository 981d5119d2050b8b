// scene_kernels.cu — scene-side kernels around the cull: transform scatter (UpdateObjectTransform),
// dynamic-object rotation, and the occluder-box depth rasteriser that produces the per-view depth
// buffers the pyramid is built from.
#include "blz_device.cuh"
#include "kernels.h"

namespace blz {

// transforms[ids[i]] = in[i]: the device half of UpdateObjectTransform + UpdateBuffers
// (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:46-60,816-820).
__global__ void transforms_scatter_kernel(BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                                          const BlzMeshTransform* in, uint32_t n, unsigned int* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = ids[i];
    if (id >= tableCount) {
        atomicOr(status, BLZ_FLAG_BAD_INDEX);
        return;
    }
    const float4* src = reinterpret_cast<const float4*>(in + i);
    float4* dst = reinterpret_cast<float4*>(table + id);
    dst[0] = src[0];
    dst[1] = src[1];
}

// dst[i] = table[ids[i]] with orientation r (x) q, r = (s * axis_i, c); the rotation of
// src/Game/blitzenObject.cpp:30-46 applied incrementally on the device. s, c = sin/cos(angle/2)
// are computed once on the host.
__global__ void transforms_rotate_kernel(const BlzMeshTransform* table, uint32_t tableCount, const BlzMeshTransform* dynRows,
                                         uint32_t dynCount, const uint32_t* ids, const float* axes, float s, float c,
                                         uint32_t n, BlzMeshTransform* dst, unsigned int* status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = ids[i];
    if (id >= tableCount) {
        atomicOr(status, BLZ_FLAG_BAD_INDEX);
        return;
    }
    const float4* src = reinterpret_cast<const float4*>((id < dynCount ? dynRows : table) + id);
    const float4 ps = src[0], q = src[1];
    const float rx = BLZ_FM(s, axes[3 * i + 0]), ry = BLZ_FM(s, axes[3 * i + 1]), rz = BLZ_FM(s, axes[3 * i + 2]);
    const float rw = c;
    float4 o;
    o.x = BLZ_FS(BLZ_FA(BLZ_FA(BLZ_FM(rw, q.x), BLZ_FM(rx, q.w)), BLZ_FM(ry, q.z)), BLZ_FM(rz, q.y));
    o.y = BLZ_FA(BLZ_FA(BLZ_FS(BLZ_FM(rw, q.y), BLZ_FM(rx, q.z)), BLZ_FM(ry, q.w)), BLZ_FM(rz, q.x));
    o.z = BLZ_FA(BLZ_FS(BLZ_FA(BLZ_FM(rw, q.z), BLZ_FM(rx, q.y)), BLZ_FM(ry, q.x)), BLZ_FM(rz, q.w));
    o.w = BLZ_FS(BLZ_FS(BLZ_FS(BLZ_FM(rw, q.w), BLZ_FM(rx, q.x)), BLZ_FM(ry, q.y)), BLZ_FM(rz, q.z));
    float4* d = reinterpret_cast<float4*>(dst + i);
    d[0] = ps;
    d[1] = o;
}

cudaError_t launch_transforms_scatter(BlzMeshTransform* table, uint32_t tableCount, const uint32_t* ids,
                                      const BlzMeshTransform* in, uint32_t n, unsigned int* status, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    transforms_scatter_kernel<<<(n + 255) / 256, 256, 0, s>>>(table, tableCount, ids, in, n, status);
    return cudaGetLastError();
}

cudaError_t launch_transforms_rotate(const BlzMeshTransform* table, uint32_t tableCount, const BlzMeshTransform* dynRows,
                                     uint32_t dynCount, const uint32_t* ids, const float* axes, float angle, uint32_t n,
                                     BlzMeshTransform* dst, unsigned int* status, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const float h = angle * 0.5f;
    const float sn = sinf(h), cs = cosf(h);  // host libm, the same values the host oracle uses
    transforms_rotate_kernel<<<(n + 255) / 256, 256, 0, s>>>(table, tableCount, dynRows, dynCount, ids, axes, sn, cs, n,
                                                               dst, status);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ occluder raster

struct BoxRect {
    int x0, y0, x1, y1;
    float depth;
};

__device__ __forceinline__ BoxRect box_rect(const ViewConsts& v, const float* bx, uint32_t width, uint32_t height) {
    BoxRect r{0, 0, 0, 0, 0.0f};
    const float fw = static_cast<float>(width), fh = static_cast<float>(height);
    float minx = INFINITY, maxx = -INFINITY, miny = INFINITY, maxy = -INFINITY, zmax = -INFINITY;
    for (int k = 0; k < 8; ++k) {
        const Vec3 p{bx[(k & 1) ? 3 : 0], bx[(k & 2) ? 4 : 1], bx[(k & 4) ? 5 : 2]};
        const Vec3 q = view_transform(v.rows, p);
        if (!(q.z > v.zNear)) return r;  // boxes reaching the near plane are skipped
        const float sx = BLZ_FM(BLZ_FA(BLZ_FM(BLZ_FD(BLZ_FM(q.x, v.proj0), q.z), 0.5f), 0.5f), fw);
        const float sy = BLZ_FM(BLZ_FS(0.5f, BLZ_FM(BLZ_FD(BLZ_FM(q.y, v.proj5), q.z), 0.5f)), fh);
        minx = fmin_nan(minx, sx);
        maxx = fmax_nan(maxx, sx);
        miny = fmin_nan(miny, sy);
        maxy = fmax_nan(maxy, sy);
        zmax = fmax_nan(zmax, q.z);
    }
    r.depth = BLZ_FD(v.zNear, zmax);
    const float fx0 = floorf(minx), fy0 = floorf(miny), fx1 = ceilf(maxx), fy1 = ceilf(maxy);
    r.x0 = fx0 < 0.0f ? 0 : (fx0 > fw ? static_cast<int>(width) : static_cast<int>(fx0));
    r.y0 = fy0 < 0.0f ? 0 : (fy0 > fh ? static_cast<int>(height) : static_cast<int>(fy0));
    r.x1 = fx1 < 0.0f ? 0 : (fx1 > fw ? static_cast<int>(width) : static_cast<int>(fx1));
    r.y1 = fy1 < 0.0f ? 0 : (fy1 > fh ? static_cast<int>(height) : static_cast<int>(fy1));
    return r;
}

__global__ void depth_clear_kernel(float4* depth, size_t n4, float* tail, uint32_t ntail) {
    for (size_t i = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; i < n4; i += static_cast<size_t>(gridDim.x) * blockDim.x)
        depth[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    if (blockIdx.x == 0 && threadIdx.x < ntail) tail[threadIdx.x] = 0.0f;
}

// One block per box: the block walks the box's screen rectangle and max-writes its depth.
// Depths are positive, so the float maximum is the integer maximum of the bit patterns, which
// makes the result independent of the order boxes land in.
__global__ void depth_raster_kernel(const BlzCameraViewData view, const float* boxes, uint32_t boxCount, float* depth,
                                    uint32_t width, uint32_t height) {
    __shared__ BoxRect s_r;
    const ViewConsts v = load_view(view);
    for (uint32_t b = blockIdx.x; b < boxCount; b += gridDim.x) {
        if (threadIdx.x == 0) s_r = box_rect(v, boxes + 6 * static_cast<size_t>(b), width, height);
        __syncthreads();
        const BoxRect r = s_r;
        if (r.x1 > r.x0 && r.y1 > r.y0 && r.depth > 0.0f) {
            const int w = r.x1 - r.x0;
            const int n = w * (r.y1 - r.y0);
            const int bits = __float_as_int(r.depth);
            for (int idx = threadIdx.x; idx < n; idx += blockDim.x) {
                const int x = r.x0 + idx % w, y = r.y0 + idx / w;
                atomicMax(reinterpret_cast<int*>(depth) + static_cast<size_t>(y) * width + x, bits);
            }
        }
        __syncthreads();
    }
}

cudaError_t launch_depth_raster(const BlzCameraViewData& view, const float* boxes, uint32_t boxCount, float* depth,
                                uint32_t width, uint32_t height, cudaStream_t s, uint32_t* launches) {
    const size_t n = static_cast<size_t>(width) * height;
    const size_t n4 = (reinterpret_cast<uintptr_t>(depth) % 16 == 0) ? n / 4 : 0;
    const uint32_t ntail = static_cast<uint32_t>(n - n4 * 4);
    if (ntail > 1024) {
        cudaError_t e = cudaMemsetAsync(depth, 0, n * sizeof(float), s);
        if (e != cudaSuccess) return e;
    } else {
        depth_clear_kernel<<<1024, 256, 0, s>>>(reinterpret_cast<float4*>(depth), n4, depth + n4 * 4, ntail);
        if (launches) *launches += 1;
    }
    if (boxCount > 0) {
        const uint32_t grid = boxCount < 4096 ? boxCount : 4096;
        depth_raster_kernel<<<grid, 256, 0, s>>>(view, boxes, boxCount, depth, width, height);
        if (launches) *launches += 1;
    }
    return cudaGetLastError();
}

}  // namespace blz

namespace blz {

__global__ void take_status_kernel(unsigned int* status, unsigned int* out) { *out = atomicExch(status, 0u); }

__global__ void add_word_kernel(unsigned int* word, unsigned int n) { atomicAdd(word, n); }

cudaError_t launch_add_word(unsigned int* word, unsigned int n, cudaStream_t s) {
    add_word_kernel<<<1, 1, 0, s>>>(word, n);
    return cudaGetLastError();
}

cudaError_t launch_take_status(unsigned int* status, unsigned int* out, cudaStream_t s) {
    take_status_kernel<<<1, 1, 0, s>>>(status, out);
    return cudaGetLastError();
}

}  // namespace blz
