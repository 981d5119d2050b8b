// cull_clusters.cu — object pass, cluster expansion and per-cluster culling in one launch.
//
// The reference splits this into PreClusterDrawCull.comp.glsl:13-47 (object frustum + LOD, then a
// serial loop that materialises one 12-byte ClusterDispatchData per cluster), a fence wait and CPU
// read-back of the cluster count (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:874-905), and
// InitialClusterCull.comp.glsl:12-55 (one draw per cluster, its cone test commented out). Here a
// block takes a tile of objects, decides them and prefix-sums their cluster counts in shared
// memory, then walks the tile's clusters in order (a binary search maps a cluster slot back to
// its object), testing each one: sphere frustum, Hi-Z when a pyramid is bound, and the normal cone
// in meshoptimizer's documented form (VendorCode/Meshoptimizer/meshoptimizer.h:561-569).
// Two launches, no block waiting on another: the count launch writes each tile's number of
// surviving clusters; the write launch sums the counts of the tiles before its own (a strided
// read), repeats the same tests and writes the records at their final slots. Nothing is
// materialised and the host never waits.
#include "blz_device.cuh"
#include "kernels.h"

namespace blz {

constexpr int kClThreads = 256;
constexpr int kClWarps = kClThreads / 32;
constexpr uint32_t kClObjects = 32;  // objects per tile

struct ClusterObj {
    float4 posScale;
    float4 quat;
    uint32_t objectId;
    uint32_t clusterOffset;
};

// Sphere, Hi-Z and cone tests of one cluster of an object. snorm[i] holds (float)(i - 128) / 127,
// divided once per block: the int8 cone axis and cutoff take only those 256 values.
__device__ __forceinline__ bool cluster_visible(const ClusterParams& p, const ViewConsts& v, const ClusterObj& o,
                                                uint32_t cid, const float* snorm, uint32_t& indexCount,
                                                uint32_t& dataOffset) {
    const float4* cp = reinterpret_cast<const float4*>(p.sc.clusters + cid);
    const float4 sph = __ldg(cp);
    const uint4 meta = __ldg(reinterpret_cast<const uint4*>(cp + 1));  // cone s8x4, dataOffset, counts, pad
    const Vec3 w = model_to_world(Vec3{sph.x, sph.y, sph.z}, o.posScale, o.quat);
    const Vec3 c = view_transform(v.rows, w);
    const float r = BLZ_FM(sph.w, o.posScale.w);
    bool vis = frustum_check(c, r, v);
    if (vis && p.hasPyramid) {
        float4 aabb;
        if (project_sphere(c, r, v.zNear, v.proj0, v.proj5, aabb)) vis = vis && occlusion(aabb, p.pyr, v, c, r);
    }
    if (vis) {
        const int ax = static_cast<int8_t>(meta.x & 0xFFu), ay = static_cast<int8_t>((meta.x >> 8) & 0xFFu);
        const int az = static_cast<int8_t>((meta.x >> 16) & 0xFFu), ac = static_cast<int8_t>(meta.x >> 24);
        const Vec3 axm{snorm[ax + 128], snorm[ay + 128], snorm[az + 128]};
        const float cutoff = snorm[ac + 128];
        const Vec3 axis = rotate_quat(axm, o.quat);
        const float dx = BLZ_FS(w.x, v.camX), dy = BLZ_FS(w.y, v.camY), dz = BLZ_FS(w.z, v.camZ);
        const float len = __fsqrt_rn(BLZ_FA(BLZ_FA(BLZ_FM(dx, dx), BLZ_FM(dy, dy)), BLZ_FM(dz, dz)));
        const float nx = BLZ_FD(dx, len), ny = BLZ_FD(dy, len), nz = BLZ_FD(dz, len);
        const float dp = BLZ_FA(BLZ_FA(BLZ_FM(nx, axis.x), BLZ_FM(ny, axis.y)), BLZ_FM(nz, axis.z));
        if (dp >= cutoff) vis = false;
    }
    dataOffset = meta.y;
    indexCount = ((meta.z >> 8) & 0xFFu) * 3u;  // triangleCount * 3
    return vis;
}

template <bool WRITE>
__global__ void __launch_bounds__(kClThreads) cull_clusters_kernel(const ClusterParams p, const BlzCameraViewData view) {
    __shared__ ClusterObj s_obj[kClObjects];
    __shared__ uint32_t s_start[kClObjects + 1];
    __shared__ uint32_t s_warp[kClWarps];
    __shared__ uint32_t s_base;
    __shared__ unsigned int s_flags;
    __shared__ float s_snorm[256];
    if (threadIdx.x == 0) s_flags = 0u;
    for (uint32_t i = threadIdx.x; i < 256u; i += kClThreads)
        s_snorm[i] = BLZ_FD(static_cast<float>(static_cast<int>(i) - 128), 127.0f);
    __syncthreads();
    const uint32_t tile = blockIdx.x;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const ViewConsts v = load_view(view);

    // object pass: PreClusterDrawCull.comp.glsl:20-37
    uint32_t count = 0;
    unsigned int flags = 0u;
    if (threadIdx.x < kClObjects) {
        const uint32_t i = tile * kClObjects + threadIdx.x;
        ClusterObj o;
        o.objectId = i;
        o.clusterOffset = 0;
        o.posScale = make_float4(0.f, 0.f, 0.f, 1.f);
        o.quat = make_float4(0.f, 0.f, 0.f, 1.f);
        if (i < p.count) {
            const uint2 ro = __ldg(reinterpret_cast<const uint2*>(p.objects) + i);
            bool ok = ro.x < p.sc.transformCount && ro.y < p.sc.surfaceCount;
            uint4 sm = make_uint4(0u, 0u, 0u, 0u);
            float4 sph = make_float4(0.f, 0.f, 0.f, 0.f);
            if (ok) {
                const float4* tp = reinterpret_cast<const float4*>(p.sc.transforms + ro.x);
                o.posScale = __ldg(tp);
                o.quat = __ldg(tp + 1);
                const float4* sp = reinterpret_cast<const float4*>(p.sc.surfaces + ro.y);
                sph = __ldg(sp);
                sm = __ldg(reinterpret_cast<const uint4*>(sp + 1));
                ok = sm.y < p.sc.lodCount && sm.z <= p.sc.lodCount - sm.y;
            }
            if (!ok) {
                flags |= BLZ_FLAG_BAD_INDEX;
            } else {
                const Vec3 c = view_transform(v.rows, model_to_world(Vec3{sph.x, sph.y, sph.z}, o.posScale, o.quat));
                const float r = BLZ_FM(sph.w, o.posScale.w);
                if (frustum_check(c, r, v)) {
                    const float threshold = lod_threshold(c, r, o.posScale.w, v.lodTarget);
                    uint32_t idx = 0;
                    for (uint32_t k = 1; k < sm.z; ++k)
                        if (__ldg(&p.sc.lods[sm.y + k].error) < threshold) idx = k;
                    const uint4 lod = __ldg(reinterpret_cast<const uint4*>(p.sc.lods + sm.y + idx));
                    // lod.z = clusterOffset, lod.w = clusterCount
                    if (lod.z > p.sc.clusterCount || lod.w > p.sc.clusterCount - lod.z) {
                        flags |= BLZ_FLAG_BAD_INDEX;
                    } else {
                        o.clusterOffset = lod.z;
                        count = lod.w;
                    }
                }
            }
        }
        s_obj[threadIdx.x] = o;
    }
    if (flags) atomicOr(&s_flags, flags);
    // exclusive scan of the per-object cluster counts (the first kClObjects / 32 warps hold them)
    constexpr uint32_t kObjWarps = kClObjects / 32;
    static_assert(kClObjects % 32 == 0 && kObjWarps >= 1 && kObjWarps <= 2, "one or two warps of objects");
    if (warp < kObjWarps) {
        uint32_t incl = count;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += n;
        }
        if (lane == 31) s_warp[warp] = incl;
        s_start[threadIdx.x] = incl - count;  // provisional (warp-local)
    }
    __syncthreads();
    if (threadIdx.x >= 32 && threadIdx.x < kClObjects) s_start[threadIdx.x] += s_warp[0];
    if (threadIdx.x == 0) s_start[kClObjects] = kObjWarps == 2 ? s_warp[0] + s_warp[1] : s_warp[0];
    __syncthreads();
    const uint32_t T = s_start[kClObjects];

    if constexpr (!WRITE) {
        // count the surviving clusters of the tile
        uint32_t survivors = 0;
        for (uint32_t slot = threadIdx.x; slot < T; slot += kClThreads) {
            uint32_t lo = 0, hi = kClObjects;  // last object with start <= slot
            while (hi - lo > 1u) {
                const uint32_t mid = (lo + hi) >> 1;
                if (s_start[mid] <= slot) lo = mid;
                else hi = mid;
            }
            uint32_t ic, doff;
            if (cluster_visible(p, v, s_obj[lo], s_obj[lo].clusterOffset + (slot - s_start[lo]), s_snorm, ic, doff)) ++survivors;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) survivors += __shfl_xor_sync(0xFFFFFFFFu, survivors, o);
        __syncthreads();  // every s_warp read of the scan above is done
        if (lane == 0) s_warp[warp] = survivors;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t total = 0;
            for (int w = 0; w < kClWarps; ++w) total += s_warp[w];
            p.tileCount[tile] = total;
            if (s_flags) atomicOr(&p.scratch->status, s_flags);
        }
    } else {
        // the records of the tiles before this one
        uint32_t before = 0;
        for (uint32_t t = threadIdx.x; t < tile; t += kClThreads) before += __ldcg(p.tileCount + t);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) before += __shfl_xor_sync(0xFFFFFFFFu, before, o);
        __syncthreads();  // every s_warp read of the scan above is done
        if (lane == 0) s_warp[warp] = before;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t b = 0;
            for (int w = 0; w < kClWarps; ++w) b += s_warp[w];
            s_base = b;
        }
        __syncthreads();

        // the tile's clusters in slot order, records at their final positions
        uint32_t run = s_base;
        const uint32_t lt = lanemask_lt();
        for (uint32_t chunk = 0; chunk < T; chunk += kClThreads) {
            const uint32_t slot = chunk + threadIdx.x;
            bool vis = false;
            uint32_t ic = 0, doff = 0, cid = 0, obj = 0;
            if (slot < T) {
                uint32_t lo = 0, hi = kClObjects;
                while (hi - lo > 1u) {
                    const uint32_t mid = (lo + hi) >> 1;
                    if (s_start[mid] <= slot) lo = mid;
                    else hi = mid;
                }
                cid = s_obj[lo].clusterOffset + (slot - s_start[lo]);
                obj = s_obj[lo].objectId;
                vis = cluster_visible(p, v, s_obj[lo], cid, s_snorm, ic, doff);
            }
            const unsigned b = __ballot_sync(0xFFFFFFFFu, vis);
            __syncthreads();  // the previous chunk's s_warp reads are done
            if (lane == 0) s_warp[warp] = __popc(b);
            __syncthreads();
            uint32_t beforeW = 0, chunkTotal = 0;
#pragma unroll
            for (int w = 0; w < kClWarps; ++w) {
                const uint32_t c = s_warp[w];
                if (w < static_cast<int>(warp)) beforeW += c;
                chunkTotal += c;
            }
            if (vis) {
                const uint32_t out = run + beforeW + __popc(b & lt);
                if (out < p.capacity) {
                    uint32_t* rec = reinterpret_cast<uint32_t*>(p.cmds + static_cast<size_t>(out) * p.stride);
                    rec[0] = obj;
                    rec[1] = ic;
                    rec[2] = 1u;
                    rec[3] = doff;
                    rec[4] = 0u;
                    rec[5] = 0u;
                    if (p.clusterIds) p.clusterIds[out] = cid;
                }
            }
            run += chunkTotal;
        }
        if (threadIdx.x == 0 && tile == gridDim.x - 1u) {
            *p.drawCount = run;
            if (run > p.capacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
        }
    }
}

uint32_t cluster_tile_objects() { return kClObjects; }

cudaError_t launch_cluster_cull(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    uint32_t tiles = (p.count + kClObjects - 1) / kClObjects;
    if (tiles == 0) tiles = 1;
    cull_clusters_kernel<false><<<tiles, kClThreads, 0, s>>>(p, view);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cull_clusters_kernel<true><<<tiles, kClThreads, 0, s>>>(p, view);
    return cudaGetLastError();
}

}  // namespace blz
