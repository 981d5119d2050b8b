// cull_clusters.cu — object pass, cluster expansion and per-cluster culling.
//
// The reference splits this into PreClusterDrawCull.comp.glsl:13-47 (object frustum + LOD, then a
// serial loop that materialises one 12-byte ClusterDispatchData per cluster), a fence wait and CPU
// read-back of the cluster count (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:874-905), and
// InitialClusterCull.comp.glsl:12-55 (one draw per cluster, its cone test commented out). Here a
// block takes a tile of 32 objects, decides them and prefix-sums their cluster counts in shared
// memory, then walks the tile's clusters in order (a binary search maps a cluster slot back to
// its object), testing each one: sphere frustum, Hi-Z when a pyramid is bound, and the normal cone
// in meshoptimizer's documented form (VendorCode/Meshoptimizer/meshoptimizer.h:561-569).
// Two launches, no block waiting on another. The test launch keeps one visibility bit per
// candidate cluster, each object's cluster range and the tile's survivor count; the emit launch
// sums the counts of the tiles before its own (a strided read) and writes a record for every set
// bit at its final position, without repeating a test. Nothing is materialised per candidate but
// the bit, and the host never waits.
//
// The task form (mesh-shader consumers) runs the same tests; its test launch also keeps each
// object's number of survivors, from which the emit launch places the object's task record and
// its run of 32-meshlet payloads (MeshTaskPayload, VulkanShaderHeaders/ShaderBuffers.glsl:203-206).
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
                                                uint32_t cid, const float* snorm) {
    const float4* cp = reinterpret_cast<const float4*>(p.sc.clusters + cid);
    const float4 sph = __ldg(cp);
    const uint32_t cone = __ldg(reinterpret_cast<const uint32_t*>(cp + 1));  // int8 axis xyz, cutoff
    const Vec3 w = model_to_world(Vec3{sph.x, sph.y, sph.z}, o.posScale, o.quat);
    const Vec3 c = view_transform(v.rows, w);
    const float r = BLZ_FM(sph.w, o.posScale.w);
    bool vis = frustum_check(c, r, v);
    if (vis && p.hasPyramid) {
        float4 aabb;
        if (project_sphere(c, r, v.zNear, v.proj0, v.proj5, aabb)) vis = vis && occlusion(aabb, p.pyr, v, c, r);
    }
    if (vis) {
        const int ax = static_cast<int8_t>(cone & 0xFFu), ay = static_cast<int8_t>((cone >> 8) & 0xFFu);
        const int az = static_cast<int8_t>((cone >> 16) & 0xFFu), ac = static_cast<int8_t>(cone >> 24);
        const Vec3 axm{snorm[ax + 128], snorm[ay + 128], snorm[az + 128]};
        const float cutoff = snorm[ac + 128];
        const Vec3 axis = rotate_quat(axm, o.quat);
        const float dx = BLZ_FS(w.x, v.camX), dy = BLZ_FS(w.y, v.camY), dz = BLZ_FS(w.z, v.camZ);
        const float len = __fsqrt_rn(BLZ_FA(BLZ_FA(BLZ_FM(dx, dx), BLZ_FM(dy, dy)), BLZ_FM(dz, dz)));
        const float nx = BLZ_FD(dx, len), ny = BLZ_FD(dy, len), nz = BLZ_FD(dz, len);
        const float dp = BLZ_FA(BLZ_FA(BLZ_FM(nx, axis.x), BLZ_FM(ny, axis.y)), BLZ_FM(nz, axis.z));
        if (dp >= cutoff) vis = false;
    }
    return vis;
}

// Last object of the tile whose first slot is <= slot.
__device__ __forceinline__ uint32_t slot_object(const uint32_t* s_start, uint32_t slot) {
    uint32_t lo = 0, hi = kClObjects;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (s_start[mid] <= slot) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Test launch: object pass, expansion over the chosen LODs' clusters and the cluster tests. Keeps
// for the emit launch each object's cluster range (objInfo), one visibility bit per candidate
// (bits: the tile's slots in order, bitWords words per tile) and the tile's survivor count
// (task form: per-object survivors, and the tile's {tasks, payloads}).
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_test_kernel(const ClusterParams p, const BlzCameraViewData view) {
    static_assert(kClObjects == 32, "the tile's objects are one warp");
    __shared__ ClusterObj s_obj[kClObjects];
    __shared__ uint32_t s_start[kClObjects + 1];
    __shared__ uint32_t s_warp[kClWarps];
    __shared__ uint32_t s_surv[kClObjects];
    __shared__ unsigned int s_flags;
    __shared__ float s_snorm[256];
    if (threadIdx.x == 0) s_flags = 0u;
    for (uint32_t i = threadIdx.x; i < 256u; i += kClThreads)
        s_snorm[i] = BLZ_FD(static_cast<float>(static_cast<int>(i) - 128), 127.0f);
    const uint32_t tile = blockIdx.x;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;

    // object pass: PreClusterDrawCull.comp.glsl:20-37
    if (warp == 0) {
        const ViewConsts v = load_view(view);
        const uint32_t i = tile * kClObjects + lane;
        uint32_t count = 0;
        unsigned int flags = 0u;
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
        // exclusive scan of the per-object cluster counts
        uint32_t incl = count;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= static_cast<uint32_t>(d)) incl += n;
        }
        if (__shfl_sync(0xFFFFFFFFu, incl, 31) > 32u * p.bitWords) {
            // a LOD's cluster range grew past the largest one the scene had at upload: the tile's
            // bits would not fit, so it emits nothing and flags the scene
            flags |= BLZ_FLAG_BAD_INDEX;
            count = 0u;
            incl = 0u;
        }
        s_obj[lane] = o;
        s_surv[lane] = 0u;
        p.objInfo[tile * kClObjects + lane] = make_uint2(o.clusterOffset, count);
        s_start[lane] = incl - count;
        if (lane == 31) s_start[kClObjects] = incl;
        flags = __reduce_or_sync(0xFFFFFFFFu, flags);
        if (lane == 0) s_flags = flags;
    }
    __syncthreads();
    const uint32_t T = s_start[kClObjects];
    const ViewConsts v = load_view(view);
    uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;
    const uint32_t lt = lanemask_lt();
    uint32_t survivors = 0;
    for (uint32_t chunk = 0; chunk < T; chunk += kClThreads) {
        const uint32_t slot = chunk + threadIdx.x;
        bool vis = false;
        uint32_t lo = 0;
        if (slot < T) {
            lo = slot_object(s_start, slot);
            vis = cluster_visible(p, v, s_obj[lo], s_obj[lo].clusterOffset + (slot - s_start[lo]), s_snorm);
        }
        const unsigned bal = __ballot_sync(0xFFFFFFFFu, vis);
        if (lane == 0 && chunk + 32u * warp < T) bits[(chunk >> 5) + warp] = bal;
        if constexpr (TASKS) {
            // lanes of one object add once
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, vis ? lo : 0x100u + lane);
            if (vis && (peers & lt) == 0u) atomicAdd(&s_surv[lo], static_cast<uint32_t>(__popc(peers)));
        } else {
            survivors += __popc(bal);
        }
    }
    if constexpr (!TASKS) {
        if (lane == 0) s_warp[warp] = survivors;
    }
    __syncthreads();
    if constexpr (TASKS) {
        if (warp == 0) {
            const uint32_t sv = s_surv[lane];
            p.objSurv[tile * kClObjects + lane] = sv;
            const uint32_t tasks = __popc(__ballot_sync(0xFFFFFFFFu, sv != 0u));
            const uint32_t payloads = __reduce_add_sync(0xFFFFFFFFu, (sv + 31u) >> 5);
            if (lane == 0) reinterpret_cast<uint2*>(p.tileCount)[tile] = make_uint2(tasks, payloads);
        }
    } else if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (int w = 0; w < kClWarps; ++w) total += s_warp[w];
        p.tileCount[tile] = total;
    }
    if (threadIdx.x == 0 && s_flags) atomicOr(&p.scratch->status, s_flags);
}

// Emit launch: no test is repeated. The tile's cluster ranges and visibility bits come from the
// test launch; the records (task form: tasks and payloads) of the tiles before this one are summed
// from their counts, and each set bit is written at its final position in slot order.
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_emit_kernel(const ClusterParams p) {
    __shared__ uint32_t s_start[kClObjects + 1];
    __shared__ uint32_t s_off[kClObjects];
    __shared__ uint32_t s_first[kClObjects];  // task form: the object's first payload
    __shared__ uint32_t s_rank[kClObjects];   // task form: survivors of the tile before the object
    __shared__ uint32_t s_warp[kClWarps];
    __shared__ uint32_t s_warp2[kClWarps];
    __shared__ uint32_t s_base;
    const uint32_t tile = blockIdx.x;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t lt = lanemask_lt();

    // the records (task form: tasks, payloads) of the tiles before this one
    uint32_t before = 0, before2 = 0;
    if constexpr (TASKS) {
        const uint2* tc = reinterpret_cast<const uint2*>(p.tileCount);
        for (uint32_t t = threadIdx.x; t < tile; t += kClThreads) {
            const uint2 c = __ldcg(tc + t);
            before += c.x;
            before2 += c.y;
        }
        before2 = __reduce_add_sync(0xFFFFFFFFu, before2);
    } else {
        for (uint32_t t = threadIdx.x; t < tile; t += kClThreads) before += __ldcg(p.tileCount + t);
    }
    before = __reduce_add_sync(0xFFFFFFFFu, before);
    if (lane == 0) {
        s_warp[warp] = before;
        s_warp2[warp] = before2;
    }
    __syncthreads();
    if (warp == 0) {
        uint32_t base = 0, baseP = 0;
#pragma unroll
        for (int w = 0; w < kClWarps; ++w) {
            base += s_warp[w];
            baseP += s_warp2[w];
        }
        const uint2 info = __ldcg(p.objInfo + tile * kClObjects + lane);  // {clusterOffset, count}
        uint32_t incl = info.y;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= static_cast<uint32_t>(d)) incl += n;
        }
        s_start[lane] = incl - info.y;
        s_off[lane] = info.x;
        if (lane == 31) s_start[kClObjects] = incl;
        if constexpr (TASKS) {
            // per object: its task slot, first payload and the tile's survivors before it
            const uint32_t sv = __ldcg(p.objSurv + tile * kClObjects + lane);
            const uint32_t k = (sv + 31u) >> 5;
            uint32_t is = sv, ik = k;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t a = __shfl_up_sync(0xFFFFFFFFu, is, d);
                const uint32_t b = __shfl_up_sync(0xFFFFFFFFu, ik, d);
                if (lane >= static_cast<uint32_t>(d)) {
                    is += a;
                    ik += b;
                }
            }
            const unsigned has = __ballot_sync(0xFFFFFFFFu, sv != 0u);
            const uint32_t first = baseP + ik - k;
            s_rank[lane] = is - sv;
            s_first[lane] = first;
            if (sv != 0u) {
                const uint32_t t = base + __popc(has & lt);
                if (t < p.taskCapacity) {
                    uint32_t* tw = p.tasks + static_cast<size_t>(t) * 4u;
                    tw[0] = first;
                    tw[1] = k;
                    tw[2] = 1u;
                    tw[3] = 1u;
                }
                const uint32_t tail = sv & 31u;  // the last payload's unused slots
                const uint32_t last = first + k - 1u;
                if (tail != 0u && last < p.payloadCapacity) {
                    uint32_t* pw = p.payloads + static_cast<size_t>(last) * 33u + 1u;
                    for (uint32_t e = tail; e < 32u; ++e) pw[e] = BLZ_NO_MESHLET;
                }
            }
            if (lane == 31 && tile == gridDim.x - 1u) {
                const uint32_t nt = base + __popc(has), np = baseP + ik;
                *p.taskCount = nt;
                *p.payloadCount = np;
                if (nt > p.taskCapacity || np > p.payloadCapacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
            }
        } else if (lane == 0) {
            s_base = base;
        }
    }
    __syncthreads();
    const uint32_t T = s_start[kClObjects];
    const uint32_t words = (T + 31u) >> 5;
    const uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;
    uint32_t run = TASKS ? 0u : s_base;  // records before the current round of words
    for (uint32_t w0 = 0; w0 < words; w0 += kClThreads) {
        const uint32_t w = w0 + threadIdx.x;
        uint32_t b = w < words ? __ldcg(bits + w) : 0u;
        const uint32_t c = __popc(b);
        uint32_t incl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= static_cast<uint32_t>(d)) incl += n;
        }
        if (w0 != 0) __syncthreads();  // the previous round's s_warp reads are done
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        uint32_t q = run + incl - c, total = 0;
#pragma unroll
        for (int ww = 0; ww < kClWarps; ++ww) {
            const uint32_t n = s_warp[ww];
            if (ww < static_cast<int>(warp)) q += n;
            total += n;
        }
        while (b != 0u) {
            const uint32_t slot = w * 32u + static_cast<uint32_t>(__ffs(b) - 1);
            b &= b - 1u;
            const uint32_t lo = slot_object(s_start, slot);
            const uint32_t cid = s_off[lo] + (slot - s_start[lo]);
            if constexpr (TASKS) {
                const uint32_t rank = q - s_rank[lo];
                const uint32_t pi = s_first[lo] + (rank >> 5);
                if (pi < p.payloadCapacity) {
                    uint32_t* pw = p.payloads + static_cast<size_t>(pi) * 33u;
                    pw[1u + (rank & 31u)] = cid;
                    if ((rank & 31u) == 0u) pw[0] = tile * kClObjects + lo;
                }
            } else if (q < p.capacity) {
                // InitialClusterCull.comp.glsl:48-54: {objectId, triangleCount * 3, 1, dataOffset, 0, 0}
                const uint4 meta = __ldg(reinterpret_cast<const uint4*>(p.sc.clusters + cid) + 1);
                uint32_t* rec = reinterpret_cast<uint32_t*>(p.cmds + static_cast<size_t>(q) * p.stride);
                rec[0] = tile * kClObjects + lo;
                rec[1] = ((meta.z >> 8) & 0xFFu) * 3u;
                rec[2] = 1u;
                rec[3] = meta.y;
                rec[4] = 0u;
                rec[5] = 0u;
                if (p.clusterIds) p.clusterIds[q] = cid;
            }
            ++q;
        }
        run += total;
    }
    if constexpr (!TASKS) {
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
    cluster_test_kernel<false><<<tiles, kClThreads, 0, s>>>(p, view);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cluster_emit_kernel<false><<<tiles, kClThreads, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_cluster_tasks(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    uint32_t tiles = (p.count + kClObjects - 1) / kClObjects;
    if (tiles == 0) tiles = 1;
    cluster_test_kernel<true><<<tiles, kClThreads, 0, s>>>(p, view);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cluster_emit_kernel<true><<<tiles, kClThreads, 0, s>>>(p);
    return cudaGetLastError();
}

}  // namespace blz
