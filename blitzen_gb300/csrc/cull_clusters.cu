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
constexpr uint32_t kClMaxSplit = 4;  // test blocks per tile, at most

// Sphere, Hi-Z and cone tests of one cluster of an object. The int8 cone axis and cutoff are divided
// by 127 only for the clusters that reach the cone test (about 2 % of them behind the occluders of a
// typical frame), not per block for every value they can take.
__device__ __forceinline__ bool cluster_visible(const ClusterParams& p, const ViewConsts& v, const float4 posScale,
                                                const float4 quat, uint32_t cid) {
    const float4* cp = reinterpret_cast<const float4*>(p.sc.clusters + cid);
    const float4 sph = __ldg(cp);
    const uint32_t cone = __ldg(reinterpret_cast<const uint32_t*>(cp + 1));  // int8 axis xyz, cutoff
    const Vec3 w = model_to_world(Vec3{sph.x, sph.y, sph.z}, posScale, quat);
    const Vec3 c = view_transform(v.rows, w);
    const float r = BLZ_FM(sph.w, posScale.w);
    bool vis = frustum_check(c, r, v);
    if (vis && p.hasPyramid) {
        float4 aabb;
        if (project_sphere(c, r, v.zNear, v.proj0, v.proj5, aabb)) vis = vis && occlusion(aabb, p.pyr, v, c, r);
    }
    if (vis) {
        const int ax = static_cast<int8_t>(cone & 0xFFu), ay = static_cast<int8_t>((cone >> 8) & 0xFFu);
        const int az = static_cast<int8_t>((cone >> 16) & 0xFFu), ac = static_cast<int8_t>(cone >> 24);
        const Vec3 axm{BLZ_FD(static_cast<float>(ax), 127.0f), BLZ_FD(static_cast<float>(ay), 127.0f),
                       BLZ_FD(static_cast<float>(az), 127.0f)};
        const float cutoff = BLZ_FD(static_cast<float>(ac), 127.0f);
        const Vec3 axis = rotate_quat(axm, quat);
        const float dx = BLZ_FS(w.x, v.camX), dy = BLZ_FS(w.y, v.camY), dz = BLZ_FS(w.z, v.camZ);
        const float len = __fsqrt_rn(BLZ_FA(BLZ_FA(BLZ_FM(dx, dx), BLZ_FM(dy, dy)), BLZ_FM(dz, dz)));
        const float nx = BLZ_FD(dx, len), ny = BLZ_FD(dy, len), nz = BLZ_FD(dz, len);
        const float dp = BLZ_FA(BLZ_FA(BLZ_FM(nx, axis.x), BLZ_FM(ny, axis.y)), BLZ_FM(nz, axis.z));
        if (dp >= cutoff) vis = false;
    }
    return vis;
}

// Position of set bit n (0-based, n < popc(w)) of w: skip halves, quarters, ... that hold fewer
// than n + 1 set bits.
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t w, uint32_t n) {
    uint32_t pos = 0;
#pragma unroll
    for (uint32_t step = 16; step > 0; step >>= 1) {
        const uint32_t c = static_cast<uint32_t>(__popc(w & ((1u << step) - 1u)));
        if (n >= c) {
            n -= c;
            w >>= step;
            pos += step;
        }
    }
    return pos;
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

// Object launch, one warp per tile of 32 objects: frustum + LOD select (PreClusterDrawCull.comp.glsl:
// 20-37). Keeps each object's cluster range and transform and the tile's number of candidate
// clusters for the test launch.
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_object_kernel(const ClusterParams p, const BlzCameraViewData view) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t tile = blockIdx.x * kClWarps + warp;
    if (tile >= p.tiles) return;
    const ViewConsts v = load_view(view);
    const uint32_t i = tile * kClObjects + lane;
    uint32_t count = 0, clusterOffset = 0;
    unsigned int flags = 0u;
    float4 posScale = make_float4(0.f, 0.f, 0.f, 1.f), quat = make_float4(0.f, 0.f, 0.f, 1.f);
    if (i < p.count) {
        const uint2 ro = __ldg(reinterpret_cast<const uint2*>(p.objects) + i);
        bool ok = ro.x < p.sc.transformCount && ro.y < p.sc.surfaceCount;
        uint4 sm = make_uint4(0u, 0u, 0u, 0u);
        float4 sph = make_float4(0.f, 0.f, 0.f, 0.f);
        if (ok) {
            load_transform(p.sc, ro.x, posScale, quat);
            const float4* sp = reinterpret_cast<const float4*>(p.sc.surfaces + ro.y);
            sph = __ldg(sp);
            sm = __ldg(reinterpret_cast<const uint4*>(sp + 1));
            ok = sm.y < p.sc.lodCount && sm.z <= p.sc.lodCount - sm.y;
        }
        if (!ok) {
            flags |= BLZ_FLAG_BAD_INDEX;
        } else {
            const Vec3 c = view_transform(v.rows, model_to_world(Vec3{sph.x, sph.y, sph.z}, posScale, quat));
            const float r = BLZ_FM(sph.w, posScale.w);
            if (frustum_check(c, r, v)) {
                const float threshold = lod_threshold(c, r, posScale.w, v.lodTarget);
                uint32_t idx = 0;
                for (uint32_t k = 1; k < sm.z; ++k)
                    if (__ldg(&p.sc.lods[sm.y + k].error) < threshold) idx = k;
                const uint4 lod = __ldg(reinterpret_cast<const uint4*>(p.sc.lods + sm.y + idx));
                // lod.z = clusterOffset, lod.w = clusterCount
                if (lod.z > p.sc.clusterCount || lod.w > p.sc.clusterCount - lod.z) {
                    flags |= BLZ_FLAG_BAD_INDEX;
                } else {
                    clusterOffset = lod.z;
                    count = lod.w;
                }
            }
        }
    }
    uint32_t total = __reduce_add_sync(0xFFFFFFFFu, count);
    if (total > 32u * p.bitWords) {
        // a LOD's cluster range grew past the largest one the scene had at upload: the tile's
        // bits would not fit, so it emits nothing and flags the scene
        flags |= BLZ_FLAG_BAD_INDEX;
        count = 0u;
        total = 0u;
    }
    p.objInfo[i] = make_uint2(clusterOffset, count);
    if constexpr (TASKS) p.objSurv[i] = 0u;
    p.objXf[2u * i] = posScale;
    p.objXf[2u * i + 1u] = quat;
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    if (lane == 0) {
        p.tileSlots[tile] = total;
        reinterpret_cast<uint2*>(p.tileCount)[tile] = make_uint2(0u, 0u);
        if (flags) atomicOr(&p.scratch->status, flags);
    }
}

constexpr int kScanThreads = 1024;

// Scan launch, one block: exclusive prefix of the tiles' {records, 0} (task form: {tasks,
// payloads}) counts, tileCount -> tilePrefix.
__global__ void __launch_bounds__(kScanThreads) cluster_scan_kernel(const ClusterParams p) {
    __shared__ uint32_t s_a[kScanThreads / 32];
    __shared__ uint32_t s_b[kScanThreads / 32];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint2* tc = reinterpret_cast<const uint2*>(p.tileCount);
    constexpr uint32_t kPer = 2;  // tiles per thread per round
    uint32_t carryA = 0, carryB = 0;
    for (uint32_t base = 0; base < p.tiles; base += kScanThreads * kPer) {
        const uint32_t t0 = base + threadIdx.x * kPer;
        uint2 v[kPer];
        uint32_t a = 0, b = 0;
#pragma unroll
        for (uint32_t j = 0; j < kPer; ++j) {
            v[j] = t0 + j < p.tiles ? __ldcg(tc + t0 + j) : make_uint2(0u, 0u);
            a += v[j].x;
            b += v[j].y;
        }
        uint32_t ia = a, ib = b;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t na = __shfl_up_sync(0xFFFFFFFFu, ia, d);
            const uint32_t nb = __shfl_up_sync(0xFFFFFFFFu, ib, d);
            if (lane >= static_cast<uint32_t>(d)) {
                ia += na;
                ib += nb;
            }
        }
        if (lane == 31) {
            s_a[warp] = ia;
            s_b[warp] = ib;
        }
        __syncthreads();
        if (warp == 0) {  // scan of the warp totals
            uint32_t wa = s_a[lane], wb = s_b[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t na = __shfl_up_sync(0xFFFFFFFFu, wa, d);
                const uint32_t nb = __shfl_up_sync(0xFFFFFFFFu, wb, d);
                if (lane >= static_cast<uint32_t>(d)) {
                    wa += na;
                    wb += nb;
                }
            }
            s_a[lane] = wa;
            s_b[lane] = wb;
        }
        __syncthreads();
        uint32_t ra = carryA + ia - a + (warp ? s_a[warp - 1] : 0u);
        uint32_t rb = carryB + ib - b + (warp ? s_b[warp - 1] : 0u);
#pragma unroll
        for (uint32_t j = 0; j < kPer; ++j) {
            if (t0 + j < p.tiles) p.tilePrefix[t0 + j] = make_uint2(ra, rb);
            ra += v[j].x;
            rb += v[j].y;
        }
        carryA += s_a[31];
        carryB += s_b[31];
        __syncthreads();  // s_a, s_b are reused
    }
}

// Test launch: `split` blocks per tile, block `part` taking the tile's 256-slot chunks part,
// part + split, ... so that a tile with many candidates spreads over several SMs. Each chunk
// stores its eight visibility words and survivors are added to the tile's count (task form: to
// the objects' counts, each visibility word split at the object boundaries inside it).
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_test_kernel(const ClusterParams p, const BlzCameraViewData view) {
    static_assert(kClObjects == 32, "the tile's objects are one warp");
    __shared__ float4 s_xf[kClObjects][2];
    __shared__ uint32_t s_off[kClObjects];
    __shared__ uint32_t s_start[kClObjects + 1];
    __shared__ uint32_t s_warp[kClWarps];
    __shared__ uint32_t s_surv[kClObjects];
    const uint32_t tile = blockIdx.x / p.split, part = blockIdx.x - tile * p.split;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t T = __ldcg(p.tileSlots + tile);
    if (part * static_cast<uint32_t>(kClThreads) >= T) return;  // no chunk for this block
    if (warp == 0) {
        const uint32_t o = tile * kClObjects + lane;
        const uint2 info = __ldcg(p.objInfo + o);
        s_xf[lane][0] = __ldcg(p.objXf + 2u * o);
        s_xf[lane][1] = __ldcg(p.objXf + 2u * o + 1u);
        uint32_t incl = info.y;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= static_cast<uint32_t>(d)) incl += n;
        }
        s_start[lane] = incl - info.y;
        if (lane == 31) s_start[kClObjects] = incl;
        s_off[lane] = info.x;
        s_surv[lane] = 0u;
    }
    __syncthreads();
    const ViewConsts v = load_view(view);
    uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;
    uint32_t survivors = 0;
    for (uint32_t chunk = part * kClThreads; chunk < T; chunk += p.split * kClThreads) {
        const uint32_t slot = chunk + threadIdx.x;
        bool vis = false;
        uint32_t lo = 0;
        if (slot < T) {
            lo = slot_object(s_start, slot);
            vis = cluster_visible(p, v, s_xf[lo][0], s_xf[lo][1], s_off[lo] + (slot - s_start[lo]));
        }
        uint32_t bal = __ballot_sync(0xFFFFFFFFu, vis);
        if (lane == 0 && bal != 0u) {
            bits[(chunk >> 5) + warp] = bal;
            if constexpr (TASKS) {
                // the word's set bits per object, from lane 0's object on
                const uint32_t slot0 = chunk + 32u * warp;
                while (bal != 0u && lo < kClObjects) {
                    const uint32_t n = min(32u, s_start[lo + 1u] - slot0);  // low bits in objects <= lo
                    const uint32_t mask = n >= 32u ? 0xFFFFFFFFu : (1u << n) - 1u;
                    const uint32_t c = __popc(bal & mask);
                    if (c != 0u) atomicAdd(&s_surv[lo], c);
                    bal &= ~mask;
                    ++lo;
                }
            } else {
                survivors += __popc(bal);
            }
        } else if (lane == 0 && chunk + 32u * warp < T) {
            bits[(chunk >> 5) + warp] = 0u;
        }
    }
    if constexpr (!TASKS) {
        if (lane == 0) s_warp[warp] = survivors;
    }
    __syncthreads();
    if constexpr (TASKS) {
        if (warp == 0 && s_surv[lane] != 0u) atomicAdd(p.objSurv + tile * kClObjects + lane, s_surv[lane]);
    } else if (threadIdx.x == 0) {
        uint32_t total = 0;
        for (int w = 0; w < kClWarps; ++w) total += s_warp[w];
        if (total != 0u) atomicAdd(p.tileCount + 2u * tile, total);
    }
}

// Task form, one warp per tile: the tile's {tasks, payloads} from its objects' survivor counts.
__global__ void __launch_bounds__(kClThreads) cluster_task_totals_kernel(const ClusterParams p) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t tile = blockIdx.x * kClWarps + warp;
    if (tile >= p.tiles) return;
    const uint32_t sv = __ldcg(p.objSurv + tile * kClObjects + lane);
    const uint32_t tasks = __popc(__ballot_sync(0xFFFFFFFFu, sv != 0u));
    const uint32_t payloads = __reduce_add_sync(0xFFFFFFFFu, (sv + 31u) >> 5);
    if (lane == 0) reinterpret_cast<uint2*>(p.tileCount)[tile] = make_uint2(tasks, payloads);
}

// Emit launch, one warp per tile (lane = object): no test is repeated. The tile's cluster ranges,
// visibility bits and the records (task form: tasks and payloads) before it come from the earlier
// launches; every set bit is written at its final position in slot order, the tile's set bits
// spread over the lanes 32 at a time.
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_emit_kernel(const ClusterParams p) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t tile = blockIdx.x * kClWarps + warp;
    if (tile >= p.tiles) return;
    const uint32_t lt = lanemask_lt();
    const uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;

    // independent loads first
    const uint32_t T = __ldcg(p.tileSlots + tile);
    const uint32_t bFirst = lane < p.bitWords ? __ldcg(bits + lane) : 0u;
    const uint2 info = __ldcg(p.objInfo + tile * kClObjects + lane);  // {clusterOffset, count}
    const uint2 pre = __ldcg(p.tilePrefix + tile);                    // records (tasks, payloads) before the tile
    const uint32_t sv = TASKS ? __ldcg(p.objSurv + tile * kClObjects + lane) : 0u;

    uint32_t incl = info.y;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        if (lane >= static_cast<uint32_t>(d)) incl += n;
    }
    const uint32_t start = incl - info.y;  // the object's first slot
    uint32_t first = 0, before = 0;        // task form: first payload, the tile's survivors before the object
    if constexpr (TASKS) {
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
        first = pre.y + ik - k;
        before = is - sv;
        if (sv != 0u) {
            const uint32_t t = pre.x + __popc(has & lt);
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
        if (lane == 31 && tile == p.tiles - 1u) {
            const uint32_t nt = pre.x + __popc(has), np = pre.y + ik;
            *p.taskCount = nt;
            *p.payloadCount = np;
            if (nt > p.taskCapacity || np > p.payloadCapacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
        }
    }

    const uint32_t words = (T + 31u) >> 5;
    uint32_t run = TASKS ? 0u : pre.x;  // records (task form: the tile's survivors) before this round
    uint32_t bNext = lane < words ? bFirst : 0u;
    for (uint32_t w0 = 0; w0 < words; w0 += 32u) {
        const uint32_t b = bNext;  // this round's word; the next round's is loaded ahead
        bNext = w0 + 32u + lane < words ? __ldcg(bits + w0 + 32u + lane) : 0u;
        const uint32_t c = __popc(b);
        uint32_t wincl = c;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, wincl, d);
            if (lane >= static_cast<uint32_t>(d)) wincl += n;
        }
        const uint32_t wexcl = wincl - c;
        const uint32_t roundTotal = __shfl_sync(0xFFFFFFFFu, wincl, 31);
        for (uint32_t k0 = 0; k0 < roundTotal; k0 += 32u) {
            const uint32_t k = k0 + lane;  // the round's set bit taken by this lane
            uint32_t j = 0;                // its word: the number of words with wincl <= k
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xFFFFFFFFu, wincl, j + step - 1u) <= k) j += step;
            const uint32_t wj = __shfl_sync(0xFFFFFFFFu, b, j);
            const uint32_t ej = __shfl_sync(0xFFFFFFFFu, wexcl, j);
            const uint32_t slot = (w0 + j) * 32u + (k < roundTotal ? nth_set_bit(wj, k - ej) : 0u);
            uint32_t lo = 0;  // its object: the last one whose first slot is <= slot
#pragma unroll
            for (uint32_t step = 16; step > 0; step >>= 1)
                if (__shfl_sync(0xFFFFFFFFu, start, lo + step) <= slot) lo += step;
            const uint32_t cid = __shfl_sync(0xFFFFFFFFu, info.x, lo) + (slot - __shfl_sync(0xFFFFFFFFu, start, lo));
            const uint32_t q = run + k;
            if constexpr (TASKS) {
                const uint32_t rank = q - __shfl_sync(0xFFFFFFFFu, before, lo);
                const uint32_t pi = __shfl_sync(0xFFFFFFFFu, first, lo) + (rank >> 5);
                if (k < roundTotal && pi < p.payloadCapacity) {
                    uint32_t* pw = p.payloads + static_cast<size_t>(pi) * 33u;
                    pw[1u + (rank & 31u)] = cid;
                    if ((rank & 31u) == 0u) pw[0] = tile * kClObjects + lo;
                }
            } else if (k < roundTotal && q < p.capacity) {
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
        }
        run += roundTotal;
    }
    if constexpr (!TASKS) {
        if (lane == 0 && tile == p.tiles - 1u) {
            *p.drawCount = run;
            if (run > p.capacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
        }
    }
}

uint32_t cluster_tile_objects() { return kClObjects; }

template <bool TASKS>
static cudaError_t launch_cluster(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    cluster_object_kernel<TASKS><<<(p.tiles + kClWarps - 1) / kClWarps, kClThreads, 0, s>>>(p, view);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cluster_test_kernel<TASKS><<<p.tiles * p.split, kClThreads, 0, s>>>(p, view);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    if constexpr (TASKS) {
        cluster_task_totals_kernel<<<(p.tiles + kClWarps - 1) / kClWarps, kClThreads, 0, s>>>(p);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    cluster_scan_kernel<<<1, kScanThreads, 0, s>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cluster_emit_kernel<TASKS><<<(p.tiles + kClWarps - 1) / kClWarps, kClThreads, 0, s>>>(p);
    return cudaGetLastError();
}

uint32_t cluster_split(uint32_t lodClusterMax) {
    // blocks per tile: enough that the most a tile can hold (32 objects x the largest LOD) spreads
    // over several SMs, at most kClMaxSplit
    const uint32_t chunks = (kClObjects * lodClusterMax + kClThreads - 1) / kClThreads;
    return chunks < 1u ? 1u : (chunks > kClMaxSplit ? kClMaxSplit : chunks);
}

cudaError_t launch_cluster_cull(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    return launch_cluster<false>(p, view, s);
}

cudaError_t launch_cluster_tasks(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    return launch_cluster<true>(p, view, s);
}

}  // namespace blz
