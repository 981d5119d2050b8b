// cull_clusters.cu — object pass, cluster expansion and per-cluster culling.
//
// The reference splits this into PreClusterDrawCull.comp.glsl:13-47 (object frustum + LOD, then a
// serial loop that materialises one 12-byte ClusterDispatchData per cluster), a fence wait and CPU
// read-back of the cluster count (src/Renderer/BlitzenVulkan/vulkanDraw.cpp:874-905), and
// InitialClusterCull.comp.glsl:12-55 (one draw per cluster, its cone test commented out). Here,
// three launches with no block waiting on another and no host wait:
//   objects  one warp per tile of 32 objects: frustum + LOD select; the chosen LODs' clusters are
//            numbered object by object inside the tile (slots), and each object's clusters join a
//            work list in items of up to 64;
//   test     a persistent grid of warps, one item at a time: every cluster of the item is tested,
//            sphere frustum, Hi-Z when a pyramid is bound, and the normal cone in meshoptimizer's
//            documented form (VendorCode/Meshoptimizer/meshoptimizer.h:561-569). A visible cluster
//            sets its bit in the tile's slot-ordered visibility words and counts towards its tile
//            and the frame;
//   emit     one warp per tile with records: the records of the tiles before it (from the counts
//            per group of 64 tiles, which the test launch also keeps), then a record for every set
//            bit at its final position, without repeating a test.
// Nothing is materialised per candidate cluster but its bit.
//
// The task form (mesh-shader consumers) runs the same tests; its test launch also counts each
// object's survivors, from which the emit launch places the object's task record and its run of
// 32-meshlet payloads (MeshTaskPayload, VulkanShaderHeaders/ShaderBuffers.glsl:203-206).
#include <algorithm>

#include "blz_device.cuh"
#include "kernels.h"

namespace blz {

constexpr int kClThreads = 256;
constexpr int kClWarps = kClThreads / 32;
constexpr uint32_t kClObjects = 32;  // objects per tile
constexpr uint32_t kClItem = 64;     // clusters per work item of the test launch (two per lane)
constexpr uint32_t kClSuper = 64;     // tiles per group whose counts the test launch also sums
constexpr uint32_t kClPrefixLoads = 4;   // emit launch: group and tile counts each lane loads at once

// Sphere, Hi-Z and cone tests of one cluster of an object. The int8 cone axis and cutoff are divided
// by 127 only for the clusters that reach the cone test (about 2 % of them behind the occluders of a
// typical frame), not per block for every value they can take.
__device__ __forceinline__ bool cluster_visible(const ClusterParams& p, const ViewConsts& v, const float4 posScale,
                                                const float4 quat, uint32_t cid) {
    const float4* cp = reinterpret_cast<const float4*>(p.sc.clusters + cid);
    const float4 sph = __ldg(cp);
    const Vec3 w = model_to_world(Vec3{sph.x, sph.y, sph.z}, posScale, quat);
    const Vec3 c = view_transform(v.rows, w);
    const float r = BLZ_FM(sph.w, posScale.w);
    bool vis = frustum_check(c, r, v);
    if (vis && p.hasPyramid) {
        float4 aabb;
        if (project_sphere(c, r, v.zNear, v.proj0, v.proj5, aabb)) vis = vis && occlusion(aabb, p.pyr, v, c, r);
    }
    if (vis) {
        const uint32_t cone = __ldg(reinterpret_cast<const uint32_t*>(cp + 1));  // int8 axis xyz, cutoff
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

// Object launch, one warp per tile of 32 objects: frustum + LOD select (PreClusterDrawCull.comp.glsl:
// 20-37). Keeps each object's cluster range and transform and the tile's number of candidate
// clusters (slots, numbered object by object) for the later launches, zeroes the tile's visibility
// words, survivor counts and tile counts, and appends the object's clusters to the work list as
// items of up to kClItem clusters {object, first cluster, first slot in the tile, clusters}.
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
                if (lod.z > p.sc.clusterCount || lod.w > p.sc.clusterCount - lod.z || lod.w > p.bitWords) {
                    // (a range longer than the longest the scene had at upload does not fit the
                    // tile's visibility words or the work list: the object emits nothing)
                    flags |= BLZ_FLAG_BAD_INDEX;
                } else {
                    clusterOffset = lod.z;
                    count = lod.w;
                }
            }
        }
    }
    uint32_t incl = count;
    const uint32_t nItems = (count + kClItem - 1u) / kClItem;
    uint32_t itemIncl = nItems;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, d);
        const uint32_t m = __shfl_up_sync(0xFFFFFFFFu, itemIncl, d);
        if (lane >= static_cast<uint32_t>(d)) {
            incl += n;
            itemIncl += m;
        }
    }
    const uint32_t total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    const uint32_t itemTotal = __shfl_sync(0xFFFFFFFFu, itemIncl, 31);
    uint32_t itemBase = 0;
    if (lane == 31 && itemTotal != 0u) itemBase = atomicAdd(p.itemCount, itemTotal);
    itemBase = __shfl_sync(0xFFFFFFFFu, itemBase, 31) + itemIncl - nItems;
    const uint32_t start = incl - count;  // the object's first slot
    // the list holds every item a call can make; a count left over by a call whose later launches
    // never ran could still push past it, so nothing is written past the end (the test launch reads
    // at most itemCapacity items, and the call is flagged)
    for (uint32_t q = 0; q < nItems; ++q) {
        if (itemBase + q < p.itemCapacity)
            p.items[itemBase + q] = make_uint4(i, clusterOffset + q * kClItem, start + q * kClItem, min(kClItem, count - q * kClItem));
        else
            flags |= BLZ_FLAG_BAD_INDEX;
    }
    uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;
    for (uint32_t w = lane; w < (total + 31u) / 32u; w += 32u) bits[w] = 0u;
    p.objInfo[i] = make_uint2(clusterOffset, count);
    p.objSurv[i] = 0u;
    p.objXf[2u * i] = posScale;
    p.objXf[2u * i + 1u] = quat;
    flags = __reduce_or_sync(0xFFFFFFFFu, flags);
    if (tile == 0u && lane == 0) *p.totals = make_uint2(0u, 0u);
    if (tile % kClSuper == 0u && lane == 0) p.superCount[tile / kClSuper] = make_uint2(0u, 0u);
    if (lane == 0) {
        p.tileSlots[tile] = total;
        reinterpret_cast<uint2*>(p.tileCount)[tile] = make_uint2(0u, 0u);
        if (flags) atomicOr(&p.scratch->status, flags);
    }
}

// ORs a 32-slot ballot whose first slot is s0 into the slot-ordered visibility words (the ballot
// straddles two words unless s0 is a multiple of 32).
__device__ __forceinline__ void or_bits(uint32_t* bits, uint32_t s0, uint32_t bal) {
    if (bal == 0u) return;
    const uint32_t sh = s0 & 31u;
    atomicOr(bits + (s0 >> 5), bal << sh);
    if (sh != 0u && (bal >> (32u - sh)) != 0u) atomicOr(bits + (s0 >> 5) + 1u, bal >> (32u - sh));
}

// Test launch, a persistent grid of warps over the work list, one item per warp at a time: lane l
// tests the item's clusters l and l + 32 (two independent chains of loads and arithmetic), all of
// one object, whose transform every lane reads from the same address. The object and the cluster
// table rows are contiguous, so the loads coalesce and no lane searches for its object. Visible
// clusters set their bits (slot order) and count towards their tile (task form: towards their
// object, and the tile's tasks and payloads grow by what the object's new count adds: a task when
// it leaves zero, a payload per 32 survivors; the additions telescope to the final counts whatever
// the order of the items), and towards the frame's totals.
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_test_kernel(const ClusterParams p, const BlzCameraViewData view) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t nItems = min(__ldcg(p.itemCount), p.itemCapacity);
    const ViewConsts v = load_view(view);
    const uint32_t warpsTotal = gridDim.x * kClWarps;
    for (uint32_t it = blockIdx.x * kClWarps + warp; it < nItems; it += warpsTotal) {
        const uint4 item = __ldcg(p.items + it);  // {object, first cluster, first slot, clusters}
        const uint32_t o = item.x;
        const float4 ps = __ldcg(p.objXf + 2u * o), q = __ldcg(p.objXf + 2u * o + 1u);
        bool v0 = false, v1 = false;
        if (lane < item.w) v0 = cluster_visible(p, v, ps, q, item.y + lane);
        if (lane + 32u < item.w) v1 = cluster_visible(p, v, ps, q, item.y + 32u + lane);
        const uint32_t b0 = __ballot_sync(0xFFFFFFFFu, v0), b1 = __ballot_sync(0xFFFFFFFFu, v1);
        const uint32_t add = static_cast<uint32_t>(__popc(b0) + __popc(b1));
        if (add != 0u && lane == 0) {
            const uint32_t tile = o / kClObjects;
            uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;
            or_bits(bits, item.z, b0);
            or_bits(bits, item.z + 32u, b1);
            if constexpr (TASKS) {
                const uint32_t old = atomicAdd(p.objSurv + o, add);
                if (old == 0u) {
                    atomicAdd(p.tileCount + 2u * tile, 1u);
                    atomicAdd(&p.superCount[tile / kClSuper].x, 1u);
                    atomicAdd(&p.totals->x, 1u);
                }
                const uint32_t dp = (old + add + 31u) / 32u - (old + 31u) / 32u;
                if (dp != 0u) {
                    atomicAdd(p.tileCount + 2u * tile + 1u, dp);
                    atomicAdd(&p.superCount[tile / kClSuper].y, dp);
                    atomicAdd(&p.totals->y, dp);
                }
            } else {
                atomicAdd(p.tileCount + 2u * tile, add);
                atomicAdd(&p.superCount[tile / kClSuper].x, add);
                atomicAdd(&p.totals->x, add);
            }
        }
    }
}

// Emit launch, one warp per tile (lane = object): no test is repeated. The last tile's warp writes
// the frame's counts; a tile without records returns. The tile's cluster ranges, visibility bits
// and counts come from the earlier launches, the records (task form: tasks and payloads) before it
// from the counts of the groups of tiles before its group and of the tiles of its group before it;
// every set bit is written at its final position in slot order, the tile's set bits spread over
// the lanes 32 at a time.
template <bool TASKS>
__global__ void __launch_bounds__(kClThreads) cluster_emit_kernel(const ClusterParams p) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t tile = blockIdx.x * kClWarps + warp;
    if (tile >= p.tiles) return;
    const uint32_t lt = lanemask_lt();
    const uint32_t* bits = p.bits + static_cast<size_t>(tile) * p.bitWords;

    // the frame's totals (counted by the test launch) and, from the last tile, the rewind of the
    // work list, which the test launch has finished reading
    if (tile == p.tiles - 1u && lane == 0) {
        const uint2 tot = __ldcg(p.totals);
        if constexpr (TASKS) {
            *p.taskCount = tot.x;
            *p.payloadCount = tot.y;
            if (tot.x > p.taskCapacity || tot.y > p.payloadCapacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
        } else {
            *p.drawCount = tot.x;
            if (tot.x > p.capacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
        }
        *p.itemCount = 0u;
    }
    // a tile without records (task form: without tasks, so without payloads) writes nothing
    const uint2* tc = reinterpret_cast<const uint2*>(p.tileCount);
    if (__ldcg(tc + tile).x == 0u) return;

    // independent loads first
    const uint32_t T = __ldcg(p.tileSlots + tile);
    const uint32_t bFirst = lane < p.bitWords ? __ldcg(bits + lane) : 0u;
    const uint2 info = __ldcg(p.objInfo + tile * kClObjects + lane);  // {clusterOffset, count}
    const uint32_t sv = TASKS ? __ldcg(p.objSurv + tile * kClObjects + lane) : 0u;
    // records (task form: tasks, payloads) before the tile: the counts of the groups of kClSuper
    // tiles before its group, then of the tiles of its group before it, all loaded at once
    uint2 pre = make_uint2(0u, 0u);
    {
        const uint32_t sg = tile / kClSuper, t0 = sg * kClSuper;
        uint2 x[kClPrefixLoads];
#pragma unroll
        for (uint32_t j = 0; j < kClPrefixLoads; ++j) {
            const uint32_t i = j * 32u + lane;  // i < sg: group i; then tile t0 + (i - sg) while below `tile`
            if (i < sg) x[j] = __ldcg(p.superCount + i);
            else x[j] = t0 + (i - sg) < tile ? __ldcg(tc + t0 + (i - sg)) : make_uint2(0u, 0u);
        }
#pragma unroll
        for (uint32_t j = 0; j < kClPrefixLoads; ++j) {
            pre.x += x[j].x;
            pre.y += x[j].y;
        }
        for (uint32_t i = kClPrefixLoads * 32u + lane; i < sg + (tile - t0); i += 32u) {  // more groups than one round holds
            const uint2 y = i < sg ? __ldcg(p.superCount + i) : __ldcg(tc + t0 + (i - sg));
            pre.x += y.x;
            pre.y += y.y;
        }
    }
    pre.x = __reduce_add_sync(0xFFFFFFFFu, pre.x);
    pre.y = __reduce_add_sync(0xFFFFFFFFu, pre.y);

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
}

uint32_t cluster_tile_objects() { return kClObjects; }

uint32_t cluster_tile_groups(uint32_t tiles) { return (tiles + kClSuper - 1) / kClSuper; }

template <bool TASKS>
static cudaError_t launch_cluster(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    cluster_object_kernel<TASKS><<<(p.tiles + kClWarps - 1) / kClWarps, kClThreads, 0, s>>>(p, view);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // the test launch: every resident warp at once, or one warp per item when there are fewer
    const uint64_t maxItems = cluster_max_items(p.tiles, p.bitWords);
    uint64_t blocks = static_cast<uint64_t>(p.testBlocksPerSm > 0 ? p.testBlocksPerSm : 1) * (p.smCount > 0 ? p.smCount : 1);
    blocks = std::min<uint64_t>(blocks, (maxItems + kClWarps - 1) / kClWarps);
    cluster_test_kernel<TASKS><<<static_cast<uint32_t>(blocks ? blocks : 1), kClThreads, 0, s>>>(p, view);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cluster_emit_kernel<TASKS><<<(p.tiles + kClWarps - 1) / kClWarps, kClThreads, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t cluster_test_blocks_per_sm(bool tasks, int* out) {
    *out = 0;
    cudaError_t e = tasks ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, cluster_test_kernel<true>, kClThreads, 0)
                          : cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, cluster_test_kernel<false>, kClThreads, 0);
    if (e == cudaSuccess && *out < 1) *out = 1;
    return e;
}

uint64_t cluster_max_items(uint32_t tiles, uint32_t lodClusterMax) {
    // every object of every tile with the longest cluster range, in items of kClItem clusters
    return static_cast<uint64_t>(tiles) * kClObjects * ((std::max<uint32_t>(lodClusterMax, 1u) + kClItem - 1) / kClItem);
}

cudaError_t launch_cluster_cull(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    return launch_cluster<false>(p, view, s);
}

cudaError_t launch_cluster_tasks(const ClusterParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    return launch_cluster<true>(p, view, s);
}

}  // namespace blz
