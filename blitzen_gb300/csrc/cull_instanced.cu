// cull_instanced.cu — instanced cull in one pass: per-LOD instance lists plus one command per
// non-empty LOD.
//
// The reference runs three dispatches with atomics (drawInstCountReset.cs.hlsl:9-18,
// drawInstCull.cs.hlsl:12-42, drawInstCmd.cs.hlsl:9-38; dispatch at
// src/Renderer/BlitzenDX12/dx12Draw.cpp:340-415). Here a single launch partitions the visible
// objects stably into LOD buckets: each warp ranks its objects per bucket with __match_any_sync
// into a warp-private histogram row, the block scans the rows per bucket, and every bucket has
// its own decoupled look-back chain across tiles. Instance ids land in ascending object order
// inside each LOD; the tile that finishes the chain writes the counters and the commands in
// ascending LOD order.
#include "blz_device.cuh"
#include "kernels.h"

namespace blz {

constexpr int kInstThreads = 256;
constexpr int kInstOpt = 8;
constexpr int kInstWarps = kInstThreads / 32;
constexpr uint32_t kInstTile = kInstThreads * kInstOpt;
constexpr uint32_t kNoBucket = 0xFFFFFFFFu;

// Frustum + LOD decision (drawInstCull.cs.hlsl:22-36). Returns the global LOD id or kNoBucket.
__device__ __forceinline__ uint32_t inst_bucket(const SceneTables& sc, const BlzRenderObject* objects, uint32_t i,
                                                const ViewConsts& v, unsigned int& flags) {
    const uint2 ro = __ldg(reinterpret_cast<const uint2*>(objects) + i);
    if (ro.x >= sc.transformCount || ro.y >= sc.surfaceCount) {
        flags |= BLZ_FLAG_BAD_INDEX;
        return kNoBucket;
    }
    float4 ps, q;
    load_transform(sc, ro.x, ps, q);
    const float4* sp = reinterpret_cast<const float4*>(sc.surfaces + ro.y);
    const float4 sph = __ldg(sp);
    const uint4 sm = __ldg(reinterpret_cast<const uint4*>(sp + 1));
    if (!(sm.y < sc.lodCount && sm.z <= sc.lodCount - sm.y)) {
        flags |= BLZ_FLAG_BAD_INDEX;
        return kNoBucket;
    }
    const Vec3 c = view_transform(v.rows, model_to_world(Vec3{sph.x, sph.y, sph.z}, ps, q));
    const float r = BLZ_FM(sph.w, ps.w);
    if (!frustum_check(c, r, v)) return kNoBucket;
    const float threshold = lod_threshold(c, r, ps.w, v.lodTarget);
    uint32_t idx = 0;
    for (uint32_t k = 1; k < sm.z; ++k)
        if (__ldg(&sc.lods[sm.y + k].error) < threshold) idx = k;
    return sm.y + idx;
}

__global__ void __launch_bounds__(kInstThreads) cull_instanced_kernel(const InstancedParams p, const BlzCameraViewData view) {
    extern __shared__ uint32_t s_dyn[];
    const uint32_t nL = p.sc.lodCount;
    uint32_t* hist = s_dyn;                  // [kInstWarps][nL] warp rows, then exclusive offsets
    uint32_t* bucketBase = s_dyn + kInstWarps * nL;  // [nL] global exclusive prefix per bucket
    __shared__ uint32_t s_tile, s_epoch;
    __shared__ unsigned int s_flags;
    __shared__ uint32_t s_warpSums[kInstWarps];
    Scratch* scr = p.scratch;
    unsigned long long* states = scr->state;  // [tiles][nL]

    if (threadIdx.x == 0) {
        s_tile = atomicAdd(&scr->ticket, 1u);
        s_epoch = *reinterpret_cast<volatile unsigned int*>(&scr->epoch);
        s_flags = 0u;
    }
    for (uint32_t j = threadIdx.x; j < kInstWarps * nL; j += kInstThreads) hist[j] = 0u;
    __syncthreads();
    const uint32_t tile = s_tile, epoch = s_epoch;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    if (tile >= gridDim.x) {
        // a ticket past the grid: the protocol state was left behind by a launch that gave up on a
        // wait; this block touches no tile state and only takes part in the exit protocol
        if (threadIdx.x == 0) {
            atomicOr(&scr->status, BLZ_FLAG_TIMEOUT);
            __threadfence();
            if (atomicAdd(&scr->doneBlocks, 1u) == gridDim.x - 1u) {
                scr->ticket = 0u;
                scr->doneBlocks = 0u;
                __threadfence();
                atomicExch(&scr->epoch, epoch + 1u);
            }
        }
        return;
    }
    const ViewConsts v = load_view(view);
    // warp w owns objects [base + w*32*OPT, base + (w+1)*32*OPT), visited k-major (coalesced)
    const uint32_t wbase = tile * kInstTile + warp * 32u * kInstOpt;
    const uint32_t lt = lanemask_lt();
    uint32_t bucket[kInstOpt], off[kInstOpt];
    unsigned int flags = 0u;
    uint32_t* row = hist + warp * nL;
#pragma unroll
    for (int k = 0; k < kInstOpt; ++k) {
        const uint32_t i = wbase + k * 32u + lane;
        bucket[k] = (i < p.count) ? inst_bucket(p.sc, p.objects, i, v, flags) : kNoBucket;
    }
#pragma unroll
    for (int k = 0; k < kInstOpt; ++k) {
        const unsigned peers = __match_any_sync(0xFFFFFFFFu, bucket[k]);
        const uint32_t leader = __ffs(peers) - 1u;
        uint32_t old = 0;
        if (bucket[k] != kNoBucket && lane == leader) {
            old = row[bucket[k]];
            row[bucket[k]] = old + __popc(peers);
        }
        old = __shfl_sync(0xFFFFFFFFu, old, leader);
        off[k] = old + __popc(peers & lt);
        __syncwarp();
    }
    if (flags) atomicOr(&s_flags, flags);
    __syncthreads();

    // per bucket: exclusive scan over warp rows, publish the tile aggregate, look back
    for (uint32_t b = threadIdx.x; b < nL; b += kInstThreads) {
        uint32_t run = 0;
#pragma unroll
        for (int w = 0; w < kInstWarps; ++w) {
            const uint32_t c = hist[w * nL + b];
            hist[w * nL + b] = run;
            run += c;
        }
        unsigned long long* st = states + static_cast<size_t>(tile) * nL + b;
        uint32_t excl = 0;
        if (tile == 0) {
            store_state(st, pack_state(epoch, kStatePrefix, run));
        } else {
            store_state(st, pack_state(epoch, kStateAggregate, run));
            unsigned long long spins = 0;
            for (int64_t t = static_cast<int64_t>(tile) - 1; t >= 0;) {
                const unsigned long long s = load_state(states + static_cast<size_t>(t) * nL + b);
                const uint32_t lo = static_cast<uint32_t>(s);
                const uint32_t flag = (static_cast<uint32_t>(s >> 32) == epoch) ? (lo >> 30) : 0u;
                if (flag == 0u) {
                    if (++spins > p.spinLimit) {
                        atomicOr(&scr->status, BLZ_FLAG_TIMEOUT);
                        break;
                    }
                    continue;
                }
                excl += lo & kValueMask;
                if (flag == kStatePrefix) break;
                --t;
            }
            store_state(st, pack_state(epoch, kStatePrefix, excl + run));
        }
        bucketBase[b] = excl;
    }
    __syncthreads();

    // scatter instance ids
    const uint32_t slots = p.slotsPerLod ? p.slotsPerLod : 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < kInstOpt; ++k) {
        if (bucket[k] == kNoBucket) continue;
        const uint32_t b = bucket[k];
        const uint32_t pos = bucketBase[b] + hist[warp * nL + b] + off[k];
        const uint64_t at = static_cast<uint64_t>(__ldg(&p.counters[b].instanceOffset)) + pos;
        if (pos < slots && at < p.instanceCapacity) p.instances[at] = wbase + k * 32u + lane;
        else flags |= BLZ_FLAG_INSTANCE_OVERFLOW;
    }
    if (flags) atomicOr(&s_flags, flags);

    // the last tile holds every bucket's total: counters, then commands in ascending LOD order
    if (tile == gridDim.x - 1u) {
        __syncthreads();
        uint32_t running = 0;  // commands before this thread's chunk of buckets
        const uint32_t per = (nL + kInstThreads - 1) / kInstThreads;
        const uint32_t b0 = min(nL, threadIdx.x * per), b1 = min(nL, b0 + per);
        uint32_t mine = 0;
        // every bucket's total is this tile's published inclusive prefix
        for (uint32_t b = b0; b < b1; ++b) {
            const unsigned long long s = load_state(states + static_cast<size_t>(tile) * nL + b);
            const uint32_t total = static_cast<uint32_t>(s) & kValueMask;
            hist[b] = total;  // reuse row 0 as the totals array
            mine += total ? 1u : 0u;
        }
        // block exclusive scan of per-thread non-empty counts
        uint32_t incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += n;
        }
        if (lane == 31) s_warpSums[warp] = incl;
        __syncthreads();
        uint32_t warpOff = 0, all = 0;
        for (int w = 0; w < kInstWarps; ++w) {
            if (w < static_cast<int>(warp)) warpOff += s_warpSums[w];
            all += s_warpSums[w];
        }
        running = warpOff + incl - mine;
        unsigned int f = 0u;
        for (uint32_t b = b0; b < b1; ++b) {
            const uint32_t total = hist[b];
            p.counters[b].instanceCount = total;
            if (total > slots || static_cast<uint64_t>(__ldg(&p.counters[b].instanceOffset)) + min(total, slots) > p.instanceCapacity)
                f |= BLZ_FLAG_INSTANCE_OVERFLOW;
            if (total == 0u) continue;
            if (running < p.capacity) {
                uint8_t* rec = p.cmds + static_cast<size_t>(running) * p.stride;
                uint32_t* w = reinterpret_cast<uint32_t*>(rec);
                const uint2 lod = __ldg(reinterpret_cast<const uint2*>(p.sc.lods + b));
                w[0] = __ldg(&p.counters[b].instanceOffset);
                w[1] = lod.x;
                w[2] = min(total, slots);
                w[3] = lod.y;
                w[4] = 0u;
                w[5] = 0u;
            }
            ++running;
        }
        if (all > p.capacity) f |= BLZ_FLAG_COMMAND_OVERFLOW;
        if (f) atomicOr(&s_flags, f);
        if (threadIdx.x == 0) *p.drawCount = all;
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_flags) atomicOr(&scr->status, s_flags);
    // exit protocol shared with the object kernels
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&scr->doneBlocks, 1u) == gridDim.x - 1u) {
            scr->ticket = 0u;
            scr->doneBlocks = 0u;
            __threadfence();
            atomicExch(&scr->epoch, epoch + 1u);
        }
    }
}

uint32_t instanced_tile_size() { return kInstTile; }

size_t instanced_smem_bytes(uint32_t lodCount) { return (static_cast<size_t>(kInstWarps) + 1) * lodCount * sizeof(uint32_t); }

cudaError_t launch_instanced_cull(const InstancedParams& p, const BlzCameraViewData& view, cudaStream_t s) {
    uint32_t tiles = (p.count + kInstTile - 1) / kInstTile;
    if (tiles == 0) tiles = 1;
    const size_t smem = instanced_smem_bytes(p.sc.lodCount);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(cull_instanced_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smem));
        if (e != cudaSuccess) return e;
    }
    cull_instanced_kernel<<<tiles, kInstThreads, smem, s>>>(p, view);
    return cudaGetLastError();
}

}  // namespace blz
