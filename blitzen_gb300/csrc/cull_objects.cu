// cull_objects.cu — per-object cull kernels: frustum, occlusion pass 1 / pass 2, temporal
// occlusion, for one view or many views in one launch.
//
// Two kernels per launch, no block ever waiting on another:
//   decide   a streaming grid (several blocks per SM, grid-stride over 512-object chunks of all
//            views) loads render objects and gathers their transforms with batched read-only loads,
//            decides every object, ranks the emitted ones in ascending object order with warp
//            ballots and a block scan, and stages them compacted — (objectId, lodId), 8 bytes — in
//            the chunk's slice of a scratch buffer, with the chunk's count. The last block to
//            finish scans the chunk counts per view (output offsets and draw counts).
//   scatter  copies each chunk's staged records to their final slots as full indirect records,
//            coalesced.
// The scratch traffic is 16 bytes per emitted object, against 40-48 bytes read per object.
//
// Reference passes (paths inside the Blitzen project):
//   FRUSTUM   TransparentDrawCull.comp.glsl:13-65, drawCull.cs.hlsl:10-52
//   FIRST     InitialDrawCull.comp.glsl:12-59,     drawOccFirst.cs.hlsl:13-58
//   LATE      LateDrawCull.comp.glsl:13-72,        drawOccLate.cs.hlsl:13-67
//   TEMPORAL  drawOccTemporal.hlsl:13-64
#include "blz_device.cuh"
#include "kernels.h"

namespace blz {

constexpr int kModeRuntime = -1;  // batch: the mode is read per view

// ------------------------------------------------------------------ per-view access

template <bool SINGLE>
__device__ __forceinline__ const BatchViewDev& view_of(const PipeParams& p, uint32_t vi) {
    if constexpr (SINGLE) {
        return p.single;
    } else {
        return p.views[vi];
    }
}

// Chunk c belongs to the view v with tileStart[v] <= c < tileStart[v + 1].
__device__ __forceinline__ uint32_t find_view(const uint32_t* tileStart, uint32_t nViews, uint32_t c) {
    uint32_t lo = 0, hi = nViews;
    while (hi - lo > 1u) {
        const uint32_t mid = (lo + hi) >> 1;
        if (__ldg(tileStart + mid) <= c) lo = mid;
        else hi = mid;
    }
    return lo;
}

// ------------------------------------------------------------------ decisions

constexpr uint32_t kChunk = 512;  // objects per chunk: the unit of staging, counting and scanning

// One warp decides a chunk of kChunk consecutive render objects of a view, 32 * OPT at a time
// (object base + k * 32 + lane for k < OPT, so the step is k-major and lanes ascend).
// For each step:
//   1  every lane loads its OPT render objects and then their transforms (all reads issued before
//      any arithmetic) and runs the frustum test;
//   2  the frustum survivors are ranked with ballots — survivor order is object order — and handed
//      to dense lanes with __fns + shuffles, so the sphere projection, Hi-Z test (LATE/TEMPORAL)
//      and LOD selection run on packed lanes, not on every lane of every warp with a survivor;
//   3  the emitted survivors are ranked with one more ballot and appended to the chunk's staging
//      as (objectId, lodId); LATE writes every object's new visibility.
// No shared memory and no block barrier: warps never wait for one another.
template <int MODE, int OPT>
__device__ __forceinline__ uint32_t decide_chunk_warp(const SceneTables& sc, const BatchViewDev& bv, uint32_t base,
                                                      uint2* stage, unsigned int& flags) {
    constexpr uint32_t STEP = 32u * OPT;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t count = bv.count;
    const ViewConsts v = load_view(bv.view);
    uint32_t run = 0;  // emitted so far in this chunk
    const uint32_t limit = min(base + kChunk, count);
    // render objects and visibility words of the next step are fetched one step ahead, so a step
    // waits on one DRAM latency (its transforms), not two
    uint2 nro[OPT];
    uint32_t nvis[OPT];
    auto prefetch = [&](uint32_t at) {
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            const uint32_t i = at + k * 32u + lane;
            const bool in = i < limit;
            nro[k] = in ? __ldg(reinterpret_cast<const uint2*>(bv.objects) + i) : make_uint2(0u, 0u);
            nvis[k] = 1u;
            if (MODE == BLZ_MODE_FIRST && in) nvis[k] = __ldg(bv.vis + i);
            if (MODE == BLZ_MODE_LATE && in) nvis[k] = bv.vis[i];  // rewritten later by this warp: coherent load
        }
    };
    prefetch(base);
    for (uint32_t sb = base; sb < limit; sb += STEP) {
        // 1. loads, then the frustum test on the owning lane
        uint32_t visPrev[OPT];
        bool act[OPT];
        uint2 ro[OPT];
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            const uint32_t i = sb + k * 32u + lane;
            act[k] = i < limit;
            visPrev[k] = nvis[k];
            if (MODE == BLZ_MODE_FIRST) act[k] = act[k] && visPrev[k] != 0u;  // drawOccFirst.cs.hlsl:22-25
            ro[k] = act[k] ? nro[k] : make_uint2(0u, 0u);
        }
        float4 ps[OPT], q[OPT];
        bool ok[OPT];
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            ok[k] = act[k] && ro[k].x < sc.transformCount && ro[k].y < sc.surfaceCount;
            ps[k] = make_float4(0.f, 0.f, 0.f, 1.f);
            q[k] = make_float4(0.f, 0.f, 0.f, 1.f);
            if (ok[k]) {
                const BlzMeshTransform* t = ((bv.dynT != nullptr && ro[k].x < bv.dynCount) ? bv.dynT : sc.transforms) + ro[k].x;
                const float4* tp = reinterpret_cast<const float4*>(t);
                ps[k] = __ldg(tp);
                q[k] = __ldg(tp + 1);
            }
        }
        if (sb + STEP < limit) prefetch(sb + STEP);
        float cx[OPT], cy[OPT], cz[OPT], cr[OPT];
        uint32_t lodOff[OPT], lodCnt[OPT];
        unsigned survivors[OPT];
        uint32_t before[OPT + 1];
        before[0] = 0;
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            bool inFrustum = false;
            cx[k] = cy[k] = cz[k] = cr[k] = 0.f;
            lodOff[k] = lodCnt[k] = 0u;
            if (ok[k]) {
                const float4* sp = reinterpret_cast<const float4*>(sc.surfaces + ro[k].y);
                const float4 sph = __ldg(sp);
                const uint4 s1 = __ldg(reinterpret_cast<const uint4*>(sp + 1));  // materialId, lodOffset, lodCount, vertexOffset
                if (s1.y < sc.lodCount && s1.z <= sc.lodCount - s1.y) {
                    const Vec3 c = view_transform(v.rows, model_to_world(Vec3{sph.x, sph.y, sph.z}, ps[k], q[k]));
                    const float r = BLZ_FM(sph.w, ps[k].w);
                    inFrustum = frustum_check(c, r, v);
                    cx[k] = c.x;
                    cy[k] = c.y;
                    cz[k] = c.z;
                    cr[k] = r;
                    lodOff[k] = s1.y;
                    lodCnt[k] = s1.z;
                } else {
                    flags |= BLZ_FLAG_BAD_INDEX;
                }
            } else if (act[k]) {
                flags |= BLZ_FLAG_BAD_INDEX;
            }
            if (MODE == BLZ_MODE_LATE && act[k] && !inFrustum) bv.vis[sb + k * 32u + lane] = 0u;  // drawOccLate.cs.hlsl:67
            survivors[k] = __ballot_sync(0xFFFFFFFFu, inFrustum);
            before[k + 1] = before[k] + __popc(survivors[k]);
        }
        const uint32_t n = before[OPT];
        // 2. dense rounds over the survivors, in object order
        for (uint32_t jb = 0; jb < n; jb += 32u) {
            const uint32_t j = jb + lane;
            const bool mine = j < n;
            int kk = 0;
#pragma unroll
            for (int k = 1; k < OPT; ++k)
                if (j >= before[k]) kk = k;
            uint32_t src = lane;
            if (mine) src = __fns(survivors[kk], 0u, static_cast<int>(j - before[kk]) + 1);
            float fx = 0.f, fy = 0.f, fz = 0.f, fr = 0.f, fs = 0.f;
            uint32_t fo = 0u, fc = 0u, fv = 0u;
#pragma unroll
            for (int k = 0; k < OPT; ++k) {  // every lane takes part in every shuffle
                const float x = __shfl_sync(0xFFFFFFFFu, cx[k], src), y = __shfl_sync(0xFFFFFFFFu, cy[k], src);
                const float z = __shfl_sync(0xFFFFFFFFu, cz[k], src), r = __shfl_sync(0xFFFFFFFFu, cr[k], src);
                const float sc_ = __shfl_sync(0xFFFFFFFFu, ps[k].w, src);
                const uint32_t o = __shfl_sync(0xFFFFFFFFu, lodOff[k], src), c = __shfl_sync(0xFFFFFFFFu, lodCnt[k], src);
                const uint32_t vp = __shfl_sync(0xFFFFFFFFu, visPrev[k], src);
                if (k == kk) {
                    fx = x; fy = y; fz = z; fr = r; fs = sc_; fo = o; fc = c; fv = vp;
                }
            }
            bool visible = mine;
            uint32_t lid = 0u;
            const uint32_t obj = sb + static_cast<uint32_t>(kk) * 32u + src;
            if (mine) {
                const Vec3 c{fx, fy, fz};
                if (MODE == BLZ_MODE_LATE || MODE == BLZ_MODE_TEMPORAL) {
                    float4 aabb;
                    if (project_sphere(c, fr, v.zNear, v.proj0, v.proj5, aabb)) visible = occlusion(aabb, bv.pyr, v, c, fr);
                }
                if (MODE == BLZ_MODE_LATE) bv.vis[obj] = visible ? 1u : 0u;  // drawOccLate.cs.hlsl:67
            }
            bool emitted = visible && (MODE == BLZ_MODE_LATE ? fv == 0u : true);  // drawOccLate.cs.hlsl:45
            if (emitted) {
                // cullBuffers.hlsl:42-55 — last LOD in [1, lodCount) with error < threshold
                const float threshold = lod_threshold(Vec3{fx, fy, fz}, fr, fs, v.lodTarget);
                uint32_t sel = 0;
                for (uint32_t t = 1; t < fc; ++t)
                    if (__ldg(&sc.lods[fo + t].error) < threshold) sel = t;
                lid = fo + sel;
            }
            // 3. stage the emitted ones in order
            const unsigned e = __ballot_sync(0xFFFFFFFFu, emitted);
            if (emitted) stage[run + __popc(e & lanemask_lt())] = make_uint2(obj, lid);
            run += __popc(e);
        }
    }
    return run;
}

// Writes one record {objId, indexCount, 1, firstIndex, 0, 0}; pad words of 32-byte records are
// left untouched like the reference shaders leave them.
__device__ __forceinline__ void put_record(uint8_t* cmds, uint32_t stride, uint32_t slot, uint32_t objId,
                                           uint32_t indexCount, uint32_t firstIndex) {
    uint8_t* rec = cmds + static_cast<size_t>(slot) * stride;
    if (stride == BLZ_STRIDE_D3D12) {
        *reinterpret_cast<uint4*>(rec) = make_uint4(objId, indexCount, 1u, firstIndex);
        *reinterpret_cast<uint2*>(rec + 16) = make_uint2(0u, 0u);
    } else {
        uint2* w = reinterpret_cast<uint2*>(rec);
        w[0] = make_uint2(objId, indexCount);
        w[1] = make_uint2(1u, firstIndex);
        w[2] = make_uint2(0u, 0u);
    }
}

// Segmented exclusive scan of the chunk counts by one block, segments being the views: every
// thread owns a contiguous run of chunks, sums it (loads of a run are independent, so a thread pays
// about one L2 latency per eight chunks), the block scans the (sum, starts-a-segment) pairs, and
// each thread rescans its run writing offsets and, at the end of a view, that view's draw count.
template <bool SINGLE, int THREADS>
__device__ __forceinline__ void scan_chunk_counts(const PipeParams& p, uint32_t* s_sum, uint32_t* s_flag) {
    const uint32_t n = p.totalTiles;
    const uint32_t runLen = (n + THREADS - 1) / THREADS;
    const uint32_t r0 = min(n, threadIdx.x * runLen), r1 = min(n, r0 + runLen);
    uint32_t vi = 0, nextStart = n;
    if constexpr (!SINGLE) {
        if (r0 < r1) {
            vi = find_view(p.tileStart, p.viewCount, r0);
            nextStart = __ldg(p.tileStart + vi + 1);
        }
    }
    // pass 1: run sum since the last segment start inside the run
    uint32_t sum = 0, hasStart = 0;
    {
        uint32_t v = vi, ns = nextStart;
        for (uint32_t c = r0; c < r1; c += 8) {
            uint32_t x[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) x[u] = (c + u < r1) ? __ldcg(p.chunkCount + c + u) : 0u;
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const uint32_t cc = c + u;
                if (cc >= r1) break;
                if constexpr (!SINGLE) {
                    while (cc >= ns) {
                        ++v;
                        ns = __ldg(p.tileStart + v + 1);
                    }
                    if (cc == __ldg(p.tileStart + v)) {
                        sum = 0;
                        hasStart = 1;
                    }
                } else if (cc == 0) {
                    sum = 0;
                    hasStart = 1;
                }
                sum += x[u];
            }
        }
    }
    // block-wide segmented exclusive scan of (sum, hasStart): combine(a, b) = b.hasStart ? b : a + b
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    uint32_t isum = sum, iflag = hasStart;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t ps = __shfl_up_sync(0xFFFFFFFFu, isum, o);
        const uint32_t pf = __shfl_up_sync(0xFFFFFFFFu, iflag, o);
        if (lane >= static_cast<uint32_t>(o) && !iflag) {
            isum += ps;
            iflag = pf;
        }
    }
    if (lane == 31) {
        s_sum[warp] = isum;
        s_flag[warp] = iflag;
    }
    __syncthreads();
    // carry into this warp from the warps before it
    uint32_t wsum = 0;
    for (int w = 0; w < static_cast<int>(warp); ++w) wsum = s_flag[w] ? s_sum[w] : wsum + s_sum[w];
    // exclusive carry for this thread = inclusive of previous lanes (within warp) combined with wsum
    uint32_t prevSum = __shfl_up_sync(0xFFFFFFFFu, isum, 1);
    uint32_t prevFlag = __shfl_up_sync(0xFFFFFFFFu, iflag, 1);
    if (lane == 0) {
        prevSum = 0;
        prevFlag = 0;
    }
    uint32_t carry = prevFlag ? prevSum : wsum + prevSum;
    // pass 2: offsets, and each view's total at its last chunk
    {
        uint32_t v = vi, ns = nextStart, run = carry;
        for (uint32_t c = r0; c < r1; ++c) {
            if constexpr (!SINGLE) {
                while (c >= ns) {
                    ++v;
                    ns = __ldg(p.tileStart + v + 1);
                }
                if (c == __ldg(p.tileStart + v)) run = 0;
            } else if (c == 0) {
                run = 0;
            }
            const uint32_t x = __ldcg(p.chunkCount + c);
            p.chunkPrefix[c] = run;
            run += x;
            const bool lastOfView = SINGLE ? (c + 1 == n) : (c + 1 == ns);
            if (lastOfView) {
                const BatchViewDev& bv = view_of<SINGLE>(p, v);
                *bv.drawCount = run;
                if (run > bv.capacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
            }
        }
    }
}

// ------------------------------------------------------------------ decide kernel

template <int MODE, bool SINGLE, int THREADS, int OPT>
__global__ void __launch_bounds__(THREADS) cull_decide_kernel(const PipeParams p) {
    constexpr int NW = THREADS / 32;
    __shared__ uint32_t s_sum[NW], s_flag[NW];
    __shared__ int s_last;
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warpsTotal = gridDim.x * NW;
    unsigned int flags = 0u;
    for (uint32_t chunk = blockIdx.x * NW + (threadIdx.x >> 5); chunk < p.totalTiles; chunk += warpsTotal) {
        uint32_t vi = 0, first = 0;
        if constexpr (!SINGLE) {
            vi = find_view(p.tileStart, p.viewCount, chunk);
            first = __ldg(p.tileStart + vi);
        }
        const BatchViewDev& bv = view_of<SINGLE>(p, vi);
        const uint32_t base = (chunk - first) * kChunk;
        uint2* stage = p.staged + static_cast<size_t>(chunk) * kChunk;
        uint32_t total = 0;
        if (MODE == kModeRuntime) {
            switch (bv.mode) {
                case BLZ_MODE_FIRST: total = decide_chunk_warp<BLZ_MODE_FIRST, OPT>(p.sc, bv, base, stage, flags); break;
                case BLZ_MODE_LATE: total = decide_chunk_warp<BLZ_MODE_LATE, OPT>(p.sc, bv, base, stage, flags); break;
                case BLZ_MODE_TEMPORAL: total = decide_chunk_warp<BLZ_MODE_TEMPORAL, OPT>(p.sc, bv, base, stage, flags); break;
                default: total = decide_chunk_warp<BLZ_MODE_FRUSTUM, OPT>(p.sc, bv, base, stage, flags); break;
            }
        } else {
            total = decide_chunk_warp<(MODE < 0 ? 0 : MODE), OPT>(p.sc, bv, base, stage, flags);
        }
        if (lane == 0) p.chunkCount[chunk] = total;
    }
    if (flags) atomicOr(&p.scratch->status, flags);

    // the last block to finish turns the chunk counts into per-view output offsets and draw counts
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_last = (atomicAdd(p.doneBlocks, 1u) == gridDim.x - 1u) ? 1 : 0;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    scan_chunk_counts<SINGLE, THREADS>(p, s_sum, s_flag);
    if (threadIdx.x == 0) *p.doneBlocks = 0u;
}

// ------------------------------------------------------------------ scatter kernel

// Each warp copies one chunk's staged records to their final slots as full records.
template <bool SINGLE>
__global__ void __launch_bounds__(256) cull_scatter_kernel(const PipeParams p, uint32_t chunkSize) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warpsTotal = gridDim.x * (blockDim.x >> 5);
    for (uint32_t chunk = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); chunk < p.totalTiles; chunk += warpsTotal) {
        const uint32_t n = __ldg(p.chunkCount + chunk);
        if (n == 0) continue;
        const uint32_t vi = SINGLE ? 0u : find_view(p.tileStart, p.viewCount, chunk);
        const BatchViewDev& bv = view_of<SINGLE>(p, vi);
        const uint32_t base = __ldg(p.chunkPrefix + chunk);
        const uint2* stage = p.staged + static_cast<size_t>(chunk) * chunkSize;
        for (uint32_t j = lane; j < n; j += 32) {
            const uint32_t slot = base + j;
            if (slot >= bv.capacity) break;
            const uint2 rec = __ldg(stage + j);
            const uint2 lod = __ldg(reinterpret_cast<const uint2*>(p.sc.lods + rec.y));  // indexCount, firstIndex
            put_record(bv.cmds, bv.stride, slot, rec.x, lod.x, lod.y);
        }
    }
}

// ------------------------------------------------------------------ launchers

template <int MODE, bool SINGLE, int THREADS, int OPT>
static cudaError_t launch_t(const PipeParams& p, uint32_t blocksPerSm, int smCount, cudaStream_t s) {
    auto kern = cull_decide_kernel<MODE, SINGLE, THREADS, OPT>;
    int occ = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, kern, THREADS, 0);
    if (e != cudaSuccess) return e;
    if (occ < 1) occ = 1;
    const uint32_t per = blocksPerSm ? (blocksPerSm < static_cast<uint32_t>(occ) ? blocksPerSm : static_cast<uint32_t>(occ))
                                     : static_cast<uint32_t>(occ);
    uint32_t grid = per * static_cast<uint32_t>(smCount);
    const uint32_t needed = (p.totalTiles + THREADS / 32 - 1) / (THREADS / 32);  // one warp per chunk at most
    if (grid > needed) grid = needed;
    if (grid == 0) grid = 1;
    kern<<<grid, THREADS, 0, s>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint32_t sgrid = (p.totalTiles + 7) / 8;  // one warp per chunk
    const uint32_t maxGrid = 16u * static_cast<uint32_t>(smCount);
    if (sgrid > maxGrid) sgrid = maxGrid;
    if (sgrid == 0) sgrid = 1;
    cull_scatter_kernel<SINGLE><<<sgrid, 256, 0, s>>>(p, kChunk);
    return cudaGetLastError();
}

uint32_t object_tile_size() { return kChunk; }

bool single_shape_supported(uint32_t threads, uint32_t opt) {
    return (threads == 256 && (opt == 1 || opt == 2 || opt == 4)) || (threads == 128 && (opt == 2 || opt == 4)) ||
           (threads == 512 && opt == 1);
}

template <int MODE>
static cudaError_t launch_single_mode(const PipeParams& p, uint32_t threads, uint32_t opt, int smCount, cudaStream_t s) {
    if (threads == 256 && opt == 1) return launch_t<MODE, true, 256, 1>(p, 0, smCount, s);
    if (threads == 256 && opt == 4) return launch_t<MODE, true, 256, 4>(p, 0, smCount, s);
    if (threads == 128 && opt == 2) return launch_t<MODE, true, 128, 2>(p, 0, smCount, s);
    if (threads == 128 && opt == 4) return launch_t<MODE, true, 128, 4>(p, 0, smCount, s);
    if (threads == 512 && opt == 1) return launch_t<MODE, true, 512, 1>(p, 0, smCount, s);
    return launch_t<MODE, true, kObjThreads, kObjOpt>(p, 0, smCount, s);
}

cudaError_t launch_object_cull(uint32_t mode, const PipeParams& p, uint32_t threads, uint32_t opt, int smCount,
                               cudaStream_t s) {
    switch (mode) {
        case BLZ_MODE_FRUSTUM: return launch_single_mode<BLZ_MODE_FRUSTUM>(p, threads, opt, smCount, s);
        case BLZ_MODE_FIRST: return launch_single_mode<BLZ_MODE_FIRST>(p, threads, opt, smCount, s);
        case BLZ_MODE_LATE: return launch_single_mode<BLZ_MODE_LATE>(p, threads, opt, smCount, s);
        case BLZ_MODE_TEMPORAL: return launch_single_mode<BLZ_MODE_TEMPORAL>(p, threads, opt, smCount, s);
        default: return cudaErrorInvalidValue;
    }
}

bool batch_shape_supported(uint32_t threads, uint32_t opt) {
    if (!(threads == 128 || threads == 256 || threads == 512)) return false;
    if (!(opt == 1 || opt == 2 || opt == 4 || opt == 8)) return false;
    return threads * opt <= 1024;
}

cudaError_t launch_batch_cull(const PipeParams& p, uint32_t threads, uint32_t opt, uint32_t blocksPerSm, int smCount,
                              cudaStream_t s) {
#define BLZ_BATCH_CASE(T, O) \
    if (threads == T && opt == O) return launch_t<kModeRuntime, false, T, O>(p, blocksPerSm, smCount, s);
    BLZ_BATCH_CASE(128, 1) BLZ_BATCH_CASE(128, 2) BLZ_BATCH_CASE(128, 4) BLZ_BATCH_CASE(128, 8)
    BLZ_BATCH_CASE(256, 1) BLZ_BATCH_CASE(256, 2) BLZ_BATCH_CASE(256, 4)
    BLZ_BATCH_CASE(512, 1) BLZ_BATCH_CASE(512, 2)
#undef BLZ_BATCH_CASE
    return cudaErrorInvalidValue;
}

}  // namespace blz
