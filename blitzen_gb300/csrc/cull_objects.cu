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

// Per-block shared memory of the decide kernel: the queue of frustum survivors of a chunk (their
// view-space spheres and LOD ranges) and the per-object results the queue work hands back.
template <int CHUNK>
struct DecideSmem {
    float qx[CHUNK], qy[CHUNK], qz[CHUNK], qr[CHUNK], qs[CHUNK];
    uint32_t qidx[CHUNK];      // object index in the chunk | want-emit flag in bit 31
    uint32_t qlodOff[CHUNK];   // the surface's LOD range
    uint32_t qlodCnt[CHUNK];
    uint32_t result[CHUNK];    // per object: lodId if emitted, kNotEmitted otherwise
    uint8_t visible[CHUNK];    // per object: final visibility (LATE rewrites the buffer with it)
    uint32_t queueLen;
};

constexpr uint32_t kNotEmitted = 0xFFFFFFFFu;

// Decisions of one chunk in three phases:
//   A  every thread loads its OPT objects (render object, then transform — all reads issued before
//      any arithmetic) and runs the frustum test; survivors are appended to a shared queue with one
//      shared atomic per warp and k;
//   B  the block walks the queue — the sphere projection, Hi-Z test (LATE/TEMPORAL) and LOD
//      selection run on dense lanes instead of on every lane of every warp that has one survivor;
//   C  every thread reads its objects' results back in object order (the caller ranks them).
template <int MODE, int THREADS, int OPT>
__device__ __forceinline__ void decide_chunk(const SceneTables& sc, const BatchViewDev& bv, uint32_t base,
                                             DecideSmem<THREADS * OPT>& sm, bool (&emit)[OPT], uint32_t (&lodId)[OPT],
                                             unsigned int& flags) {
    const uint32_t count = bv.count;
    const uint32_t lane = threadIdx.x & 31u;
    if (threadIdx.x == 0) sm.queueLen = 0u;
    uint32_t visPrev[OPT];
    bool act[OPT];
#pragma unroll
    for (int k = 0; k < OPT; ++k) {
        const uint32_t i = base + k * THREADS + threadIdx.x;
        act[k] = i < count;
        visPrev[k] = 1u;
        if (MODE == BLZ_MODE_FIRST && act[k]) visPrev[k] = __ldg(bv.vis + i);
        if (MODE == BLZ_MODE_LATE && act[k]) visPrev[k] = bv.vis[i];  // rewritten below: coherent load
    }
    if (MODE == BLZ_MODE_FIRST) {
#pragma unroll
        for (int k = 0; k < OPT; ++k) act[k] = act[k] && visPrev[k] != 0u;  // drawOccFirst.cs.hlsl:22-25
    }
    uint2 ro[OPT];
#pragma unroll
    for (int k = 0; k < OPT; ++k) {
        ro[k] = make_uint2(0u, 0u);
        if (act[k]) ro[k] = __ldg(reinterpret_cast<const uint2*>(bv.objects) + base + k * THREADS + threadIdx.x);
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
    __syncthreads();  // queueLen reset is visible
    const ViewConsts v = load_view(bv.view);
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < OPT; ++k) {
        const uint32_t idx = k * THREADS + threadIdx.x;
        bool inFrustum = false;
        Vec3 c{0.f, 0.f, 0.f};
        float r = 0.f;
        uint4 s1 = make_uint4(0u, 0u, 0u, 0u);
        if (ok[k]) {
            const float4* sp = reinterpret_cast<const float4*>(sc.surfaces + ro[k].y);
            const float4 sph = __ldg(sp);
            s1 = __ldg(reinterpret_cast<const uint4*>(sp + 1));  // materialId, lodOffset, lodCount, vertexOffset
            if (s1.y < sc.lodCount && s1.z <= sc.lodCount - s1.y) {
                c = view_transform(v.rows, model_to_world(Vec3{sph.x, sph.y, sph.z}, ps[k], q[k]));
                r = BLZ_FM(sph.w, ps[k].w);
                inFrustum = frustum_check(c, r, v);
            } else {
                flags |= BLZ_FLAG_BAD_INDEX;
            }
        } else if (act[k]) {
            flags |= BLZ_FLAG_BAD_INDEX;
        }
        sm.visible[idx] = 0;
        sm.result[idx] = kNotEmitted;
        // append the survivors: one shared atomic per warp
        const unsigned b = __ballot_sync(0xFFFFFFFFu, inFrustum);
        uint32_t at = 0;
        if (lane == 0 && b) at = atomicAdd(&sm.queueLen, static_cast<uint32_t>(__popc(b)));
        at = __shfl_sync(0xFFFFFFFFu, at, 0) + __popc(b & lt);
        if (inFrustum) {
            const bool want = (MODE == BLZ_MODE_LATE) ? (visPrev[k] == 0u) : true;
            sm.qx[at] = c.x;
            sm.qy[at] = c.y;
            sm.qz[at] = c.z;
            sm.qr[at] = r;
            sm.qs[at] = ps[k].w;
            sm.qidx[at] = idx | (want ? 0x80000000u : 0u);
            sm.qlodOff[at] = s1.y;
            sm.qlodCnt[at] = s1.z;
        }
    }
    __syncthreads();
    // B: dense work over the survivors
    const uint32_t n = sm.queueLen;
    for (uint32_t j = threadIdx.x; j < n; j += THREADS) {
        const Vec3 c{sm.qx[j], sm.qy[j], sm.qz[j]};
        const float r = sm.qr[j];
        const uint32_t id = sm.qidx[j];
        bool visible = true;
        if (MODE == BLZ_MODE_LATE || MODE == BLZ_MODE_TEMPORAL) {
            float4 aabb;
            if (project_sphere(c, r, v.zNear, v.proj0, v.proj5, aabb)) visible = occlusion(aabb, bv.pyr, v, c, r);
        }
        const uint32_t idx = id & 0x7FFFFFFFu;
        sm.visible[idx] = visible ? 1 : 0;
        if (visible && (id & 0x80000000u)) {
            // cullBuffers.hlsl:42-55 — last LOD in [1, lodCount) with error < threshold
            const uint32_t lodOff = sm.qlodOff[j], lodCnt = sm.qlodCnt[j];
            const float threshold = lod_threshold(c, r, sm.qs[j], v.lodTarget);
            uint32_t sel = 0;
            for (uint32_t t = 1; t < lodCnt; ++t)
                if (__ldg(&sc.lods[lodOff + t].error) < threshold) sel = t;
            sm.result[idx] = lodOff + sel;
        }
    }
    __syncthreads();
    // C: results back to the owning threads, in object order
#pragma unroll
    for (int k = 0; k < OPT; ++k) {
        const uint32_t idx = k * THREADS + threadIdx.x;
        const uint32_t res = sm.result[idx];
        emit[k] = res != kNotEmitted;
        lodId[k] = res;
        if (MODE == BLZ_MODE_LATE && act[k]) bv.vis[base + idx] = sm.visible[idx];  // drawOccLate.cs.hlsl:67
    }
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

// Block-wide stable ranking of OPT ballots per thread in k-major order (object index order).
// Returns the block's count (valid in warp 0); s_off[k * NW + w] becomes the exclusive offset of
// (k, warp w) once the caller has synchronised.
template <int THREADS, int OPT>
__device__ __forceinline__ uint32_t block_rank(const bool (&emit)[OPT], uint32_t (&lrank)[OPT], uint32_t* s_off) {
    constexpr int NW = THREADS / 32;
    constexpr int M = OPT * NW;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    const uint32_t lt = lanemask_lt();
#pragma unroll
    for (int k = 0; k < OPT; ++k) {
        const unsigned b = __ballot_sync(0xFFFFFFFFu, emit[k]);
        lrank[k] = __popc(b & lt);
        if (lane == 0) s_off[k * NW + warp] = __popc(b);
    }
    __syncthreads();
    uint32_t total = 0;
    if (warp == 0) {
        constexpr int E = (M + 31) / 32;
        uint32_t vals[E];
        uint32_t sum = 0;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int idx = lane * E + e;
            vals[e] = idx < M ? s_off[idx] : 0u;
            sum += vals[e];
        }
        uint32_t incl = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += n;
        }
        uint32_t run = incl - sum;
#pragma unroll
        for (int e = 0; e < E; ++e) {
            const int idx = lane * E + e;
            if (idx < M) s_off[idx] = run;
            run += vals[e];
        }
        total = __shfl_sync(0xFFFFFFFFu, incl, 31);
    }
    return total;
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
    constexpr uint32_t CHUNK = THREADS * OPT;
    __shared__ uint32_t s_off[OPT * NW];
    __shared__ uint32_t s_sum[NW], s_flag[NW];
    __shared__ int s_last;
    __shared__ DecideSmem<CHUNK> s_dec;
    const uint32_t warp = threadIdx.x >> 5;
    unsigned int flags = 0u;
    for (uint32_t chunk = blockIdx.x; chunk < p.totalTiles; chunk += gridDim.x) {
        uint32_t vi = 0, first = 0;
        if constexpr (!SINGLE) {
            vi = find_view(p.tileStart, p.viewCount, chunk);
            first = __ldg(p.tileStart + vi);
        }
        const BatchViewDev& bv = view_of<SINGLE>(p, vi);
        const uint32_t base = (chunk - first) * CHUNK;
        bool emit[OPT];
        uint32_t lod[OPT];
        if (MODE == kModeRuntime) {
            switch (bv.mode) {
                case BLZ_MODE_FIRST: decide_chunk<BLZ_MODE_FIRST, THREADS, OPT>(p.sc, bv, base, s_dec, emit, lod, flags); break;
                case BLZ_MODE_LATE: decide_chunk<BLZ_MODE_LATE, THREADS, OPT>(p.sc, bv, base, s_dec, emit, lod, flags); break;
                case BLZ_MODE_TEMPORAL: decide_chunk<BLZ_MODE_TEMPORAL, THREADS, OPT>(p.sc, bv, base, s_dec, emit, lod, flags); break;
                default: decide_chunk<BLZ_MODE_FRUSTUM, THREADS, OPT>(p.sc, bv, base, s_dec, emit, lod, flags); break;
            }
        } else {
            decide_chunk<(MODE < 0 ? 0 : MODE), THREADS, OPT>(p.sc, bv, base, s_dec, emit, lod, flags);
        }
        uint32_t lrank[OPT];
        const uint32_t total = block_rank<THREADS, OPT>(emit, lrank, s_off);
        if (threadIdx.x == 0) p.chunkCount[chunk] = total;
        __syncthreads();  // warp 0's offsets are visible to every warp
        uint2* stage = p.staged + static_cast<size_t>(chunk) * CHUNK;
#pragma unroll
        for (int k = 0; k < OPT; ++k)
            if (emit[k]) stage[s_off[k * NW + warp] + lrank[k]] = make_uint2(base + k * THREADS + threadIdx.x, lod[k]);
        __syncthreads();  // s_off is rewritten by the next chunk
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
    if (grid > p.totalTiles) grid = p.totalTiles;
    if (grid == 0) grid = 1;
    kern<<<grid, THREADS, 0, s>>>(p);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    uint32_t sgrid = (p.totalTiles + 7) / 8;  // one warp per chunk
    const uint32_t maxGrid = 16u * static_cast<uint32_t>(smCount);
    if (sgrid > maxGrid) sgrid = maxGrid;
    if (sgrid == 0) sgrid = 1;
    cull_scatter_kernel<SINGLE><<<sgrid, 256, 0, s>>>(p, THREADS * OPT);
    return cudaGetLastError();
}

uint32_t object_tile_size() { return kObjThreads * kObjOpt; }

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
