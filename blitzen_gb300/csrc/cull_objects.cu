// cull_objects.cu — per-object cull kernels: frustum, occlusion pass 1 / pass 2, temporal
// occlusion, for one view or many views in one launch.
//
// Two kernels per launch, no block ever waiting on another:
//   decide   a streaming grid of warps, each deciding contiguous chunks of a view's render objects
//            (single views: one chunk per resident warp, assigned by warp index; batches: 512-object
//            chunks of all views, taken from a work counter), staging the emitted ones compacted in
//            object order — (objectId, lodId), 8 bytes — in the chunk's slice of a scratch buffer,
//            with the chunk's count;
//   scatter  one block per 32 chunks: the block finds its chunks' output offsets from the counts
//            (no grid-wide scan), copies the staged records to their final slots as full indirect
//            records, and the owner of each view's last chunk writes the view's draw count.
// The scratch traffic is 16 bytes per emitted object, against 40-48 bytes read per object.
//
// Reference passes (paths inside the Blitzen project):
//   FRUSTUM   TransparentDrawCull.comp.glsl:13-65, drawCull.cs.hlsl:10-52
//   FIRST     InitialDrawCull.comp.glsl:12-59,     drawOccFirst.cs.hlsl:13-58
//   LATE      LateDrawCull.comp.glsl:13-72,        drawOccLate.cs.hlsl:13-67
//   TEMPORAL  drawOccTemporal.hlsl:13-64
#include "blz_device.cuh"
#include "pyramid_tile.cuh"
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

// The same for a chunk index c that is equal on every lane of the warp: a 32-ary search, one round
// of loads per factor of 32 views instead of one dependent load per halving.
__device__ __forceinline__ uint32_t find_view_warp(const uint32_t* tileStart, uint32_t nViews, uint32_t c) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t lo = 0, n = nViews;  // the view is in [lo, lo + n), and tileStart[lo] <= c
    while (n > 1u) {
        const uint32_t step = (n + 31u) >> 5;
        const uint32_t cand = lo + lane * step;
        const bool le = cand < lo + n && __ldg(tileStart + cand) <= c;
        const uint32_t k = 31u - static_cast<uint32_t>(__clz(static_cast<int>(__ballot_sync(0xFFFFFFFFu, le))));
        const uint32_t end = lo + n;
        lo += k * step;
        n = min(step, end - lo);
    }
    return lo;
}

// ------------------------------------------------------------------ decisions

constexpr uint32_t kChunk = 512;  // objects per chunk of batched views (single views size theirs)
constexpr uint32_t kInstGroup = 32;  // chunks per group of the instanced counting sort, one warp each

// A frustum survivor waiting for the dense stage (32 bytes, two 16-byte shared-memory words).
struct Survivor {
    uint32_t obj;      // object index within the view; bit 31: visible last frame (LATE)
    float cx, cy, cz;  // view-space sphere centre
    float r, scale;
    uint32_t lodOff, lodCnt;
};
constexpr uint32_t kRing = 64;  // per-warp survivor ring: under 32 waiting plus one 32-object slice

// Both passes of a frame decided in one sweep, with the pyramid built before the launch or inside it.
__host__ __device__ constexpr bool fused_mode(int m) { return m == kModeFrameFused || m == kModeFramePyr; }

// A warp's wait for the pyramid its own launch builds (kModeFramePyr): the whole warp polls the
// ready flag with acquire semantics (one load serves every lane, so all see the same value), at
// most `limit` times; then it raises BLZ_FLAG_TIMEOUT and goes on with whatever the pyramid holds.
__device__ __forceinline__ void wait_pyramid(const unsigned int* ready, uint32_t limit, unsigned int& flags) {
    for (uint32_t polls = 0; ld_acquire_gpu(ready) == 0u;) {
        if (++polls >= limit) {
            flags |= BLZ_FLAG_TIMEOUT;
            break;
        }
        __nanosleep(128);
    }
    __syncwarp();
}

// The lanes of the warp whose record has the same LOD id as this lane's (ids below 2^bits): one
// ballot per bit of the id, each lane keeping the lanes that agree with it on every bit. Votes, not
// a match instruction, so the ranking stays off the shared-memory pipe. Lanes without a record
// (valid false) get a mask their callers do not use.
__device__ __forceinline__ unsigned same_lod_lanes(uint32_t b, uint32_t bits, bool valid) {
    unsigned m = __ballot_sync(0xFFFFFFFFu, valid);
    for (uint32_t k = 0; k < bits; ++k) {
        const bool bit = ((b >> k) & 1u) != 0u;
        const unsigned v = __ballot_sync(0xFFFFFFFFu, bit);
        m &= bit ? v : ~v;
    }
    return m;
}

// Dense stage over one survivor per lane (lanes with `mine`), in object order: the sphere
// projection and Hi-Z test (LATE/TEMPORAL), LATE's visibility write, LOD selection of the emitted
// ones, and their staging as (objectId, lodId) after the `run` already staged for the chunk.
// A survivor is the two words of a Survivor: a = {obj | tags, centre}, b = {r, scale, lodOff, lodCnt}.
// kModeFrame1 emits the survivors visible last frame (its pass-1 records) and tests no pyramid.
// The fused modes stage pass 2's records in `stage` and pass 1's in `stage1` (run1).
template <int MODE>
__device__ __forceinline__ void dense_entry(const SceneTables& sc, const BatchViewDev& bv, const ViewConsts& v, uint4 a,
                                            uint4 b, bool mine, uint2* stage, uint32_t& run, uint2* stage1 = nullptr,
                                            uint32_t* run1 = nullptr, uint32_t* hist = nullptr) {
    constexpr bool FUSED = fused_mode(MODE);
    constexpr bool REWRITE = MODE == BLZ_MODE_LATE || FUSED;  // pass 2's visibility rewrite
    const uint32_t obj = a.x & 0x3FFFFFFFu;  // LATE: bit 31 previous visibility != 0, bit 30 == 1
    const Vec3 c{__uint_as_float(a.y), __uint_as_float(a.z), __uint_as_float(a.w)};
    const float r = __uint_as_float(b.x), scale = __uint_as_float(b.y);
    const bool wasNonZero = (a.x >> 31) != 0u;
    bool visible = mine;
    if (mine) {
        if (MODE == BLZ_MODE_LATE || MODE == BLZ_MODE_TEMPORAL || FUSED) {
            float4 aabb;
            if (project_sphere(c, r, v.zNear, v.proj0, v.proj5, aabb))
                visible = occlusion<MODE == kModeFramePyr>(aabb, bv.pyr, v, c, r);
        }
        if (REWRITE) {
            // drawOccLate.cs.hlsl:67, storing only a value that changes
            const bool wasOne = ((a.x >> 30) & 1u) != 0u;
            if (visible ? !wasOne : wasNonZero) bv.vis[obj] = visible ? 1u : 0u;
        }
    }
    // drawOccLate.cs.hlsl:45; a kept frame's pass 1 emits what drawOccFirst.cs.hlsl:22-25 admits
    const bool emitted = visible && (REWRITE ? !wasNonZero : (MODE == kModeFrame1 ? wasNonZero : true));
    // the fused sweep's pass 1: every survivor visible last frame (its frustum test passed)
    const bool emitted1 = FUSED && mine && wasNonZero;
    uint32_t lid = 0u;
    if (emitted || emitted1) {
        // cullBuffers.hlsl:42-55 — last LOD in [1, lodCount) with error < threshold
        const float threshold = lod_threshold(c, r, scale, v.lodTarget);
        uint32_t sel = 0;
        for (uint32_t t = 1; t < b.w; ++t)
            if (__ldg(&sc.lods[b.z + t].error) < threshold) sel = t;
        lid = b.z + sel;
    }
    const unsigned e = __ballot_sync(0xFFFFFFFFu, emitted);
    if (emitted) stage[run + __popc(e & lanemask_lt())] = make_uint2(obj, lid);
    run += __popc(e);
    if constexpr (MODE == kModeInstanced) {
        // the group's histogram row (hist = row of this chunk's group): one add per distinct LOD
        const uint32_t idBits = sc.lodCount > 1u ? 32u - static_cast<uint32_t>(__clz(static_cast<int>(sc.lodCount - 1u))) : 0u;
        const unsigned peers = same_lod_lanes(lid, idBits, emitted);
        if (emitted && (peers & lanemask_lt()) == 0u) atomicAdd(hist + lid, static_cast<uint32_t>(__popc(peers)));
    }
    if constexpr (FUSED) {
        const unsigned e1 = __ballot_sync(0xFFFFFFFFu, emitted1);
        if (emitted1) stage1[*run1 + __popc(e1 & lanemask_lt())] = make_uint2(obj, lid);
        *run1 += __popc(e1);
    }
}

// dense_entry over n <= 32 queued survivors starting at ring index head. kModeFrame1 also appends
// them to the chunk's kept survivors (keep[kept ...], 32 bytes each, coalesced).
template <int MODE>
__device__ __forceinline__ void dense_round(const SceneTables& sc, const BatchViewDev& bv, const ViewConsts& v,
                                            const Survivor* ring, uint32_t head, uint32_t n, uint2* stage,
                                            uint32_t& run, uint4* keep, uint32_t& kept, uint2* stage1, uint32_t* run1,
                                            uint32_t* hist = nullptr) {
    const uint32_t lane = threadIdx.x & 31u;
    const bool mine = lane < n;
    uint4 a = make_uint4(0u, 0u, 0u, 0u), b = make_uint4(0u, 0u, 0u, 0u);
    if (mine) {
        const uint4* e = reinterpret_cast<const uint4*>(ring + ((head + lane) & (kRing - 1u)));
        a = e[0];
        b = e[1];
        if constexpr (MODE == kModeFrame1) {
            keep[2u * (kept + lane)] = a;
            keep[2u * (kept + lane) + 1u] = b;
        }
    }
    if constexpr (MODE == kModeFrame1) kept += n;
    dense_entry<MODE>(sc, bv, v, a, b, mine, stage, run, stage1, run1, hist);
}

// The fields of the surface table the frustum stage reads (bounding sphere; LOD offset and count),
// copied into shared memory by each block when the table is small enough; null pointers: read the
// table in global memory.
struct SurfaceCache {
    const float4* sphere;
    const uint2* lod;
};

// One warp decides the objects [base, limit) of a view, 32 * OPT at a time (object
// sb + k * 32 + lane for k < OPT, so lanes ascend within each 32-object slice):
//   1  every lane loads its OPT render objects (fetched one step ahead) and their transforms and
//      surfaces, and runs the frustum test — without branches: an object that is out of range,
//      not active in this pass or has a bad id reads the tables' first rows and is masked out.
//      Pass 1 (single views) first packs the objects visible last frame into a candidate ring,
//      so the frustum stage runs on full lanes there too;
//   2  each slice's survivors are appended, in object order, to the warp's ring in shared memory;
//      whenever 32 are waiting they go through the dense stage on full lanes, so the costly part
//      (projection, Hi-Z, LOD) never runs on a lane without an object;
//   3  the dense stage stages the emitted ones in order; the rest drains at the end.
// Returns the number of records staged. No block barrier: warps never wait for one another.
template <int MODE, bool SINGLE, int OPT>
__device__ __forceinline__ uint32_t decide_run_warp(const SceneTables& sc, const BatchViewDev& bv, uint32_t base,
                                                    uint32_t limit, uint2* stage, Survivor* ring, uint4* cand,
                                                    const SurfaceCache& surf, unsigned int& flags, uint4* keep,
                                                    uint32_t& kept, uint2* stage1 = nullptr, uint32_t* run1 = nullptr,
                                                    const unsigned int* ready = nullptr, uint32_t spinLimit = 0u,
                                                    uint32_t* hist = nullptr) {
    constexpr uint32_t STEP = 32u * OPT;
    constexpr bool PACK = (MODE == BLZ_MODE_FIRST) && SINGLE;  // candidate ring of 2 * STEP entries
    // Single-view pass 2 walks its chunk from the last object down: pass 1 walked the same chunk
    // upwards just before (with only the pyramid build between), so the lines it touched last are
    // the ones still in L2. Records are then staged in descending order; the scatter writes each
    // chunk's records back to front. Slot i of the walk is object `walk(i)`; past the end it is
    // kNoObject, never active.
    constexpr bool DOWN = (MODE == BLZ_MODE_LATE) && SINGLE;
    constexpr uint32_t kNoObject = 0xFFFFFFFFu;
    auto walk = [&](uint32_t i) -> uint32_t { return i < limit ? (DOWN ? base + limit - 1u - i : i) : kNoObject; };
    const uint32_t lane = threadIdx.x & 31u;
    if (sc.transformCount == 0u || sc.surfaceCount == 0u) {
        // nothing can be looked up: every object of the pass has a bad id and none is visible
        for (uint32_t i = base + lane; i < limit; i += 32u) {
            const bool act = MODE != BLZ_MODE_FIRST || __ldg(bv.vis + i) != 0u;
            if (act) flags |= BLZ_FLAG_BAD_INDEX;
            if (MODE == BLZ_MODE_LATE || MODE == kModeFrame1 || fused_mode(MODE)) bv.vis[i] = 0u;
        }
        return 0u;
    }
    const ViewConsts v = load_view(bv.view);
    uint32_t run = 0, head = 0, tail = 0;
    // kModeFramePyr: the pyramid is waited for once, before the warp's first dense round
    bool pyrSeen = MODE != kModeFramePyr;
    auto dense = [&](uint32_t n) {
        if (!pyrSeen) {
            wait_pyramid(ready, spinLimit, flags);
            pyrSeen = true;
        }
        dense_round<MODE>(sc, bv, v, ring, head, n, stage, run, keep, kept, stage1, run1, hist);
    };

    // frustum stage over OPT slices: obj[k] the object index, ro[k] its render object, vis[k] the
    // object's visibility word (LATE: as read; the object is active when in range) or, in the other
    // passes, non-zero when the object is active
    float4 ps[OPT], q[OPT], sph[OPT];
    uint2 lod[OPT];
    bool ok[OPT];
    // LATE and kModeFrame1 test every object (vis[k] holds its visibility word), the others the
    // objects with vis[k] != 0
    constexpr bool ALL = MODE == BLZ_MODE_LATE || MODE == kModeFrame1 || fused_mode(MODE);
    auto active = [&](uint32_t obj, uint32_t vis) -> bool { return ALL ? obj < limit : vis != 0u; };
    auto gather = [&](const uint32_t (&obj)[OPT], const uint2 (&ro)[OPT], const uint32_t (&vis)[OPT]) {
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            ok[k] = active(obj[k], vis[k]) && ro[k].x < sc.transformCount && ro[k].y < sc.surfaceCount;
            const uint32_t tid = ok[k] ? ro[k].x : 0u, sid = ok[k] ? ro[k].y : 0u;
            if constexpr (!SINGLE) {
                if (bv.dynT != nullptr && tid < bv.dynCount) {  // the view's own rows first
                    ldg_transform(bv.dynT + tid, ps[k], q[k]);
                } else {
                    load_transform(sc, tid, ps[k], q[k]);
                }
            } else {
                load_transform(sc, tid, ps[k], q[k]);
            }
            if (surf.sphere != nullptr) {
                sph[k] = surf.sphere[sid];
                lod[k] = surf.lod[sid];
            } else {
                const float4* sp = reinterpret_cast<const float4*>(sc.surfaces + sid);
                sph[k] = __ldg(sp);
                const uint4 s1 = __ldg(reinterpret_cast<const uint4*>(sp + 1));  // materialId, lodOffset, lodCount, vertexOffset
                lod[k] = make_uint2(s1.y, s1.z);
            }
        }
    };
    auto test = [&](const uint32_t (&obj)[OPT], const uint32_t (&vis)[OPT]) {
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            const bool act = active(obj[k], vis[k]);
            const bool lodOk = lod[k].x < sc.lodCount && lod[k].y <= sc.lodCount - lod[k].x;
            const bool good = ok[k] && lodOk;
            if (act && !good) flags |= BLZ_FLAG_BAD_INDEX;
            const Vec3 c = view_transform(v.rows, model_to_world(Vec3{sph[k].x, sph[k].y, sph[k].z}, ps[k], q[k]));
            const float r = BLZ_FM(sph[k].w, ps[k].w);
            const bool inFrustum = good && frustum_check(c, r, v);
            // drawOccLate.cs.hlsl:67, storing only a value that changes
            if (ALL && act && !inFrustum && vis[k] != 0u) bv.vis[obj[k]] = 0u;
            const unsigned m = __ballot_sync(0xFFFFFFFFu, inFrustum);
            if (inFrustum) {
                uint4* e = reinterpret_cast<uint4*>(ring + ((tail + __popc(m & lanemask_lt())) & (kRing - 1u)));
                const uint32_t tag = !ALL ? 0u : (vis[k] != 0u ? 0x80000000u : 0u) | (vis[k] == 1u ? 0x40000000u : 0u);
                e[0] = make_uint4(obj[k] | tag, __float_as_uint(c.x), __float_as_uint(c.y), __float_as_uint(c.z));
                e[1] = make_uint4(__float_as_uint(r), __float_as_uint(ps[k].w), lod[k].x, lod[k].y);
            }
            tail += __popc(m);
            if (tail - head >= 32u) {
                __syncwarp();
                dense(32u);
                head += 32u;
                __syncwarp();
            }
        }
    };

    uint2 nro[OPT];
    uint32_t nvis[OPT];
    auto prefetch = [&](uint32_t at) {
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            const uint32_t i = walk(at + k * 32u + lane);
            const bool in = i != kNoObject;
            nro[k] = in ? __ldg(reinterpret_cast<const uint2*>(bv.objects) + i) : make_uint2(0u, 0u);
            nvis[k] = in ? 1u : 0u;
            if (MODE == BLZ_MODE_FIRST && in) nvis[k] = __ldg(bv.vis + i);
            if (ALL) nvis[k] = in ? bv.vis[i] : 0u;  // rewritten later by this warp: coherent load
        }
    };
    // candidates packed by pass 1, taken STEP at a time (or the rest, at the end)
    uint32_t ahead = 0, atail = 0;
    auto take_candidates = [&](uint32_t n) {
        uint2 ro[OPT];
        uint32_t obj[OPT], vis[OPT];
        __syncwarp();
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            const uint32_t j = k * 32u + lane;
            const uint4 e = cand[(ahead + j) & (2u * STEP - 1u)];
            const bool in = j < n;
            obj[k] = e.x;
            ro[k] = make_uint2(e.y, e.z);
            vis[k] = in ? 1u : 0u;
        }
        __syncwarp();
        ahead += n;
        gather(obj, ro, vis);
        test(obj, vis);
    };

    if (base < limit) prefetch(base);
    for (uint32_t sb = base; sb < limit; sb += STEP) {
        uint2 ro[OPT];
        uint32_t obj[OPT], vis[OPT];
#pragma unroll
        for (int k = 0; k < OPT; ++k) {
            ro[k] = nro[k];
            vis[k] = nvis[k];  // pass 1: active when visible last frame (drawOccFirst.cs.hlsl:22-25)
            obj[k] = DOWN ? walk(sb + k * 32u + lane) : sb + k * 32u + lane;
        }
        if constexpr (PACK) {
            if (sb + STEP < limit) prefetch(sb + STEP);
#pragma unroll
            for (int k = 0; k < OPT; ++k) {
                const bool act = vis[k] != 0u;
                const unsigned m = __ballot_sync(0xFFFFFFFFu, act);
                if (act) cand[(atail + __popc(m & lanemask_lt())) & (2u * STEP - 1u)] = make_uint4(obj[k], ro[k].x, ro[k].y, 0u);
                atail += __popc(m);
            }
            if (atail - ahead >= STEP) take_candidates(STEP);
        } else {
            gather(obj, ro, vis);
            if (sb + STEP < limit) prefetch(sb + STEP);
            test(obj, vis);
        }
    }
    if constexpr (PACK) {
        if (atail != ahead) take_candidates(atail - ahead);
    }
    if (tail != head) {
        __syncwarp();
        dense(tail - head);
        __syncwarp();
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

// ------------------------------------------------------------------ decide kernel

// Shared memory of the decide kernels: one survivor ring per warp, pass 1's candidate rings, and the
// surface table in what static shared memory is left (48 KB per block).
template <int MODE, bool SINGLE, int THREADS, int OPT>
struct DecideSmem {
    static constexpr int NW = THREADS / 32;
    static constexpr bool PACK = (MODE == BLZ_MODE_FIRST) && SINGLE;
    static constexpr size_t kUsed = sizeof(Survivor) * kRing * NW + (PACK ? sizeof(uint4) * NW * 2 * 32 * OPT : 0);
    static constexpr size_t kLeft = kUsed + 1024 < 48 * 1024 ? 48 * 1024 - 1024 - kUsed : 0;
    static constexpr uint32_t kSurf = kLeft >= 512 * 24 ? 512u : (kLeft >= 256 * 24 ? 256u : (kLeft >= 64 * 24 ? 64u : 1u));
    Survivor ring[NW][kRing];
    uint4 cand[PACK ? NW : 1][PACK ? 2 * 32 * OPT : 1];
    float4 sphere[kSurf];
    uint2 lod[kSurf];
};

// The decide kernels' body: each warp decides chunks of a view (decide_run_warp) and records each
// chunk's count. kModeFramePyr passes the context's pyramid-ready flag and its wait limit.
template <int MODE, bool SINGLE, int THREADS, int OPT>
__device__ __forceinline__ void decide_body(const PipeParams& p, DecideSmem<MODE, SINGLE, THREADS, OPT>& sm,
                                            const unsigned int* ready = nullptr, uint32_t spinLimit = 0u) {
    using Smem = DecideSmem<MODE, SINGLE, THREADS, OPT>;
    constexpr int NW = Smem::NW;
    constexpr bool PACK = Smem::PACK;
    constexpr uint32_t kSurf = Smem::kSurf;
    SurfaceCache surf{nullptr, nullptr};
    if (kSurf > 1u && p.sc.surfaceCount <= kSurf) {
        for (uint32_t i = threadIdx.x; i < p.sc.surfaceCount; i += THREADS) {
            const float4* sp = reinterpret_cast<const float4*>(p.sc.surfaces + i);
            sm.sphere[i] = __ldg(sp);
            const uint4 s1 = __ldg(reinterpret_cast<const uint4*>(sp + 1));
            sm.lod[i] = make_uint2(s1.y, s1.z);
        }
        __syncthreads();
        surf = SurfaceCache{sm.sphere, sm.lod};
    }
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t warpsTotal = gridDim.x * NW;
    const uint32_t chunkSize = p.chunkSize;
    unsigned int flags = 0u;
    // every warp starts on the chunk of its index; later chunks come from the work counter when
    // there is one (a warp that finishes early takes the next, so warps finish together), else by
    // a stride of the grid's warp count
    auto next_chunk = [&](uint32_t cur) -> uint32_t {
        if (p.workCounter == nullptr) return cur + warpsTotal;
        uint32_t c = 0;
        if (lane == 0) c = warpsTotal + atomicAdd(p.workCounter, 1u);
        return __shfl_sync(0xFFFFFFFFu, c, 0);
    };
    uint32_t chunk = blockIdx.x * NW + warp;
    while (chunk < p.totalTiles) {
        const uint32_t next = next_chunk(chunk);  // asked now, used after this chunk
        uint32_t vi = 0, first = 0;
        if constexpr (!SINGLE) {
            vi = find_view_warp(p.tileStart, p.viewCount, chunk);
            first = __ldg(p.tileStart + vi);
        }
        const BatchViewDev& bv = view_of<SINGLE>(p, vi);
        const uint32_t base = (chunk - first) * chunkSize;
        const uint32_t limit = min(base + chunkSize, bv.count);
        uint2* stage = p.staged + static_cast<size_t>(chunk) * chunkSize;
        Survivor* ring = sm.ring[warp];
        uint4* cand = sm.cand[PACK ? warp : 0];
        uint32_t total = 0, kept = 0, total1 = 0;
        uint4* keep = nullptr;
        if constexpr (MODE == kModeFrame1) keep = static_cast<uint4*>(p.keep) + 2u * static_cast<size_t>(chunk) * chunkSize;
        uint2* stage1 = nullptr;
        if constexpr (fused_mode(MODE)) stage1 = p.staged2 + static_cast<size_t>(chunk) * chunkSize;
        if (MODE == kModeRuntime) {
            switch (bv.mode) {
                case BLZ_MODE_FIRST: total = decide_run_warp<BLZ_MODE_FIRST, SINGLE, OPT>(p.sc, bv, base, limit, stage, ring, cand, surf, flags, keep, kept); break;
                case BLZ_MODE_LATE: total = decide_run_warp<BLZ_MODE_LATE, SINGLE, OPT>(p.sc, bv, base, limit, stage, ring, cand, surf, flags, keep, kept); break;
                case BLZ_MODE_TEMPORAL: total = decide_run_warp<BLZ_MODE_TEMPORAL, SINGLE, OPT>(p.sc, bv, base, limit, stage, ring, cand, surf, flags, keep, kept); break;
                default: total = decide_run_warp<BLZ_MODE_FRUSTUM, SINGLE, OPT>(p.sc, bv, base, limit, stage, ring, cand, surf, flags, keep, kept); break;
            }
        } else {
            uint32_t* hist = nullptr;
            if constexpr (MODE == kModeInstanced) hist = p.instHist + static_cast<size_t>(chunk / kInstGroup) * p.instLods;
            total = decide_run_warp<(MODE < 0 ? 0 : MODE), SINGLE, OPT>(p.sc, bv, base, limit, stage, ring, cand, surf, flags, keep, kept,
                                                                       stage1, &total1, ready, spinLimit, hist);
        }
        if (lane == 0) {
            p.chunkCount[chunk] = total;
            if constexpr (MODE == kModeFrame1) p.keepCount[chunk] = kept;
            if constexpr (fused_mode(MODE)) p.chunkCount2[chunk] = total1;
        }
        chunk = next;
    }
    if (flags) atomicOr(&p.scratch->status, flags);
}

template <int MODE, bool SINGLE, int THREADS, int OPT>
__global__ void __launch_bounds__(THREADS, (SINGLE || MODE >= 0) ? 1024 / THREADS : 1) cull_decide_kernel(const PipeParams p) {
    __shared__ DecideSmem<MODE, SINGLE, THREADS, OPT> sm;
    decide_body<MODE, SINGLE, THREADS, OPT>(p, sm);
}

// The one-call frame with its pyramid (blz_cull_frame given a depth buffer) in one launch. Each
// block first takes pyramid tiles by ticket until none is left, building each with the pyramid
// kernel's block steps in the shared memory its survivor rings use later; the block that finishes
// the last tile builds the top levels and publishes the pyramid (the context's ready flag). Then the
// block's warps run the fused sweep, each waiting for the flag before its first Hi-Z test. Tiles go
// to running blocks only, and a block waits for nothing while it builds, so every tile a warp waits
// for belongs to a block that is running; the waits are bounded all the same. The frame's scatter
// rewinds the ticket, the tile count and the flag.
template <uint32_t HIZ, int THREADS, int OPT>
__global__ void __launch_bounds__(THREADS, 1024 / THREADS) cull_frame_kernel(const PipeParams p,
                                                                           const __grid_constant__ PyramidBuildParams bp) {
    using Smem = DecideSmem<kModeFramePyr, true, THREADS, OPT>;
    __shared__ Smem sm;
    static_assert(sizeof(sm.ring) >= sizeof(float) * (kPyrSmemA + kPyrSmemB), "the tile buffers live in the rings");
    float* sA = reinterpret_cast<float*>(&sm.ring[0][0]);
    float* sB = sA + kPyrSmemA;
    __shared__ uint32_t s_tile;
    Scratch* scr = p.scratch;
    const uint32_t tilesX = (bp.width + kPyrTile - 1) / kPyrTile;
    const uint32_t tiles = tilesX * ((bp.height + kPyrTile - 1) / kPyrTile);
    for (;;) {
        if (threadIdx.x == 0) s_tile = atomicAdd(&scr->frameTicket, 1u);
        __syncthreads();
        const uint32_t t = s_tile;
        if (t >= tiles) break;
        pyramid_tile<HIZ, THREADS>(bp, (t % tilesX) * kPyrTile, (t / tilesX) * kPyrTile, sA, sB);
        pyramid_tile_finish<HIZ, THREADS>(bp, tiles, &scr->frameTilesDone, &scr->frameReady, sA, sB);
        __syncthreads();  // s_tile and the tile buffers are free again
    }
    decide_body<kModeFramePyr, true, THREADS, OPT>(p, sm, &scr->frameReady, bp.spinLimit);
}

// ------------------------------------------------------------------ scatter kernel

// Each block owns 32 consecutive chunks, one per warp, and finds where their records go without
// any grid-wide step: it sums the counts of its first chunk's view that precede that chunk (a
// strided read of at most one view's counts, from L2), and warp 0 scans the 32 chunks' counts
// (restarting at view boundaries). The block's warps then copy the chunks' staged records to their slots as full
// records, and the lane holding a view's last chunk writes that view's draw count. Block 0 also
// rewinds the decide kernel's work counter for the next launch.
constexpr int kScatterWarps = 32;  // one warp per chunk
constexpr uint32_t kScatterChunks = 32;
constexpr uint32_t kScatterPre = 3;  // 32-record slices of its chunk a warp loads before the offsets are known

template <bool SINGLE>
__device__ __forceinline__ void scatter_block(const PipeParams& p, const uint32_t block) {
    __shared__ uint32_t s_part[kScatterWarps];
    __shared__ uint32_t s_base[kScatterChunks], s_n[kScatterChunks], s_vi[kScatterChunks];
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t chunkSize = p.chunkSize;
    const uint32_t c0 = block * kScatterChunks;
    if (block == 0 && threadIdx.x == 0 && p.workCounter != nullptr) *p.workCounter = 0u;
    if (c0 >= p.totalTiles) return;
    const uint32_t vi0 = SINGLE ? 0u : find_view_warp(p.tileStart, p.viewCount, c0);
    const uint32_t viewStart0 = SINGLE ? 0u : __ldg(p.tileStart + vi0);
    // 0. each warp fetches its chunk's count (handed to warp 0 through shared memory) and, once it
    //    is known, its first kScatterPre * 32 staged records, which arrive while the block scans;
    //    their LODs are fetched after the barrier
    const uint32_t myChunk = c0 + warp;
    const uint32_t myN = myChunk < p.totalTiles ? __ldcg(p.chunkCount + myChunk) : 0u;
    const uint2* myStage = p.staged + static_cast<size_t>(myChunk) * chunkSize;
    // 1. records of the first chunk's view before c0, loaded while the count is on its way
    uint32_t part = 0;
    for (uint32_t c = viewStart0 + threadIdx.x; c < c0; c += 8u * kScatterWarps * 32u) {
        uint32_t x[8];  // eight loads in flight per thread
#pragma unroll
        for (uint32_t k = 0; k < 8u; ++k) {
            const uint32_t ck = c + k * kScatterWarps * 32u;
            x[k] = ck < c0 ? __ldcg(p.chunkCount + ck) : 0u;
        }
#pragma unroll
        for (uint32_t k = 0; k < 8u; ++k) part += x[k];
    }
    uint2 pre[kScatterPre], preLod[kScatterPre];
#pragma unroll
    for (uint32_t u = 0; u < kScatterPre; ++u) {
        const uint32_t i = lane + 32u * u;
        pre[u] = i < myN ? __ldcg(myStage + i) : make_uint2(0u, 0u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xFFFFFFFFu, part, o);
    if (lane == 0) {
        s_part[warp] = part;
        s_n[warp] = myN;
    }
    __syncthreads();
#pragma unroll
    for (uint32_t u = 0; u < kScatterPre; ++u) {
        const uint32_t i = lane + 32u * u;
        preLod[u] = i < myN ? __ldg(reinterpret_cast<const uint2*>(p.sc.lods + pre[u].y)) : make_uint2(0u, 0u);
    }
    // 2. warp 0: exclusive offsets of the block's chunks, a scan restarting at each view's first chunk
    if (warp == 0) {
        uint32_t carry = 0;
#pragma unroll
        for (int w = 0; w < kScatterWarps; ++w) carry += s_part[w];
        const uint32_t c = c0 + lane;
        const bool in = c < p.totalTiles;
        const uint32_t n = s_n[lane];  // 0 past the last chunk
        uint32_t vi = vi0;
        bool starts = false;  // this chunk starts a view (the scan restarts here)
        if constexpr (!SINGLE) {
            // the next 32 view starts after vi0: a lane's view is vi0 + those at or before its chunk
            const uint32_t j = vi0 + 1u + lane;
            const uint32_t sj = j < p.viewCount ? __ldg(p.tileStart + j) : 0xFFFFFFFFu;
            uint32_t cnt = 0;
#pragma unroll
            for (int t = 0; t < 32; ++t) cnt += __shfl_sync(0xFFFFFFFFu, sj, t) <= c ? 1u : 0u;
            if (in) {
                // more than 32 views (empty ones) can start inside the block's chunks: search then
                vi = cnt < 32u ? vi0 + cnt : find_view(p.tileStart, p.viewCount, c);
                starts = c == __ldg(p.tileStart + vi);
            }
        }
        // segmented inclusive scan: combine(a, b) = b.starts ? b : a + b
        uint32_t sum = n;
        bool flag = starts;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t ps = __shfl_up_sync(0xFFFFFFFFu, sum, o);
            const bool pf = __shfl_up_sync(0xFFFFFFFFu, flag ? 1u : 0u, o) != 0u;
            if (lane >= static_cast<uint32_t>(o) && !flag) {
                sum += ps;
                flag = pf;
            }
        }
        // lanes still in the first view (no start at or before them) add the view's earlier records
        const uint32_t excl = sum - n + (flag ? 0u : carry);
        s_base[lane] = excl;
        s_vi[lane] = vi;
        if (in) {
            const bool lastOfView = SINGLE ? (c + 1 == p.totalTiles) : (c + 1 == __ldg(p.tileStart + vi + 1));
            if (lastOfView) {
                const BatchViewDev& bv = view_of<SINGLE>(p, vi);
                *bv.drawCount = excl + n;
                if (excl + n > bv.capacity) atomicOr(&p.scratch->status, BLZ_FLAG_COMMAND_OVERFLOW);
            }
        }
    }
    __syncthreads();
    // 3. scatter: each warp its own chunk (kScatterWarps == kScatterChunks)
    static_assert(kScatterWarps == static_cast<int>(kScatterChunks), "one warp per chunk");
    if (myChunk >= p.totalTiles) return;
    const uint32_t base = s_base[warp];
    const BatchViewDev& bv = view_of<SINGLE>(p, s_vi[warp]);
    // staged record i goes to slot base + i, or base + n - 1 - i for a chunk staged last object first
    const bool down = SINGLE && p.descending != 0u;
#pragma unroll
    for (uint32_t u = 0; u < kScatterPre; ++u) {
        const uint32_t i = lane + 32u * u;
        const uint32_t slot = base + (down ? myN - 1u - i : i);
        if (i < myN && slot < bv.capacity) put_record(bv.cmds, bv.stride, slot, pre[u].x, preLod[u].x, preLod[u].y);
    }
    for (uint32_t i = lane + 32u * kScatterPre; i < myN; i += 32) {
        const uint32_t slot = base + (down ? myN - 1u - i : i);
        if (slot >= bv.capacity) {
            if (down) continue;
            break;
        }
        const uint2 rec = __ldcg(myStage + i);
        const uint2 lod = __ldg(reinterpret_cast<const uint2*>(p.sc.lods + rec.y));  // indexCount, firstIndex
        put_record(bv.cmds, bv.stride, slot, rec.x, lod.x, lod.y);
    }
}

template <bool SINGLE>
__global__ void __launch_bounds__(kScatterWarps * 32, 2) cull_scatter_kernel(const PipeParams p) {
    scatter_block<SINGLE>(p, blockIdx.x);
}

// Both record lists of a one-call frame in one launch: blocks [0, blocks1) scatter list 1, the rest
// list 2. Block 0 also rewinds the frame kernel's pyramid ticket, tile count and ready flag (the
// frame kernel has finished: this launch follows it on the stream).
__global__ void __launch_bounds__(kScatterWarps * 32, 2) cull_scatter2_kernel(const PipeParams p1, const PipeParams p2,
                                                                           const uint32_t blocks1) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        p1.scratch->frameTicket = 0u;
        p1.scratch->frameTilesDone = 0u;
        p1.scratch->frameReady = 0u;
    }
    if (blockIdx.x < blocks1) scatter_block<true>(p1, blockIdx.x);
    else scatter_block<true>(p2, blockIdx.x - blocks1);
}

// ------------------------------------------------------------------ kept frame, pass 2

// Pass 2 of a kept frame (blz_frame_late): one warp per chunk runs the dense stage of pass 2 over
// the survivors pass 1 kept for that chunk, in object order: projectSphere and the Hi-Z test
// (drawOccLate.cs.hlsl:48-58), the visibility rewrite (:67) and the emission of objects not visible
// last frame (:45), staged as (objectId, lodId) for the scatter. Every object pass 1 did not keep was
// outside the frustum and got its visibility in pass 1. A lane takes kLateRounds survivors at once
// (j, j + 32, ...): their loads, tests and LOD selections are independent, so their latencies
// overlap; they are staged in order afterwards.
constexpr uint32_t kLateRounds = 4;

template <int THREADS>
__global__ void __launch_bounds__(THREADS) frame_late_kernel(const PipeParams p) {
    constexpr int NW = THREADS / 32;
    constexpr uint32_t R = kLateRounds;
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t warpsTotal = gridDim.x * NW;
    const BatchViewDev& bv = p.single;
    const ViewConsts v = load_view(bv.view);
    const uint32_t lt = lanemask_lt();
    for (uint32_t chunk = blockIdx.x * NW + warp; chunk < p.totalTiles; chunk += warpsTotal) {
        const uint32_t n = __ldcg(p.keepCount + chunk);
        const uint4* keep = static_cast<const uint4*>(p.keep) + 2u * static_cast<size_t>(chunk) * p.chunkSize;
        uint2* stage = p.staged + static_cast<size_t>(chunk) * p.chunkSize;
        uint32_t run = 0;
        for (uint32_t j0 = 0; j0 < n; j0 += 32u * R) {
            uint4 a[R], b[R];
#pragma unroll
            for (uint32_t r = 0; r < R; ++r) {
                const uint32_t j = j0 + r * 32u + lane;
                a[r] = make_uint4(0u, 0u, 0u, 0u);
                b[r] = a[r];
                if (j < n) {
                    a[r] = __ldcg(keep + 2u * j);
                    b[r] = __ldcg(keep + 2u * j + 1u);
                }
            }
            bool emit[R];
            uint32_t lid[R];
#pragma unroll
            for (uint32_t r = 0; r < R; ++r) {
                const bool mine = j0 + r * 32u + lane < n;
                const uint32_t obj = a[r].x & 0x3FFFFFFFu;
                const Vec3 c{__uint_as_float(a[r].y), __uint_as_float(a[r].z), __uint_as_float(a[r].w)};
                const float rad = __uint_as_float(b[r].x);
                bool visible = mine;
                if (mine) {
                    float4 aabb;
                    if (project_sphere(c, rad, v.zNear, v.proj0, v.proj5, aabb)) visible = occlusion(aabb, bv.pyr, v, c, rad);
                    // drawOccLate.cs.hlsl:67, storing only a value that changes
                    const bool wasNonZero = (a[r].x >> 31) != 0u, wasOne = ((a[r].x >> 30) & 1u) != 0u;
                    if (visible ? !wasOne : wasNonZero) bv.vis[obj] = visible ? 1u : 0u;
                }
                emit[r] = visible && (a[r].x >> 31) == 0u;  // drawOccLate.cs.hlsl:45
                lid[r] = 0u;
                if (emit[r]) {
                    // cullBuffers.hlsl:42-55 — last LOD in [1, lodCount) with error < threshold
                    const float threshold = lod_threshold(c, rad, __uint_as_float(b[r].y), v.lodTarget);
                    uint32_t sel = 0;
                    for (uint32_t t = 1; t < b[r].w; ++t)
                        if (__ldg(&p.sc.lods[b[r].z + t].error) < threshold) sel = t;
                    lid[r] = b[r].z + sel;
                }
            }
#pragma unroll
            for (uint32_t r = 0; r < R; ++r) {
                const unsigned e = __ballot_sync(0xFFFFFFFFu, emit[r]);
                if (emit[r]) stage[run + __popc(e & lt)] = make_uint2(a[r].x & 0x3FFFFFFFu, lid[r]);
                run += __popc(e);
            }
        }
        if (lane == 0) p.chunkCount[chunk] = run;
    }
}

// ------------------------------------------------------------------ launchers

// Resident blocks per SM of one instantiation (a property of the kernel, asked once).
template <int MODE, bool SINGLE, int THREADS, int OPT>
static uint32_t occupancy_t() {
    static const uint32_t occ = [] {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, cull_decide_kernel<MODE, SINGLE, THREADS, OPT>, THREADS, 0) !=
            cudaSuccess) {
            (void)cudaGetLastError();
            o = 1;
        }
        return static_cast<uint32_t>(o < 1 ? 1 : o);
    }();
    return occ;
}

template <int MODE, bool SINGLE, int THREADS, int OPT>
static cudaError_t launch_decide_t(const PipeParams& p, uint32_t blocksPerSm, int smCount, cudaStream_t s) {
    auto kern = cull_decide_kernel<MODE, SINGLE, THREADS, OPT>;
    const uint32_t occ = occupancy_t<MODE, SINGLE, THREADS, OPT>();
    const uint32_t per = blocksPerSm ? (blocksPerSm < occ ? blocksPerSm : occ) : occ;
    uint32_t grid = per * static_cast<uint32_t>(smCount);
    const uint32_t needed = (p.totalTiles + THREADS / 32 - 1) / (THREADS / 32);  // one warp per chunk at most
    if (grid > needed) grid = needed;
    if (grid == 0) grid = 1;
    kern<<<grid, THREADS, 0, s>>>(p);
    return cudaGetLastError();
}

template <int MODE, bool SINGLE, int THREADS, int OPT>
static cudaError_t launch_t(const PipeParams& p, uint32_t blocksPerSm, int smCount, cudaStream_t s) {
    cudaError_t e = launch_decide_t<MODE, SINGLE, THREADS, OPT>(p, blocksPerSm, smCount, s);
    if (e != cudaSuccess) return e;
    const uint32_t sgrid = (p.totalTiles + kScatterChunks - 1) / kScatterChunks;
    cull_scatter_kernel<SINGLE><<<sgrid ? sgrid : 1u, kScatterWarps * 32, 0, s>>>(p);
    return cudaGetLastError();
}

uint32_t object_tile_size() { return kChunk; }

template <int THREADS, int OPT>
static cudaError_t launch_frame_first_t(const PipeParams& p, int smCount, cudaStream_t s, bool scatter) {
    cudaError_t e = launch_decide_t<kModeFrame1, true, THREADS, OPT>(p, 0, smCount, s);
    if (e != cudaSuccess || !scatter) return e;
    const uint32_t sgrid = (p.totalTiles + kScatterChunks - 1) / kScatterChunks;
    cull_scatter_kernel<true><<<sgrid ? sgrid : 1u, kScatterWarps * 32, 0, s>>>(p);
    return cudaGetLastError();
}

cudaError_t launch_frame_first(const PipeParams& p, uint32_t threads, uint32_t opt, int smCount, cudaStream_t s,
                               bool scatter) {
    PipeParams q = p;
    q.descending = 0u;
    if (threads == 256 && opt == 1) return launch_frame_first_t<256, 1>(q, smCount, s, scatter);
    if (threads == 256 && opt == 4) return launch_frame_first_t<256, 4>(q, smCount, s, scatter);
    if (threads == 128 && opt == 2) return launch_frame_first_t<128, 2>(q, smCount, s, scatter);
    if (threads == 128 && opt == 4) return launch_frame_first_t<128, 4>(q, smCount, s, scatter);
    if (threads == 512 && opt == 1) return launch_frame_first_t<512, 1>(q, smCount, s, scatter);
    return launch_frame_first_t<kObjThreads, kObjOpt>(q, smCount, s, scatter);
}

cudaError_t launch_frame_fused(const PipeParams& p, uint32_t threads, uint32_t opt, int smCount, cudaStream_t s) {
    PipeParams q = p;
    q.descending = 0u;
    if (threads == 256 && opt == 1) return launch_decide_t<kModeFrameFused, true, 256, 1>(q, 0, smCount, s);
    if (threads == 256 && opt == 4) return launch_decide_t<kModeFrameFused, true, 256, 4>(q, 0, smCount, s);
    if (threads == 128 && opt == 2) return launch_decide_t<kModeFrameFused, true, 128, 2>(q, 0, smCount, s);
    if (threads == 128 && opt == 4) return launch_decide_t<kModeFrameFused, true, 128, 4>(q, 0, smCount, s);
    if (threads == 512 && opt == 1) return launch_decide_t<kModeFrameFused, true, 512, 1>(q, 0, smCount, s);
    return launch_decide_t<kModeFrameFused, true, kObjThreads, kObjOpt>(q, 0, smCount, s);
}

template <uint32_t HIZ, int THREADS, int OPT>
static cudaError_t launch_frame_pyr_t(const PipeParams& p, const PyramidBuildParams& bp, int smCount, cudaStream_t s) {
    auto kern = cull_frame_kernel<HIZ, THREADS, OPT>;
    static const uint32_t occ = [&] {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, kern, THREADS, 0) != cudaSuccess) {
            (void)cudaGetLastError();
            o = 1;
        }
        return static_cast<uint32_t>(o < 1 ? 1 : o);
    }();
    // one warp per chunk at most, but enough blocks (up to one wave) to build the pyramid's tiles
    const uint32_t wave = occ * static_cast<uint32_t>(smCount > 0 ? smCount : 1);
    const uint32_t tiles = ((bp.width + kPyrTile - 1) / kPyrTile) * ((bp.height + kPyrTile - 1) / kPyrTile);
    uint32_t grid = (p.totalTiles + THREADS / 32 - 1) / (THREADS / 32);
    if (grid < tiles) grid = tiles;
    if (grid > wave) grid = wave;
    if (grid == 0) grid = 1;
    kern<<<grid, THREADS, 0, s>>>(p, bp);
    return cudaGetLastError();
}

template <uint32_t HIZ>
static cudaError_t launch_frame_pyr_hiz(const PipeParams& q, const PyramidBuildParams& bp, uint32_t threads, uint32_t opt,
                                        int smCount, cudaStream_t s) {
    if (threads == 256 && opt == 1) return launch_frame_pyr_t<HIZ, 256, 1>(q, bp, smCount, s);
    if (threads == 256 && opt == 4) return launch_frame_pyr_t<HIZ, 256, 4>(q, bp, smCount, s);
    if (threads == 128 && opt == 2) return launch_frame_pyr_t<HIZ, 128, 2>(q, bp, smCount, s);
    if (threads == 128 && opt == 4) return launch_frame_pyr_t<HIZ, 128, 4>(q, bp, smCount, s);
    if (threads == 512 && opt == 1) return launch_frame_pyr_t<HIZ, 512, 1>(q, bp, smCount, s);
    return launch_frame_pyr_t<HIZ, kObjThreads, kObjOpt>(q, bp, smCount, s);
}

cudaError_t launch_frame_pyr(const PipeParams& p, const PyramidBuildParams& bp, uint32_t threads, uint32_t opt, int smCount,
                             cudaStream_t s) {
    PipeParams q = p;
    q.descending = 0u;
    if (bp.mode == BLZ_HIZ_VULKAN) return launch_frame_pyr_hiz<BLZ_HIZ_VULKAN>(q, bp, threads, opt, smCount, s);
    return launch_frame_pyr_hiz<BLZ_HIZ_D3D12>(q, bp, threads, opt, smCount, s);
}

constexpr int kFrameLateThreads = 256;

cudaError_t launch_frame_late(const PipeParams& p, int smCount, cudaStream_t s, bool scatter) {
    static const uint32_t occ = [] {
        int o = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, frame_late_kernel<kFrameLateThreads>, kFrameLateThreads, 0) !=
            cudaSuccess) {
            (void)cudaGetLastError();
            o = 1;
        }
        return static_cast<uint32_t>(o < 1 ? 1 : o);
    }();
    constexpr uint32_t NW = kFrameLateThreads / 32;
    uint32_t grid = occ * static_cast<uint32_t>(smCount > 0 ? smCount : 1);
    const uint32_t needed = (p.totalTiles + NW - 1) / NW;
    if (grid > needed) grid = needed;
    if (grid == 0) grid = 1;
    PipeParams q = p;
    q.descending = 0u;
    frame_late_kernel<kFrameLateThreads><<<grid, kFrameLateThreads, 0, s>>>(q);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !scatter) return e;
    const uint32_t sgrid = (q.totalTiles + kScatterChunks - 1) / kScatterChunks;
    cull_scatter_kernel<true><<<sgrid ? sgrid : 1u, kScatterWarps * 32, 0, s>>>(q);
    return cudaGetLastError();
}

cudaError_t launch_frame_scatter2(const PipeParams& p1, const PipeParams& p2, cudaStream_t s) {
    const uint32_t g1 = (p1.totalTiles + kScatterChunks - 1) / kScatterChunks;
    const uint32_t g2 = (p2.totalTiles + kScatterChunks - 1) / kScatterChunks;
    PipeParams q1 = p1, q2 = p2;
    q1.descending = q2.descending = 0u;
    cull_scatter2_kernel<<<(g1 ? g1 : 1u) + (g2 ? g2 : 1u), kScatterWarps * 32, 0, s>>>(q1, q2, g1 ? g1 : 1u);
    return cudaGetLastError();
}

template <int MODE>
static uint32_t single_blocks_per_sm(uint32_t threads, uint32_t opt) {
    if (threads == 256 && opt == 1) return occupancy_t<MODE, true, 256, 1>();
    if (threads == 256 && opt == 4) return occupancy_t<MODE, true, 256, 4>();
    if (threads == 128 && opt == 2) return occupancy_t<MODE, true, 128, 2>();
    if (threads == 128 && opt == 4) return occupancy_t<MODE, true, 128, 4>();
    if (threads == 512 && opt == 1) return occupancy_t<MODE, true, 512, 1>();
    return occupancy_t<MODE, true, kObjThreads, kObjOpt>();
}

uint32_t single_chunk_size(uint32_t mode, uint32_t threads, uint32_t opt, uint32_t count, int smCount) {
    if (!single_shape_supported(threads, opt)) {
        threads = kObjThreads;
        opt = kObjOpt;
    }
    uint32_t per = 1;
    switch (mode) {
        case kModeFrame1: per = single_blocks_per_sm<kModeFrame1>(threads, opt); break;
        case kModeFrameFused: per = single_blocks_per_sm<kModeFrameFused>(threads, opt); break;
        case BLZ_MODE_FIRST: per = single_blocks_per_sm<BLZ_MODE_FIRST>(threads, opt); break;
        case BLZ_MODE_LATE: per = single_blocks_per_sm<BLZ_MODE_LATE>(threads, opt); break;
        case BLZ_MODE_TEMPORAL: per = single_blocks_per_sm<BLZ_MODE_TEMPORAL>(threads, opt); break;
        case kModeInstanced: per = single_blocks_per_sm<kModeInstanced>(threads, opt); break;
        default: per = single_blocks_per_sm<BLZ_MODE_FRUSTUM>(threads, opt); break;
    }
    const uint64_t warps = static_cast<uint64_t>(per) * static_cast<uint64_t>(smCount > 0 ? smCount : 1) * (threads / 32u);
    const uint32_t step = 32u * opt;
    uint64_t size = (count + warps - 1) / warps;
    size = (size + step - 1) / step * step;
    return static_cast<uint32_t>(size < step ? step : size);
}

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
    PipeParams q = p;
    q.descending = mode == BLZ_MODE_LATE ? 1u : 0u;  // the single-view pass-2 decide walks its chunks downwards
    switch (mode) {
        case BLZ_MODE_FRUSTUM: return launch_single_mode<BLZ_MODE_FRUSTUM>(q, threads, opt, smCount, s);
        case BLZ_MODE_FIRST: return launch_single_mode<BLZ_MODE_FIRST>(q, threads, opt, smCount, s);
        case BLZ_MODE_LATE: return launch_single_mode<BLZ_MODE_LATE>(q, threads, opt, smCount, s);
        case BLZ_MODE_TEMPORAL: return launch_single_mode<BLZ_MODE_TEMPORAL>(q, threads, opt, smCount, s);
        default: return cudaErrorInvalidValue;
    }
}

// ------------------------------------------------------------------ instanced cull from the staged records
//
// The instanced cull (drawInstCountReset + drawInstCull + drawInstCmd) decides exactly what the
// frustum + LOD pass decides: every visible object and its LOD. So it runs that decide kernel
// (kModeInstanced), whose staged (objectId, lodId) records are in object order per chunk and which
// also counts each group's records per LOD (hist[group][lod], groups of kInstGroup chunks, zeroed
// before the launch), and then one place launch, a block per group:
//   offsets  each LOD's offset for the group is the sum of the LOD's counts in the groups before it
//            (coalesced loads across LODs, the block's threads taking interleaved groups); the last
//            group's block adds its own group's counts, which gives every LOD's total, and writes
//            the counters and, in ascending LOD order, one command per non-empty LOD;
//   rows     each warp counts its chunk's records per LOD, and the block scans those rows per LOD;
//   place    each warp places its records in order (ranks inside 32-record slices from one
//            ballot per bit of the LOD id).

constexpr uint32_t kInstBatch = 5;  // 32-record slices whose loads are issued together (the first batch's ranks are kept)
constexpr uint32_t kInstThreads = kInstGroup * 32;


__global__ void __launch_bounds__(kInstThreads) inst_place_kernel(const InstStagedParams q) {
    // [kInstGroup][nL] per-warp counts, then offsets; [nL] the group's offset in each LOD's list;
    // [nL] each LOD's instanceOffset; [nL] (the last group's block) each LOD's total; [R][nL] partial sums
    extern __shared__ uint32_t s_rows[];
    __shared__ unsigned int s_flags;
    __shared__ uint32_t s_warpSums[32];
    const uint32_t nL = q.nL, G = q.groups, g = blockIdx.x;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31u;
    uint32_t* s_goff = s_rows + kInstGroup * nL;
    uint32_t* s_ioff = s_goff + nL;
    uint32_t* s_tot = s_ioff + nL;
    uint32_t* s_part = s_tot + nL;
    // thread t works on LOD t % nL as row t / nL of R rows (nL <= kInstStagedMaxLods <= kInstThreads)
    const uint32_t R = kInstThreads / nL;
    const uint32_t tb = threadIdx.x % nL, tr = threadIdx.x / nL;
    const uint32_t chunk = g * kInstGroup + warp;
    const uint32_t n = chunk < q.totalTiles ? __ldcg(q.chunkCount + chunk) : 0u;
    const uint2* st = q.staged + static_cast<size_t>(chunk) * q.chunkSize;
    auto load_batch = [&](uint32_t j0, uint2 (&r)[kInstBatch]) {
#pragma unroll
        for (uint32_t k = 0; k < kInstBatch; ++k) {
            const uint32_t j = j0 + k * 32u + lane;
            r[k] = j < n ? __ldcg(st + j) : make_uint2(0u, 0xFFFFFFFFu);
        }
    };
    uint2 first[kInstBatch];  // the chunk's first kInstBatch * 32 records, loaded once for both walks
    load_batch(0, first);
    // LOD threadIdx.x's instanceOffset (nL <= kInstThreads), stored to shared memory once phase 1
    // is done, so no barrier waits for the load
    const uint32_t ioff = threadIdx.x < nL ? __ldg(&q.counters[threadIdx.x].instanceOffset) : 0u;
    const uint32_t idBits = nL > 1u ? 32u - static_cast<uint32_t>(__clz(static_cast<int>(nL - 1u))) : 0u;
    for (uint32_t b = threadIdx.x; b < nL; b += kInstThreads) {
        s_goff[b] = 0u;
        s_tot[b] = 0u;
    }
    for (uint32_t j = threadIdx.x; j < kInstGroup * nL; j += kInstThreads) s_rows[j] = 0u;
    if (threadIdx.x == 0) s_flags = 0u;
    __syncthreads();
    // 0. the group's offset in each LOD's list: the LOD's counts of the groups before this one,
    //    row tr taking every R-th group (coalesced across LODs)
    if (tr < R) {
        const uint32_t g1 = g;
        uint32_t sum = 0, gg = tr;
        for (; gg + 7u * R < g1; gg += 8u * R) {  // eight loads in flight at a time
            uint32_t x[8];
#pragma unroll
            for (uint32_t k = 0; k < 8u; ++k) x[k] = __ldcg(q.hist + static_cast<size_t>(gg + k * R) * nL + tb);
#pragma unroll
            for (uint32_t k = 0; k < 8u; ++k) sum += x[k];
        }
        for (; gg < g1; gg += R) sum += __ldcg(q.hist + static_cast<size_t>(gg) * nL + tb);
        if (sum) atomicAdd(&s_goff[tb], sum);
    }
    uint32_t* row = s_rows + warp * nL;
    const uint32_t lt = lanemask_lt();
    // 1. this chunk's records per LOD (only this warp touches its row); each of the first batch's
    //    records also keeps its rank among the chunk's records of its LOD (the count before its
    //    32-record slice, from the slice's lowest lane of that LOD, plus the lanes below it)
    uint32_t rank[kInstBatch];
    for (uint32_t j0 = 0; j0 < n; j0 += 32u * kInstBatch) {
        uint2 r[kInstBatch];
        if (j0 == 0) {
#pragma unroll
            for (uint32_t k = 0; k < kInstBatch; ++k) r[k] = first[k];
        } else {
            load_batch(j0, r);
        }
#pragma unroll
        for (uint32_t k = 0; k < kInstBatch; ++k) {
            const uint32_t b = r[k].y;
            const unsigned peers = same_lod_lanes(b, idBits, b != 0xFFFFFFFFu);
            uint32_t before = 0;
            if (b != 0xFFFFFFFFu && (peers & lt) == 0u) {
                before = row[b];
                row[b] = before + __popc(peers);
            }
            if (j0 == 0) {  // warp-uniform
                before = __shfl_sync(0xFFFFFFFFu, before, (__ffs(peers) - 1) & 31);
                rank[k] = before + __popc(peers & lt);
            }
            __syncwarp();
        }
    }
    if (threadIdx.x < nL) s_ioff[threadIdx.x] = ioff;
    __syncthreads();
    // 2. per LOD, exclusive offsets of the warps' chunks inside the group: row tr of threads sums
    //    its kInstGroup / R consecutive warps' counts, then scans them after the sums of the rows
    //    before it
    const uint32_t per = (kInstGroup + R - 1u) / R;
    const uint32_t w0 = min(kInstGroup, tr * per), w1 = min(kInstGroup, w0 + per);
    if (tr < R) {
        uint32_t part = 0;
        for (uint32_t w = w0; w < w1; ++w) part += s_rows[w * nL + tb];
        s_part[tr * nL + tb] = part;
    }
    __syncthreads();
    if (tr < R) {
        uint32_t run = 0;
        for (uint32_t r = 0; r < tr; ++r) run += s_part[r * nL + tb];
        for (uint32_t w = w0; w < w1; ++w) {
            const uint32_t c = s_rows[w * nL + tb];
            s_rows[w * nL + tb] = run;
            run += c;
        }
    }
    __syncthreads();
    // 3. place the records in object order: a chunk the first batch holds whole places each record
    //    at its LOD's group offset + the warp's offset + its rank; a longer one ranks its records
    //    again, slice by slice
    const uint32_t slots = q.slotsPerLod ? q.slotsPerLod : 0xFFFFFFFFu;
    unsigned int flags = 0u;
    if (n <= 32u * kInstBatch) {
#pragma unroll
        for (uint32_t k = 0; k < kInstBatch; ++k) {
            const uint32_t b = first[k].y;
            if (b == 0xFFFFFFFFu) continue;
            const uint32_t pos = s_goff[b] + row[b] + rank[k];
            const uint64_t at = static_cast<uint64_t>(s_ioff[b]) + pos;
            if (pos < slots && at < q.instanceCapacity) q.instances[at] = first[k].x;
            else flags |= BLZ_FLAG_INSTANCE_OVERFLOW;
        }
    }
    for (uint32_t j0 = 0; n > 32u * kInstBatch && j0 < n; j0 += 32u * kInstBatch) {
        uint2 r[kInstBatch];
        if (j0 == 0) {
#pragma unroll
            for (uint32_t k = 0; k < kInstBatch; ++k) r[k] = first[k];
        } else {
            load_batch(j0, r);
        }
#pragma unroll
        for (uint32_t k = 0; k < kInstBatch; ++k) {
            const uint32_t b = r[k].y;
            const unsigned peers = same_lod_lanes(b, idBits, b != 0xFFFFFFFFu);
            uint32_t before = 0;
            if (b != 0xFFFFFFFFu) before = row[b];
            __syncwarp();
            if (b != 0xFFFFFFFFu) {
                if ((peers & lt) == 0u) row[b] = before + __popc(peers);
                const uint32_t pos = s_goff[b] + before + __popc(peers & lt);
                const uint64_t at = static_cast<uint64_t>(s_ioff[b]) + pos;
                if (pos < slots && at < q.instanceCapacity) q.instances[at] = r[k].x;
                else flags |= BLZ_FLAG_INSTANCE_OVERFLOW;
            }
            __syncwarp();
        }
    }
    // 4. the last group's block: every LOD's total is its group offset plus its own group's count;
    //    then the counters and, in ascending LOD order, one command per non-empty LOD
    //    (drawInstCmd.cs.hlsl:9-38)
    if (g == G - 1u) {
        for (uint32_t l = threadIdx.x; l < nL; l += kInstThreads)
            s_tot[l] = s_goff[l] + __ldcg(q.hist + static_cast<size_t>(g) * nL + l);
        __syncthreads();
        const uint32_t perT = (nL + kInstThreads - 1u) / kInstThreads;
        const uint32_t b0 = min(nL, threadIdx.x * perT), b1 = min(nL, b0 + perT);
        uint32_t mine = 0;
        for (uint32_t l = b0; l < b1; ++l) mine += s_tot[l] ? 1u : 0u;
        uint32_t incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t x = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= static_cast<uint32_t>(o)) incl += x;
        }
        if (lane == 31) s_warpSums[warp] = incl;
        __syncthreads();
        uint32_t warpOff = 0, all = 0;
        for (uint32_t w = 0; w < 32u; ++w) {
            if (w < warp) warpOff += s_warpSums[w];
            all += s_warpSums[w];
        }
        uint32_t out = warpOff + incl - mine;
        for (uint32_t l = b0; l < b1; ++l) {
            const uint32_t total = s_tot[l];
            q.counters[l].instanceCount = total;
            const uint32_t offset = s_ioff[l];
            if (total > slots || static_cast<uint64_t>(offset) + min(total, slots) > q.instanceCapacity)
                flags |= BLZ_FLAG_INSTANCE_OVERFLOW;
            if (total == 0u) continue;
            if (out < q.capacity) {
                uint32_t* w = reinterpret_cast<uint32_t*>(q.cmds + static_cast<size_t>(out) * q.stride);
                const uint2 lod = __ldg(reinterpret_cast<const uint2*>(q.lods + l));  // indexCount, firstIndex
                w[0] = offset;
                w[1] = lod.x;
                w[2] = min(total, slots);
                w[3] = lod.y;
                w[4] = 0u;
                w[5] = 0u;
            }
            ++out;
        }
        if (all > q.capacity) flags |= BLZ_FLAG_COMMAND_OVERFLOW;
        if (threadIdx.x == 0) *q.drawCount = all;
    }
    if (flags) atomicOr(&s_flags, flags);
    __syncthreads();
    if (threadIdx.x == 0 && s_flags) atomicOr(q.status, s_flags);
}

uint32_t instanced_group_count(uint32_t chunks) { return (chunks + kInstGroup - 1) / kInstGroup; }

cudaError_t launch_instanced_staged(const PipeParams& p, const InstStagedParams& q, uint32_t threads, uint32_t opt,
                                    int smCount, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(p.instHist, 0, sizeof(uint32_t) * static_cast<size_t>(q.groups) * q.nL, s);
    if (e != cudaSuccess) return e;
    if (threads == 256 && opt == 1) e = launch_decide_t<kModeInstanced, true, 256, 1>(p, 0, smCount, s);
    else if (threads == 256 && opt == 4) e = launch_decide_t<kModeInstanced, true, 256, 4>(p, 0, smCount, s);
    else if (threads == 128 && opt == 2) e = launch_decide_t<kModeInstanced, true, 128, 2>(p, 0, smCount, s);
    else if (threads == 128 && opt == 4) e = launch_decide_t<kModeInstanced, true, 128, 4>(p, 0, smCount, s);
    else if (threads == 512 && opt == 1) e = launch_decide_t<kModeInstanced, true, 512, 1>(p, 0, smCount, s);
    else e = launch_decide_t<kModeInstanced, true, kObjThreads, kObjOpt>(p, 0, smCount, s);
    if (e != cudaSuccess) return e;
    const size_t rowBytes = sizeof(uint32_t) * ((kInstGroup + 3) * q.nL + (kInstThreads / q.nL) * q.nL);
    if (rowBytes > 48 * 1024) {
        e = cudaFuncSetAttribute(inst_place_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(rowBytes));
        if (e != cudaSuccess) return e;
    }
    inst_place_kernel<<<q.groups, kInstThreads, rowBytes, s>>>(q);
    return cudaGetLastError();
}

bool batch_shape_supported(uint32_t threads, uint32_t opt) {
    if (!(threads == 128 || threads == 256 || threads == 512)) return false;
    if (!(opt == 1 || opt == 2 || opt == 4 || opt == 8)) return false;
    return threads * opt <= 1024;
}

// A batch whose views all run one pass takes a kernel compiled for that pass: without the other
// passes' code it fits 64 registers, twice the resident warps of the per-view-mode kernel (112).
template <int MODE>
static cudaError_t launch_batch_mode(const PipeParams& p, uint32_t threads, uint32_t blocksPerSm, int smCount,
                                     cudaStream_t s) {
    if (threads == 512) return launch_t<MODE, false, 512, 1>(p, blocksPerSm, smCount, s);
    return launch_t<MODE, false, 256, 1>(p, blocksPerSm, smCount, s);
}

cudaError_t launch_batch_cull(const PipeParams& p, uint32_t threads, uint32_t opt, uint32_t blocksPerSm, int smCount,
                              cudaStream_t s, int mode) {
    if (mode >= 0 && opt == 1 && (threads == 256 || threads == 512)) {
        switch (mode) {
            case BLZ_MODE_FRUSTUM: return launch_batch_mode<BLZ_MODE_FRUSTUM>(p, threads, blocksPerSm, smCount, s);
            case BLZ_MODE_FIRST: return launch_batch_mode<BLZ_MODE_FIRST>(p, threads, blocksPerSm, smCount, s);
            case BLZ_MODE_LATE: return launch_batch_mode<BLZ_MODE_LATE>(p, threads, blocksPerSm, smCount, s);
            case BLZ_MODE_TEMPORAL: return launch_batch_mode<BLZ_MODE_TEMPORAL>(p, threads, blocksPerSm, smCount, s);
            default: break;
        }
    }
#define BLZ_BATCH_CASE(T, O) \
    if (threads == T && opt == O) return launch_t<kModeRuntime, false, T, O>(p, blocksPerSm, smCount, s);
    BLZ_BATCH_CASE(128, 1) BLZ_BATCH_CASE(128, 2) BLZ_BATCH_CASE(128, 4) BLZ_BATCH_CASE(128, 8)
    BLZ_BATCH_CASE(256, 1) BLZ_BATCH_CASE(256, 2) BLZ_BATCH_CASE(256, 4)
    BLZ_BATCH_CASE(512, 1) BLZ_BATCH_CASE(512, 2)
#undef BLZ_BATCH_CASE
    return cudaErrorInvalidValue;
}

}  // namespace blz
