// pyramid_tile.cuh — the Hi-Z pyramid's block-level building steps, shared by the pyramid kernel
// (pyramid.cu) and the one-call frame kernel (cull_objects.cu), which builds the pyramid's tiles
// before its sweep.
//
// A block of NT threads owns a 32x32 tile of mip 0 (every load of the tile issued before any is
// used; D3D12 depth rows read 16 bytes at a time where the extent allows), writes it, and reduces it
// through mips 1..5 in shared memory (a 32-texel tile reaches 1 texel at mip 5). The block that
// finishes the build's last tile (a counter, taken with acquire-release semantics; no block waits)
// builds the few remaining small mips from mip 5.
//
// Texel rules:
//   D3D12   depthPyramid.cs.hlsl:16-26 — min(r, min(g, min(b, a))) of the 2x2 Loads at
//           (2x, 2y) .. (2x+1, 2y+1) of the previous level (the depth buffer for mip 0); a Load
//           outside the previous level returns 0.
//   VULKAN  DepthPyramidGeneration.comp.glsl:15-19 — MIN-reduction bilinear footprint of the
//           previous level at ((x + 0.5) / w, (y + 0.5) / h), clamp to edge. Mip 0 is a power of
//           two, so from mip 1 on the footprint of texel x is {2x, 2x+1} (or {0} on a 1-wide level)
//           and stays inside the block's tile.
#pragma once

#include "blz_device.cuh"
#include "kernels.h"

namespace blz {

constexpr uint32_t kPyrTile = 32;
constexpr uint32_t kPyrInTileLevels = 5;
constexpr uint32_t kPyrSmemA = kPyrTile * kPyrTile;      // floats: a tile's mip 0, or a top level
constexpr uint32_t kPyrSmemB = kPyrTile * kPyrTile / 2;  // floats: the tile's mip 1 (a quarter), or a top level

__device__ __forceinline__ float load_or_zero(const float* img, uint32_t w, uint32_t h, uint64_t x, uint64_t y) {
    return (x < w && y < h) ? __ldcg(img + y * w + x) : 0.0f;
}

// D3D12 2x2 min over an image in global memory (depth buffer or a finished mip).
__device__ __forceinline__ float d3d_texel(const float* src, uint32_t sw, uint32_t sh, uint32_t x, uint32_t y) {
    const uint64_t x0 = 2ull * x, y0 = 2ull * y;
    const float r = load_or_zero(src, sw, sh, x0, y0);
    const float g = load_or_zero(src, sw, sh, x0 + 1, y0);
    const float b = load_or_zero(src, sw, sh, x0, y0 + 1);
    const float a = load_or_zero(src, sw, sh, x0 + 1, y0 + 1);
    return fmin_nan(r, fmin_nan(g, fmin_nan(b, a)));
}

// Footprint indices of texel x of a w-wide level sampling an sw-wide source (Vulkan sampler).
__device__ __forceinline__ void vk_footprint(uint32_t x, uint32_t w, uint32_t sw, uint32_t& i0, uint32_t& i1) {
    const float s = BLZ_FD(BLZ_FA(static_cast<float>(x), 0.5f), static_cast<float>(w));
    const float u = BLZ_FS(BLZ_FM(s, static_cast<float>(sw)), 0.5f);
    const float fu = floorf(u);
    const float au = BLZ_FS(u, fu);
    long long a = to_index(fu);
    long long b = (au > 0.0f) ? a + 1 : a;
    const long long hi = static_cast<long long>(sw) - 1;
    a = a < 0 ? 0 : (a > hi ? hi : a);
    b = b < 0 ? 0 : (b > hi ? hi : b);
    i0 = static_cast<uint32_t>(a);
    i1 = static_cast<uint32_t>(b);
}

template <uint32_t MODE>
__device__ __forceinline__ float level_texel_global(const float* src, uint32_t sw, uint32_t sh, uint32_t x, uint32_t y,
                                                    uint32_t w, uint32_t h) {
    if (MODE == BLZ_HIZ_D3D12) return d3d_texel(src, sw, sh, x, y);
    uint32_t i0, i1, j0, j1;
    vk_footprint(x, w, sw, i0, i1);
    vk_footprint(y, h, sh, j0, j1);
    float m = __int_as_float(0x7fc00000);
    m = fmin_nan(m, __ldcg(src + static_cast<size_t>(j0) * sw + i0));
    m = fmin_nan(m, __ldcg(src + static_cast<size_t>(j0) * sw + i1));
    m = fmin_nan(m, __ldcg(src + static_cast<size_t>(j1) * sw + i0));
    m = fmin_nan(m, __ldcg(src + static_cast<size_t>(j1) * sw + i1));
    return m;
}

// The levels above the tiles' last (mip 5), built by one block from mip 5 in global memory: in
// shared memory when mip 5 fits bufA (capA texels) and half of it fits bufB (capB texels) — each
// level has at most half the texels of the one before (a quarter unless one side is already 1), so
// the levels alternate between the two buffers — else level by level through global memory.
template <uint32_t MODE, int NT>
__device__ __forceinline__ void top_levels(const PyramidBuildParams& p, float* bufA, uint32_t capA, float* bufB,
                                           uint32_t capB) {
    const uint32_t W0 = p.width, H0 = p.height;
    uint32_t k = kPyrInTileLevels + 1;
    const uint32_t Wt = mip_dim(W0, kPyrInTileLevels), Ht = mip_dim(H0, kPyrInTileLevels);
    if (Wt * Ht <= capA && Wt * Ht <= 2u * capB) {
        const float* top = p.data + p.mipOffset[kPyrInTileLevels];
        for (uint32_t i = threadIdx.x; i < Wt * Ht; i += NT) bufA[i] = __ldcg(top + i);
        __syncthreads();
        float* prev = bufA;
        float* next = bufB;
        for (; k < p.mipCount; ++k) {
            const uint32_t Wp = mip_dim(W0, k - 1), Hp = mip_dim(H0, k - 1);
            const uint32_t Wk = mip_dim(W0, k), Hk = mip_dim(H0, k);
            float* out = p.data + p.mipOffset[k];
            for (uint32_t idx = threadIdx.x; idx < Wk * Hk; idx += NT) {
                const uint32_t gx = idx % Wk, gy = idx / Wk;
                float t;
                if (MODE == BLZ_HIZ_D3D12) {
                    const uint32_t x0 = 2u * gx, y0 = 2u * gy;
                    const float r = (x0 < Wp && y0 < Hp) ? prev[y0 * Wp + x0] : 0.0f;
                    const float g = (x0 + 1 < Wp && y0 < Hp) ? prev[y0 * Wp + x0 + 1] : 0.0f;
                    const float b = (x0 < Wp && y0 + 1 < Hp) ? prev[(y0 + 1) * Wp + x0] : 0.0f;
                    const float a = (x0 + 1 < Wp && y0 + 1 < Hp) ? prev[(y0 + 1) * Wp + x0 + 1] : 0.0f;
                    t = fmin_nan(r, fmin_nan(g, fmin_nan(b, a)));
                } else {
                    uint32_t i0, i1, j0, j1;
                    vk_footprint(gx, Wk, Wp, i0, i1);
                    vk_footprint(gy, Hk, Hp, j0, j1);
                    float m = __int_as_float(0x7fc00000);
                    m = fmin_nan(m, prev[j0 * Wp + i0]);
                    m = fmin_nan(m, prev[j0 * Wp + i1]);
                    m = fmin_nan(m, prev[j1 * Wp + i0]);
                    m = fmin_nan(m, prev[j1 * Wp + i1]);
                    t = m;
                }
                next[idx] = t;
                out[idx] = t;
            }
            __syncthreads();
            float* tmp = prev;
            prev = next;
            next = tmp;
        }
        return;
    }
    for (; k < p.mipCount; ++k) {
        const uint32_t Wp = mip_dim(W0, k - 1), Hp = mip_dim(H0, k - 1);
        const uint32_t Wk = mip_dim(W0, k), Hk = mip_dim(H0, k);
        const float* prev = p.data + p.mipOffset[k - 1];
        float* out = p.data + p.mipOffset[k];
        for (uint32_t idx = threadIdx.x; idx < Wk * Hk; idx += NT) {
            const uint32_t gx = idx % Wk, gy = idx / Wk;
            out[idx] = level_texel_global<MODE>(prev, Wp, Hp, gx, gy, Wk, Hk);
        }
        __syncthreads();  // this block's writes of level k are visible to its reads of level k + 1
    }
}

// One 32x32 tile of mip 0 at (X0, Y0), written and reduced through mips 1..5 by the block's NT
// threads; sA holds kPyrSmemA floats, sB kPyrSmemB. It ends on a block barrier that every thread's
// writes precede.
template <uint32_t MODE, int NT>
__device__ __forceinline__ void pyramid_tile(const PyramidBuildParams& p, uint32_t X0, uint32_t Y0, float* sA, float* sB) {
    static_assert(NT >= 64 && NT <= 512 && (NT & (NT - 1)) == 0, "a tile needs 64..512 threads, a power of two");
    constexpr uint32_t PER = kPyrTile * kPyrTile / NT;  // mip-0 texels per thread
    const uint32_t W0 = p.width, H0 = p.height;

    // mip 0 from the depth buffer: all of a thread's source loads are in flight together
    {
        float v[PER];
        if (MODE == BLZ_HIZ_D3D12 && p.vec4) {
            // thread t takes the texel pairs (2i, 2i+1) of tile row j for the pair indices
            // t, t + NT, ... (16 pairs per row): depth rows 2y and 2y+1, columns 4i .. 4i+3, one
            // 16-byte load each. The host chose this path only for a depth width that is a multiple
            // of 4 (so the mip-0 width is even and a pair never crosses it) and a 16-byte aligned buffer.
            float4 q[PER / 2][2];
            const uint32_t dw = p.depthWidth;
#pragma unroll
            for (uint32_t j = 0; j < PER / 2; ++j) {
                const uint32_t pr = threadIdx.x + j * NT;
                const uint32_t gx = X0 + 2u * (pr % (kPyrTile / 2)), gy = Y0 + pr / (kPyrTile / 2);
                const bool in = gx < W0 && gy < H0;
                const float4* row = reinterpret_cast<const float4*>(p.depth + static_cast<size_t>(2u * gy) * dw + 2u * gx);
                q[j][0] = in ? __ldg(row) : make_float4(0.f, 0.f, 0.f, 0.f);
                q[j][1] = in ? __ldg(row + dw / 4u) : make_float4(0.f, 0.f, 0.f, 0.f);
            }
#pragma unroll
            for (uint32_t j = 0; j < PER / 2; ++j) {
                const uint32_t pr = threadIdx.x + j * NT;
                const uint32_t lx = 2u * (pr % (kPyrTile / 2)), ly = pr / (kPyrTile / 2);
                const uint32_t gx = X0 + lx, gy = Y0 + ly;
                const bool in = gx < W0 && gy < H0;
                // texel (2i): r = row0.x, g = row0.y, b = row1.x, a = row1.y; texel (2i+1): .z, .w
                const float t0 = fmin_nan(q[j][0].x, fmin_nan(q[j][0].y, fmin_nan(q[j][1].x, q[j][1].y)));
                const float t1 = fmin_nan(q[j][0].z, fmin_nan(q[j][0].w, fmin_nan(q[j][1].z, q[j][1].w)));
                if (in) *reinterpret_cast<float2*>(p.data + p.mipOffset[0] + static_cast<size_t>(gy) * W0 + gx) = make_float2(t0, t1);
                sA[ly * kPyrTile + lx] = in ? t0 : 0.0f;
                sA[ly * kPyrTile + lx + 1u] = in ? t1 : 0.0f;
            }
        } else if (MODE == BLZ_HIZ_D3D12) {
            float q[PER][4];
#pragma unroll
            for (uint32_t j = 0; j < PER; ++j) {
                const uint32_t idx = threadIdx.x + j * NT;
                const uint32_t gx = X0 + (idx % kPyrTile), gy = Y0 + (idx / kPyrTile);
                const bool in = gx < W0 && gy < H0;
                const uint64_t x0 = 2ull * gx, y0 = 2ull * gy;
                const uint32_t dw = p.depthWidth, dh = p.depthHeight;
                q[j][0] = (in && x0 < dw && y0 < dh) ? __ldg(p.depth + y0 * dw + x0) : 0.0f;
                q[j][1] = (in && x0 + 1 < dw && y0 < dh) ? __ldg(p.depth + y0 * dw + x0 + 1) : 0.0f;
                q[j][2] = (in && x0 < dw && y0 + 1 < dh) ? __ldg(p.depth + (y0 + 1) * dw + x0) : 0.0f;
                q[j][3] = (in && x0 + 1 < dw && y0 + 1 < dh) ? __ldg(p.depth + (y0 + 1) * dw + x0 + 1) : 0.0f;
            }
#pragma unroll
            for (uint32_t j = 0; j < PER; ++j) v[j] = fmin_nan(q[j][0], fmin_nan(q[j][1], fmin_nan(q[j][2], q[j][3])));
        } else {
#pragma unroll
            for (uint32_t j = 0; j < PER; ++j) {
                const uint32_t idx = threadIdx.x + j * NT;
                const uint32_t gx = X0 + (idx % kPyrTile), gy = Y0 + (idx / kPyrTile);
                v[j] = (gx < W0 && gy < H0) ? level_texel_global<MODE>(p.depth, p.depthWidth, p.depthHeight, gx, gy, W0, H0)
                                            : 0.0f;
            }
        }
        if (!(MODE == BLZ_HIZ_D3D12 && p.vec4)) {
#pragma unroll
            for (uint32_t j = 0; j < PER; ++j) {
                const uint32_t idx = threadIdx.x + j * NT;
                const uint32_t gx = X0 + (idx % kPyrTile), gy = Y0 + (idx / kPyrTile);
                const bool in = gx < W0 && gy < H0;
                if (in) p.data[p.mipOffset[0] + static_cast<size_t>(gy) * W0 + gx] = v[j];
                sA[idx] = in ? v[j] : 0.0f;
            }
        }
    }
    __syncthreads();

    // mips 1..5 inside the tile
    float* src = sA;
    float* dst = sB;
    uint32_t S = kPyrTile;  // previous level's tile extent
    for (uint32_t k = 1; k <= kPyrInTileLevels && k < p.mipCount; ++k) {
        const uint32_t Sk = S >> 1;
        const uint32_t Wp = mip_dim(W0, k - 1), Hp = mip_dim(H0, k - 1);
        const uint32_t Wk = mip_dim(W0, k), Hk = mip_dim(H0, k);
        const uint32_t Xp = X0 >> (k - 1), Yp = Y0 >> (k - 1);
        const uint32_t Xk = X0 >> k, Yk = Y0 >> k;
        for (uint32_t idx = threadIdx.x; idx < Sk * Sk; idx += NT) {
            const uint32_t lx = idx % Sk, ly = idx / Sk;
            const uint32_t gx = Xk + lx, gy = Yk + ly;
            float v = 0.0f;
            if (gx < Wk && gy < Hk) {
                if (MODE == BLZ_HIZ_D3D12) {
                    const uint32_t x0 = 2u * gx, y0 = 2u * gy;
                    const uint32_t l0 = 2u * lx, m0 = 2u * ly;
                    const float r = (x0 < Wp && y0 < Hp) ? src[m0 * S + l0] : 0.0f;
                    const float g = (x0 + 1 < Wp && y0 < Hp) ? src[m0 * S + l0 + 1] : 0.0f;
                    const float b = (x0 < Wp && y0 + 1 < Hp) ? src[(m0 + 1) * S + l0] : 0.0f;
                    const float a = (x0 + 1 < Wp && y0 + 1 < Hp) ? src[(m0 + 1) * S + l0 + 1] : 0.0f;
                    v = fmin_nan(r, fmin_nan(g, fmin_nan(b, a)));
                } else {
                    uint32_t i0, i1, j0, j1;
                    vk_footprint(gx, Wk, Wp, i0, i1);
                    vk_footprint(gy, Hk, Hp, j0, j1);
                    // the footprint lies in this tile (power-of-two levels); clamp defensively
                    const uint32_t a0 = min(i0 - Xp, S - 1), a1 = min(i1 - Xp, S - 1);
                    const uint32_t b0 = min(j0 - Yp, S - 1), b1 = min(j1 - Yp, S - 1);
                    float m = __int_as_float(0x7fc00000);
                    m = fmin_nan(m, src[b0 * S + a0]);
                    m = fmin_nan(m, src[b0 * S + a1]);
                    m = fmin_nan(m, src[b1 * S + a0]);
                    m = fmin_nan(m, src[b1 * S + a1]);
                    v = m;
                }
                p.data[p.mipOffset[k] + static_cast<size_t>(gy) * Wk + gx] = v;
            }
            dst[idx] = v;
        }
        __syncthreads();
        float* t = src;
        src = dst;
        dst = t;
        S = Sk;
    }
}

// Counts the block's tile done in `done`, after the barrier that closes pyramid_tile. Thread 0's
// add has acquire-release semantics at GPU scope: it releases the tile the whole block wrote (the
// writes precede the barrier, the barrier precedes the add) and, in the block that finishes the
// build's last tile (tiles in all), acquires every other block's tile. That block builds the levels
// above mip 5 and then, with `ready` given, publishes the finished pyramid (a barrier, then thread 0
// stores 1 with release semantics); without `ready` it rewinds `done` for the next build. sA and sB
// as for pyramid_tile.
template <uint32_t MODE, int NT>
__device__ __forceinline__ void pyramid_tile_finish(const PyramidBuildParams& p, uint32_t tiles, unsigned int* done,
                                                    unsigned int* ready, float* sA, float* sB) {
    __shared__ unsigned int s_last;
    if (threadIdx.x == 0) s_last = atom_add_acq_rel_gpu(done, 1u) == tiles - 1u ? 1u : 0u;
    __syncthreads();
    if (s_last) {
        if (p.mipCount > kPyrInTileLevels + 1) top_levels<MODE, NT>(p, sA, kPyrSmemA, sB, kPyrSmemB);
        if (ready != nullptr) {
            __syncthreads();
            if (threadIdx.x == 0) st_release_gpu(ready, 1u);
        } else if (threadIdx.x == 0) {
            *done = 0u;
        }
    }
}

}  // namespace blz
