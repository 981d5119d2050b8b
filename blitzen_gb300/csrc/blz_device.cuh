// blz_device.cuh — device-side culling arithmetic and the single-pass compaction machinery.
//
// Arithmetic: every FP32 operation on a decision path is an explicit round-to-nearest intrinsic
// (__fmul_rn, __fadd_rn, __fsub_rn, __fdiv_rn, __fsqrt_rn), so the compiler can neither contract
// nor reorder them whatever the build flags. The operation order follows the reference shaders
// term by term (each helper cites its source; paths inside the Blitzen project).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/blz_cull.h"
#include "../../include/blz_types.h"

namespace blz {

#define BLZ_FM(a, b) __fmul_rn((a), (b))
#define BLZ_FA(a, b) __fadd_rn((a), (b))
#define BLZ_FS(a, b) __fsub_rn((a), (b))
#define BLZ_FD(a, b) __fdiv_rn((a), (b))

// ------------------------------------------------------------------ scalar conventions

// D3D float -> uint: NaN and x <= 0 give 0, x >= 2^32 gives UINT32_MAX, else truncation.
__device__ __forceinline__ uint32_t ftou(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xFFFFFFFFu;
    return static_cast<uint32_t>(x);
}

// floor(log2(x)) as uint: unbiased exponent for finite x >= 1 (always a normal number),
// 0 for x < 1 or NaN, UINT32_MAX for +inf.
__device__ __forceinline__ uint32_t floor_log2_u(float x) {
    if (!(x >= 1.0f)) return 0u;
    uint32_t bits = __float_as_uint(x);
    uint32_t e = (bits >> 23) & 0xFFu;
    if (e == 0xFFu) return 0xFFFFFFFFu;
    return e - 127u;
}

// floor(log2(x)) as float for the Vulkan form: NaN for NaN/negative, -inf for 0, +inf for inf.
__device__ __forceinline__ float floor_log2_f(float x) {
    if (isnan(x) || x < 0.0f) return __int_as_float(0x7fc00000);
    if (x == 0.0f) return -INFINITY;
    uint32_t bits = __float_as_uint(x);
    uint32_t e = (bits >> 23) & 0xFFu;
    if (e == 0xFFu) return INFINITY;
    if (e == 0u) {  // subnormal: exponent of the leading one
        uint32_t m = bits & 0x7FFFFFu;
        return static_cast<float>(-127 + (31 - __clz(m)) - 22);
    }
    return static_cast<float>(static_cast<int>(e) - 127);
}

__device__ __forceinline__ float fmax_nan(float a, float b) {
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    return (b > a) ? b : a;
}

__device__ __forceinline__ float fmin_nan(float a, float b) {
    if (isnan(a)) return b;
    if (isnan(b)) return a;
    return (b < a) ? b : a;
}

// ------------------------------------------------------------------ sphere math

struct Vec3 {
    float x, y, z;
};

// v + 2 * cross(q.xyz, cross(q.xyz, v) + q.w * v)
// ShaderBuffers.glsl:197-200, hlslMath.hlsl:1-4
__device__ __forceinline__ Vec3 rotate_quat(Vec3 v, float4 q) {
    float c1x = BLZ_FS(BLZ_FM(q.y, v.z), BLZ_FM(q.z, v.y));
    float c1y = BLZ_FS(BLZ_FM(q.z, v.x), BLZ_FM(q.x, v.z));
    float c1z = BLZ_FS(BLZ_FM(q.x, v.y), BLZ_FM(q.y, v.x));
    float tx = BLZ_FA(c1x, BLZ_FM(q.w, v.x));
    float ty = BLZ_FA(c1y, BLZ_FM(q.w, v.y));
    float tz = BLZ_FA(c1z, BLZ_FM(q.w, v.z));
    float c2x = BLZ_FS(BLZ_FM(q.y, tz), BLZ_FM(q.z, ty));
    float c2y = BLZ_FS(BLZ_FM(q.z, tx), BLZ_FM(q.x, tz));
    float c2z = BLZ_FS(BLZ_FM(q.x, ty), BLZ_FM(q.y, tx));
    return Vec3{BLZ_FA(v.x, BLZ_FM(2.0f, c2x)), BLZ_FA(v.y, BLZ_FM(2.0f, c2y)), BLZ_FA(v.z, BLZ_FM(2.0f, c2z))};
}

// The view matrix rows that produce view-space x, y, z (column-major storage):
// r_k = (m[k], m[4+k], m[8+k], m[12+k]).
struct ViewRows {
    float4 r0, r1, r2;
};

// view * vec4(p, 1), terms summed left to right. The last term, m[12+k] * 1, is m[12+k] itself
// (multiplying by one is exact; a NaN stays a NaN), so it is added without the multiply.
__device__ __forceinline__ Vec3 view_transform(const ViewRows& m, Vec3 p) {
    Vec3 o;
    o.x = BLZ_FA(BLZ_FA(BLZ_FA(BLZ_FM(m.r0.x, p.x), BLZ_FM(m.r0.y, p.y)), BLZ_FM(m.r0.z, p.z)), m.r0.w);
    o.y = BLZ_FA(BLZ_FA(BLZ_FA(BLZ_FM(m.r1.x, p.x), BLZ_FM(m.r1.y, p.y)), BLZ_FM(m.r1.z, p.z)), m.r1.w);
    o.z = BLZ_FA(BLZ_FA(BLZ_FA(BLZ_FM(m.r2.x, p.x), BLZ_FM(m.r2.y, p.y)), BLZ_FM(m.r2.z, p.z)), m.r2.w);
    return o;
}

// Model sphere centre -> world (RotateQuat * scale + pos); hlslMath.hlsl:6-10.
__device__ __forceinline__ Vec3 model_to_world(Vec3 c, float4 posScale, float4 q) {
    Vec3 r = rotate_quat(c, q);
    return Vec3{BLZ_FA(BLZ_FM(r.x, posScale.w), posScale.x), BLZ_FA(BLZ_FM(r.y, posScale.w), posScale.y),
                BLZ_FA(BLZ_FM(r.z, posScale.w), posScale.z)};
}

// Per-view constants the kernels read, unpacked once per block from BlzCameraViewData.
struct ViewConsts {
    ViewRows rows;
    float frustumRight, frustumLeft, frustumTop, frustumBottom;
    float proj0, proj5, zNear, zFar;
    float pyramidWidth, pyramidHeight, lodTarget;
    float camX, camY, camZ;
};

__device__ __forceinline__ ViewConsts load_view(const BlzCameraViewData& v) {
    ViewConsts c;
    c.rows.r0 = make_float4(v.viewMatrix[0], v.viewMatrix[4], v.viewMatrix[8], v.viewMatrix[12]);
    c.rows.r1 = make_float4(v.viewMatrix[1], v.viewMatrix[5], v.viewMatrix[9], v.viewMatrix[13]);
    c.rows.r2 = make_float4(v.viewMatrix[2], v.viewMatrix[6], v.viewMatrix[10], v.viewMatrix[14]);
    c.frustumRight = v.frustumRight;
    c.frustumLeft = v.frustumLeft;
    c.frustumTop = v.frustumTop;
    c.frustumBottom = v.frustumBottom;
    c.proj0 = v.proj0;
    c.proj5 = v.proj5;
    c.zNear = v.zNear;
    c.zFar = v.zFar;
    c.pyramidWidth = v.pyramidWidth;
    c.pyramidHeight = v.pyramidHeight;
    c.lodTarget = v.lodTarget;
    c.camX = v.position[0];
    c.camY = v.position[1];
    c.camZ = v.position[2];
    return c;
}

// hlslMath.hlsl:13-27 (FrustumCheck), CullingShaderData.glsl:52-55.
__device__ __forceinline__ bool frustum_check(Vec3 c, float r, const ViewConsts& v) {
    bool vis = BLZ_FS(BLZ_FM(c.z, v.frustumLeft), BLZ_FM(fabsf(c.x), v.frustumRight)) > -r;
    vis = vis && (BLZ_FS(BLZ_FM(c.z, v.frustumBottom), BLZ_FM(fabsf(c.y), v.frustumTop)) > -r);
    vis = vis && (BLZ_FA(c.z, r) > v.zNear) && (BLZ_FS(c.z, r) < v.zFar);
    return vis;
}

// hlslMath.hlsl:30-56 (ProjectSphere), CullingShaderData.glsl:8-33. aabb in UV space, y flipped.
__device__ __forceinline__ bool project_sphere(Vec3 c, float r, float znear, float P00, float P11, float4& aabb) {
    if (c.z < BLZ_FA(r, znear)) return false;
    float sx = BLZ_FM(c.x, r), sy = BLZ_FM(c.y, r), sz = BLZ_FM(c.z, r);
    float zp = BLZ_FS(BLZ_FM(c.z, c.z), BLZ_FM(r, r));
    float xr = __fsqrt_rn(BLZ_FA(BLZ_FM(c.x, c.x), zp));
    float xmin = BLZ_FD(BLZ_FS(BLZ_FM(xr, c.x), sz), BLZ_FA(BLZ_FM(xr, c.z), sx));
    float xmax = BLZ_FD(BLZ_FA(BLZ_FM(xr, c.x), sz), BLZ_FS(BLZ_FM(xr, c.z), sx));
    float yr = __fsqrt_rn(BLZ_FA(BLZ_FM(c.y, c.y), zp));
    float ymin = BLZ_FD(BLZ_FS(BLZ_FM(yr, c.y), sz), BLZ_FA(BLZ_FM(yr, c.z), sy));
    float ymax = BLZ_FD(BLZ_FA(BLZ_FM(yr, c.y), sz), BLZ_FS(BLZ_FM(yr, c.z), sy));
    float a0 = BLZ_FM(xmin, P00), a1 = BLZ_FM(ymin, P11), a2 = BLZ_FM(xmax, P00), a3 = BLZ_FM(ymax, P11);
    aabb.x = BLZ_FA(BLZ_FM(a0, 0.5f), 0.5f);
    aabb.y = BLZ_FA(BLZ_FM(a3, -0.5f), 0.5f);
    aabb.z = BLZ_FA(BLZ_FM(a2, 0.5f), 0.5f);
    aabb.w = BLZ_FA(BLZ_FM(a1, -0.5f), 0.5f);
    return true;
}

// Hi-Z pyramid as the kernels see it.
struct PyramidView {
    const float* data;
    uint32_t width, height, mipCount, mode;
    uint32_t mipOffset[BLZ_PYRAMID_MAX_MIPS];
};

__device__ __forceinline__ uint32_t mip_dim(uint32_t base, uint32_t level) {
    uint32_t d = base >> level;
    return d ? d : 1u;
}

// A pyramid texel load. COH: the pyramid was written during this launch (the one-call frame
// kernel builds it), so the load goes to L2 (coherent), not through the read-only path.
template <bool COH>
__device__ __forceinline__ float pyr_ld(const float* a) {
    return COH ? __ldcg(a) : __ldg(a);
}

template <bool COH = false>
__device__ __forceinline__ float pyr_load(const PyramidView& p, uint32_t level, uint32_t x, uint32_t y) {
    if (level >= p.mipCount) return 0.0f;
    uint32_t w = mip_dim(p.width, level), h = mip_dim(p.height, level);
    if (x >= w || y >= h) return 0.0f;
    return pyr_ld<COH>(p.data + p.mipOffset[level] + static_cast<size_t>(y) * w + x);
}

// hlslMath.hlsl:58-78 (OcclusionCheck): one-texel Load at mip floor(log2(max extent)).
template <bool COH = false>
__device__ __forceinline__ bool occlusion_d3d12(float4 a, const PyramidView& p, const ViewConsts& v, Vec3 c, float r) {
    uint32_t pw = ftou(v.pyramidWidth), ph = ftou(v.pyramidHeight);
    float width = BLZ_FM(BLZ_FS(a.z, a.x), static_cast<float>(pw));
    float height = BLZ_FM(BLZ_FS(a.w, a.y), static_cast<float>(ph));
    uint32_t level = floor_log2_u(fmax_nan(width, height));
    float depth = 0.0f;
    if (level < p.mipCount) {
        uint32_t mw = pw >> level, mh = ph >> level;
        mw = mw ? mw : 1u;
        mh = mh ? mh : 1u;
        float sw = BLZ_FM(static_cast<float>(mw), 0.5f), sh = BLZ_FM(static_cast<float>(mh), 0.5f);
        float ax = BLZ_FM(a.x, sw), ay = BLZ_FM(a.y, sh), az = BLZ_FM(a.z, sw), aw = BLZ_FM(a.w, sh);
        depth = pyr_load<COH>(p, level, ftou(BLZ_FA(ax, az)), ftou(BLZ_FA(ay, aw)));
    }
    float depthSphere = BLZ_FD(v.zNear, BLZ_FS(c.z, r));
    return depthSphere > depth;
}

// Texel index of a floored coordinate: NaN -> 0, huge magnitudes saturate (then clamp to edge).
__device__ __forceinline__ long long to_index(float f) {
    if (isnan(f)) return 0;
    if (f < -1.0e18f) return -(1ll << 60);
    if (f > 1.0e18f) return 1ll << 60;
    return static_cast<long long>(f);
}

// MIN-reduction bilinear footprint (LINEAR + MIN sampler, clamp to edge) at (s, t) of one mip.
template <bool COH = false>
__device__ __forceinline__ float min_footprint(const float* img, uint32_t w, uint32_t h, float s, float t) {
    float u = BLZ_FS(BLZ_FM(s, static_cast<float>(w)), 0.5f);
    float vv = BLZ_FS(BLZ_FM(t, static_cast<float>(h)), 0.5f);
    float fu = floorf(u), fv = floorf(vv);
    float au = BLZ_FS(u, fu), av = BLZ_FS(vv, fv);
    long long i0 = to_index(fu), j0 = to_index(fv);
    long long i1 = (au > 0.0f) ? i0 + 1 : i0;
    long long j1 = (av > 0.0f) ? j0 + 1 : j0;
    long long xs[2] = {i0, i1}, ys[2] = {j0, j1};
    float m = __int_as_float(0x7fc00000);
#pragma unroll
    for (int jy = 0; jy < 2; ++jy)
#pragma unroll
        for (int ix = 0; ix < 2; ++ix) {
            long long x = xs[ix], y = ys[jy];
            x = x < 0 ? 0 : (x > (long long)w - 1 ? (long long)w - 1 : x);
            y = y < 0 ? 0 : (y > (long long)h - 1 ? (long long)h - 1 : y);
            m = fmin_nan(m, pyr_ld<COH>(img + static_cast<size_t>(y) * w + static_cast<size_t>(x)));
        }
    return m;
}

// CullingShaderData.glsl:60-73 (OcclusionCullingPassed) with the MIN sampler of
// vulkanResources.cpp:51-55 (NEAREST mip, LOD clamped to [0, 16] and to the last mip).
template <bool COH = false>
__device__ __forceinline__ bool occlusion_vulkan(float4 a, const PyramidView& p, const ViewConsts& v, Vec3 c, float r) {
    float width = BLZ_FM(BLZ_FS(a.z, a.x), v.pyramidWidth);
    float height = BLZ_FM(BLZ_FS(a.w, a.y), v.pyramidHeight);
    float level = floor_log2_f(fmax_nan(width, height));
    float lam = level;
    if (!(lam > 0.0f)) lam = 0.0f;
    if (lam > 16.0f) lam = 16.0f;
    uint32_t d = static_cast<uint32_t>(lam);
    if (d > p.mipCount - 1u) d = p.mipCount - 1u;
    uint32_t w = mip_dim(p.width, d), h = mip_dim(p.height, d);
    float s = BLZ_FM(BLZ_FA(a.x, a.z), 0.5f), t = BLZ_FM(BLZ_FA(a.y, a.w), 0.5f);
    float depth = min_footprint<COH>(p.data + p.mipOffset[d], w, h, s, t);
    float depthSphere = BLZ_FD(v.zNear, BLZ_FS(c.z, r));
    return depthSphere > depth;
}

template <bool COH = false>
__device__ __forceinline__ bool occlusion(float4 a, const PyramidView& p, const ViewConsts& v, Vec3 c, float r) {
    return (p.mode == BLZ_HIZ_VULKAN) ? occlusion_vulkan<COH>(a, p, v, c, r) : occlusion_d3d12<COH>(a, p, v, c, r);
}

// Distance-to-surface threshold for LOD selection; CullingShaderData.glsl:105-106,
// cullBuffers.hlsl:44-45.
__device__ __forceinline__ float lod_threshold(Vec3 c, float r, float scale, float lodTarget) {
    float len = __fsqrt_rn(BLZ_FA(BLZ_FA(BLZ_FM(c.x, c.x), BLZ_FM(c.y, c.y)), BLZ_FM(c.z, c.z)));
    float d = BLZ_FS(len, r);
    float distance = (d > 0.0f) ? d : 0.0f;
    return BLZ_FD(BLZ_FM(distance, lodTarget), scale);
}

// ------------------------------------------------------------------ scene tables

struct SceneTables {
    const BlzRenderObject* objects;
    const BlzMeshTransform* transforms;
    const BlzPrimitiveSurface* surfaces;
    const BlzLodData* lods;
    const BlzCluster* clusters;
    uint32_t transformCount, surfaceCount, lodCount, clusterCount;
    const BlzMeshTransform* dynRows;  // bound dynamic rows: transforms [0, dynCount) are read here
    uint32_t dynCount, pad0;
};

// Scratch of the single-pass kernels (one per context, zeroed once at creation).
//   ticket: next tile id to hand out; epoch: tag of the current launch's tile states.
struct Scratch {
    unsigned int ticket;
    unsigned int epoch;
    unsigned int doneBlocks;
    unsigned int pyrDone;        // pyramid build: tiles finished (zero between builds)
    unsigned int status;         // BLZ_FLAG_* bits
    unsigned int frameTicket;    // one-call frame: next pyramid tile to hand out (zero between frames)
    unsigned int frameTilesDone; // one-call frame: pyramid tiles finished (zero between frames)
    unsigned int frameReady;     // one-call frame: 1 once the pyramid is complete (zero between frames)
    unsigned int pad1[24];       // keep the state array on its own 128-byte lines
    unsigned long long state[1]; // [maxTiles] tile states: epoch << 32 | flag << 30 | value
};

constexpr uint32_t kStateAggregate = 1u;
constexpr uint32_t kStatePrefix = 2u;
constexpr uint32_t kValueMask = (1u << 30) - 1u;

__device__ __forceinline__ unsigned long long pack_state(uint32_t epoch, uint32_t flag, uint32_t value) {
    return (static_cast<unsigned long long>(epoch) << 32) | (static_cast<unsigned long long>(flag) << 30) |
           (value & kValueMask);
}

__device__ __forceinline__ void store_state(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

__device__ __forceinline__ unsigned long long load_state(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}


// One MeshTransform {pos.xyz, scale, quat.xyzw} in a single 256-bit read-only load (the table
// is 32-byte aligned, checked on upload).
__device__ __forceinline__ void ldg_transform(const BlzMeshTransform* t, float4& posScale, float4& q) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(posScale.x), "=f"(posScale.y), "=f"(posScale.z), "=f"(posScale.w), "=f"(q.x), "=f"(q.y), "=f"(q.z),
          "=f"(q.w)
        : "l"(t));
}

// Transform `tid` of the scene, from the bound dynamic rows when tid < dynCount (device or pinned
// host memory), else from the resident table: a pointer select, then one 32-byte load (both are
// 32-byte aligned).
__device__ __forceinline__ void load_transform(const SceneTables& sc, uint32_t tid, float4& posScale, float4& q) {
    const BlzMeshTransform* base = tid < sc.dynCount ? sc.dynRows : sc.transforms;
    ldg_transform(base + tid, posScale, q);
}

// Programmatic dependent launch. A kernel launched with programmatic stream serialization may be
// scheduled while the kernel before it on the stream is still finishing; pdl_wait() holds it,
// before it touches any memory, until that kernel has completed and its writes are visible (a
// kernel launched without the attribute passes straight through). pdl_launch_next() lets the
// next kernel on the stream be scheduled now, to wait in its own pdl_wait().
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_launch_next() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

__device__ __forceinline__ void st_release_gpu(unsigned int* p, unsigned int v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned int atom_add_acq_rel_gpu(unsigned int* p, unsigned int v) {
    unsigned int old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}

__device__ __forceinline__ unsigned int ld_acquire_gpu(const unsigned int* p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

}  // namespace blz
