// glsl_shim.h — TEST INFRASTRUCTURE. Just enough of GLSL's types, built-ins and resource objects
// to compile the reference's Vulkan cull, depth-pyramid and cluster compute shaders as C++ and run
// their main() serially on the CPU.
//
// What GLSL leaves to the implementation is fixed exactly as the oracle and the CUDA kernels fix
// it (the same conventions as oracle/ref_hlsl/hlsl_shim.h):
//   - each float operation is one IEEE round-to-nearest operation in source order (build with
//     -ffp-contract=off); mat4 * vec4 sums its four products left to right; length() sums the
//     squares left to right; sqrt and division are correctly rounded;
//   - floor(log2(x)) is exact (the exponent of x);
//   - min/max ignore a NaN operand, min keeps its first operand on ties;
//   - the depth-pyramid sampler of the reference (LINEAR filter, MIN reduction, NEAREST mip,
//     clamp to edge, LOD clamped to [0, 16]; src/Renderer/BlitzenVulkan/vulkanResources.cpp:51-55,
//     409-410) returns the minimum over the texels of the bilinear footprint that have a non-zero
//     weight: u = s * w - 0.5, texels floor(u) and floor(u) + 1 (the second only when the fraction
//     is above 0), each clamped to the edge, the same in t. This footprint is the one definition
//     here that is not the reference's own text: the reference leaves it to the sampler hardware;
//   - an image store outside the image is dropped;
//   - atomicAdd returns the previous value (serial execution makes every atomic sequence the
//     dispatch-order one).
#pragma once

#include <stdint.h>
#include <string.h>

typedef uint32_t uint;

// ------------------------------------------------------------------ scalars

inline float abs(float x) { return __builtin_fabsf(x); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }
inline float max(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}
inline float max(float a, int b) { return max(a, (float)b); }
inline float min(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
inline float floor_plain(float x) { return __builtin_floorf(x); }

// log2 followed by floor, evaluated exactly: floor(log2(x)) is the exponent of x.
struct Log2Of {
    float x;
};
inline Log2Of log2(float x) { return Log2Of{x}; }
inline float floor(Log2Of l) {
    const float x = l.x;
    if (x != x || x < 0.0f) return __builtin_nanf("");
    if (x == 0.0f) return -__builtin_inff();
    if (x == __builtin_inff()) return __builtin_inff();
    uint32_t bits;
    memcpy(&bits, &x, 4);
    const int e = (int)((bits >> 23) & 0xFFu);
    if (e == 0) {  // subnormal
        const uint32_t m = bits & 0x7FFFFFu;
        return (float)(-127 + (31 - __builtin_clz(m)) - 22);
    }
    return (float)(e - 127);
}
inline float floor(float x) { return __builtin_floorf(x); }

// ------------------------------------------------------------------ vectors

struct uvec2;
struct vec2 {
    float x, y;
    vec2() = default;
    vec2(float a, float b) : x(a), y(b) {}
    explicit vec2(float s) : x(s), y(s) {}
    explicit vec2(double s) : x((float)s), y((float)s) {}
    inline explicit vec2(uvec2 u);
};
inline vec2 operator+(vec2 a, vec2 b) { return vec2(a.x + b.x, a.y + b.y); }
inline vec2 operator/(vec2 a, vec2 b) { return vec2(a.x / b.x, a.y / b.y); }
inline vec2 operator*(vec2 a, float s) { return vec2(a.x * s, a.y * s); }
inline vec2 operator*(vec2 a, double s) { return a * (float)s; }  // a GLSL literal is a float

struct vec3 {
    float x, y, z;
    vec3() = default;
    vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
static_assert(sizeof(vec3) == 12, "vec3 is 12 bytes");
inline vec3 operator+(vec3 a, vec3 b) { return vec3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline vec3 operator-(vec3 a, vec3 b) { return vec3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline vec3 operator*(vec3 a, float s) { return vec3(a.x * s, a.y * s, a.z * s); }
inline vec3 operator*(float s, vec3 a) { return vec3(s * a.x, s * a.y, s * a.z); }
inline vec3 operator*(double s, vec3 a) { return (float)s * a; }

struct vec4 {
    float x, y, z, w;
    vec4() = default;
    vec4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    vec4(vec3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
    vec4(vec3 v, int d) : x(v.x), y(v.y), z(v.z), w((float)d) {}
    explicit vec4(float s) : x(s), y(s), z(s), w(s) {}
    vec3 xyz() const { return vec3(x, y, z); }
    vec2 xy() const { return vec2(x, y); }
    vec2 zw() const { return vec2(z, w); }
    vec4 xwzy() const { return vec4(x, w, z, y); }
};
static_assert(sizeof(vec4) == 16, "vec4 is 16 bytes");
inline vec4 operator*(vec4 a, vec4 b) { return vec4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline vec4 operator+(vec4 a, vec4 b) { return vec4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

struct uvec2 {
    uint32_t x, y;
};
inline vec2::vec2(uvec2 u) : x((float)u.x), y((float)u.y) {}
struct ivec2 {
    int32_t x, y;
    ivec2() = default;
    explicit ivec2(uvec2 u) : x((int32_t)u.x), y((int32_t)u.y) {}
};
struct uvec3 {
    uint32_t x, y, z;
    uvec2 xy() const { return uvec2{x, y}; }
};

inline float length(vec3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }
inline vec3 cross(vec3 a, vec3 b) {
    return vec3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

// Column-major as the engine uploads it; mat4 * vec4 treats the vector as a column.
struct mat4 {
    float m[16];
};
inline vec4 operator*(const mat4& M, vec4 v) {
    float o[4];
    for (int r = 0; r < 4; ++r) {
        float acc = M.m[r] * v.x;
        acc = acc + M.m[4 + r] * v.y;
        acc = acc + M.m[8 + r] * v.z;
        acc = acc + M.m[12 + r] * v.w;
        o[r] = acc;
    }
    return vec4(o[0], o[1], o[2], o[3]);
}

// ------------------------------------------------------------------ resources

// One R32F image, or a chain of them: level i is (max(1, width >> i), max(1, height >> i)) at
// data + offset[i]. A sampler bound to one level of a chain is a chain of one image.
struct sampler2D {
    const float* data = nullptr;
    uint32_t width = 0, height = 0, levels = 0;
    uint32_t offset[16] = {};
};

inline uint32_t level_dim(uint32_t base, uint32_t level) {
    const uint32_t d = base >> level;
    return d ? d : 1u;
}

inline long long texel_index(float f) {
    if (f != f) return 0;
    if (f < -1.0e18f) return -(1ll << 60);
    if (f > 1.0e18f) return 1ll << 60;
    return (long long)f;
}

// The MIN-reduction bilinear footprint at (s, t) of one level (see the header comment).
inline float min_footprint(const float* img, uint32_t w, uint32_t h, float s, float t) {
    const float u = s * (float)w - 0.5f;
    const float v = t * (float)h - 0.5f;
    const float fu = __builtin_floorf(u), fv = __builtin_floorf(v);
    const float au = u - fu, av = v - fv;
    const long long i0 = texel_index(fu), j0 = texel_index(fv);
    const long long i1 = (au > 0.0f) ? i0 + 1 : i0;
    const long long j1 = (av > 0.0f) ? j0 + 1 : j0;
    const long long xs[2] = {i0, i1}, ys[2] = {j0, j1};
    float m = __builtin_nanf("");
    for (int jy = 0; jy < 2; ++jy)
        for (int ix = 0; ix < 2; ++ix) {
            long long x = xs[ix], y = ys[jy];
            x = x < 0 ? 0 : (x > (long long)w - 1 ? (long long)w - 1 : x);
            y = y < 0 ? 0 : (y > (long long)h - 1 ? (long long)h - 1 : y);
            m = min(m, img[(uint64_t)y * w + (uint64_t)x]);
        }
    return m;
}

// textureLod with a NEAREST mip filter: the LOD clamped to [0, 16] (the sampler's minLod/maxLod),
// its nearest level (the LODs here are whole numbers or infinities), clamped to the chain.
inline vec4 textureLod(const sampler2D& s, vec2 uv, float lod) {
    float lam = lod;
    if (!(lam > 0.0f)) lam = 0.0f;
    if (lam > 16.0f) lam = 16.0f;
    uint32_t d = (uint32_t)lam;
    if (d > s.levels - 1u) d = s.levels - 1u;
    const float m = min_footprint(s.data + s.offset[d], level_dim(s.width, d), level_dim(s.height, d), uv.x, uv.y);
    return vec4(m, m, m, m);
}

// texture() in a compute shader samples level 0 of the bound image.
inline vec4 texture(const sampler2D& s, vec2 uv) { return textureLod(s, uv, 0.0f); }

struct image2D {
    float* data = nullptr;
    uint32_t width = 0, height = 0;
};
inline void imageStore(image2D& img, ivec2 at, vec4 v) {
    if (at.x < 0 || at.y < 0 || (uint32_t)at.x >= img.width || (uint32_t)at.y >= img.height) return;
    img.data[(uint64_t)(uint32_t)at.y * img.width + (uint32_t)at.x] = v.x;
}

inline uint atomicAdd(uint& dest, uint value) {
    const uint old = dest;
    dest = old + value;
    return old;
}
inline uint atomicAdd(uint& dest, int value) { return atomicAdd(dest, (uint)value); }

// GetComputeShaderGroupSize (src/BlitzenMathLibrary/blitML.h:64-67): N / threads + 1 groups.
inline uint32_t group_count(uint32_t n, uint32_t threads) { return n / threads + 1; }
