// hlsl_shim.h — TEST INFRASTRUCTURE. Just enough of HLSL's types, intrinsics and resource objects
// to compile the reference's D3D12 cull shaders as C++ and run their csMain serially on the CPU.
//
// The shim fixes what HLSL leaves to the GPU exactly as the oracle and the CUDA kernels do:
// each float operation is one IEEE round-to-nearest operation in source order (build with
// -ffp-contract=off), mul() sums its four products left to right, floor(log2(x)) is exact,
// float->uint is the D3D conversion (NaN/negative -> 0, saturating), shifts use the low 5 bits,
// min/max ignore a NaN operand and min keeps its first operand on ties, out-of-range buffer and
// texture reads return 0 and out-of-range writes are dropped, and InterlockedAdd returns the
// previous value (serial execution makes every atomic sequence the dispatch-order one).
//
// No math header is included on purpose: the shader's unqualified sqrt/log2/floor/abs/min/max
// must resolve to the functions below and nothing else.
#pragma once

#include <stdint.h>
#include <string.h>

// ------------------------------------------------------------------ scalars

inline uint32_t d3d_ftou(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 4294967296.0f) return 0xFFFFFFFFu;
    return (uint32_t)f;
}

struct uint {
    uint32_t v;
    uint() = default;
    constexpr uint(uint32_t x) : v(x) {}
    constexpr uint(int x) : v((uint32_t)x) {}
    uint(float f) : v(d3d_ftou(f)) {}
    uint(double d) : v(d3d_ftou((float)d)) {}
    constexpr operator uint32_t() const { return v; }
    uint& operator++() { ++v; return *this; }
    uint& operator+=(uint o) { v += o.v; return *this; }
};
static_assert(sizeof(uint) == 4, "uint is 32 bits");

inline uint operator>>(uint a, uint b) { return uint(a.v >> (b.v & 31u)); }
inline uint operator>>(uint a, int b) { return uint(a.v >> ((uint32_t)b & 31u)); }
inline uint operator<<(uint a, int b) { return uint(a.v << ((uint32_t)b & 31u)); }
inline float operator*(uint a, float b) { return (float)a.v * b; }
inline float operator*(float a, uint b) { return a * (float)b.v; }

inline float abs(float x) { return __builtin_fabsf(x); }
inline float sqrt(float x) { return __builtin_sqrtf(x); }

inline float max(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b > a) ? b : a;
}
inline float min(float a, float b) {
    if (a != a) return b;
    if (b != b) return a;
    return (b < a) ? b : a;
}
inline uint max(uint a, uint b) { return a.v > b.v ? a : b; }
inline uint max(unsigned a, uint b) { return max(uint(a), b); }

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
    int e = (int)((bits >> 23) & 0xFFu);
    if (e == 0) {  // subnormal
        uint32_t m = bits & 0x7FFFFFu;
        return (float)(-127 + (31 - __builtin_clz(m)) - 22);
    }
    return (float)(e - 127);
}

// ------------------------------------------------------------------ vectors

struct float2;
union float3;
union float4;

template <int A, int B>
struct Swz2 {
    float e[4];
    inline operator float2() const;
};
template <int A, int B, int C>
struct Swz3 {
    float e[4];
    inline operator float3() const;
};
template <int A, int B, int C, int D>
struct Swz4 {
    float e[4];
    inline operator float4() const;
};

struct float2 {
    float x, y;
    float2() = default;
    float2(float a, float b) : x(a), y(b) {}
};
inline float2 operator+(float2 a, float2 b) { return float2(a.x + b.x, a.y + b.y); }

union float3 {
    struct { float x, y, z; };
    struct { float r, g, b; };
    float3() = default;
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
};
static_assert(sizeof(float3) == 12, "float3 is 12 bytes");

union float4 {
    struct { float x, y, z, w; };
    struct { float r, g, b, a; };
    Swz3<0, 1, 2> xyz;
    Swz2<0, 1> xy;
    Swz2<2, 3> zw;
    Swz4<0, 3, 2, 1> xwzy;
    float e[4];
    float4() = default;
    float4(float a_, float b_, float c_, float d_) : x(a_), y(b_), z(c_), w(d_) {}
    float4(float3 v, float d_) : x(v.x), y(v.y), z(v.z), w(d_) {}
};
static_assert(sizeof(float4) == 16, "float4 is 16 bytes");

template <int A, int B>
inline Swz2<A, B>::operator float2() const { return float2(e[A], e[B]); }
template <int A, int B, int C>
inline Swz3<A, B, C>::operator float3() const { return float3(e[A], e[B], e[C]); }
template <int A, int B, int C, int D>
inline Swz4<A, B, C, D>::operator float4() const { return float4(e[A], e[B], e[C], e[D]); }

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator*(double s, float3 a) { return (float)s * a; }  // HLSL literal adopts float
inline float4 operator*(float4 a, float4 b) { return float4(a.x * b.x, a.y * b.y, a.z * b.z, a.w * b.w); }
inline float4 operator+(float4 a, float4 b) { return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }

inline float length(float3 v) { return sqrt(v.x * v.x + v.y * v.y + v.z * v.z); }

inline float3 cross(float3 a, float3 b) {
    return float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}

struct uint2 {
    uint x, y;
    uint2() = default;
    uint2(uint a, uint b) : x(a), y(b) {}
    uint2(int a, int b) : x(a), y(b) {}
};
inline uint2 operator<<(uint2 a, int s) { return uint2(a.x << s, a.y << s); }
inline uint2 operator+(uint2 a, uint2 b) { return uint2(uint(a.x.v + b.x.v), uint(a.y.v + b.y.v)); }

struct uint3 {
    uint x, y, z;
    uint2 xy;
    uint3() = default;
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c), xy(a, b) {}
    uint3(uint2 p, uint c) : x(p.x), y(p.y), z(c), xy(p) {}
    uint3(float2 p, uint c) : x(p.x), y(p.y), z(c), xy(x, y) {}  // float -> uint per component
};

// Column-major storage as uploaded from the engine's matrices; mul(M, v) treats v as a column.
struct float4x4 {
    float m[16];
};
inline float4 mul(const float4x4& M, float4 v) {
    float o[4];
    for (int r = 0; r < 4; ++r) {
        float acc = M.m[r] * v.x;
        acc = acc + M.m[4 + r] * v.y;
        acc = acc + M.m[8 + r] * v.z;
        acc = acc + M.m[12 + r] * v.w;
        o[r] = acc;
    }
    return float4(o[0], o[1], o[2], o[3]);
}

// ------------------------------------------------------------------ resources

template <typename T>
struct StructuredBuffer {
    const T* p = nullptr;
    uint32_t n = 0;
    T zero{};
    void bind(const void* ptr, uint32_t count) { p = static_cast<const T*>(ptr); n = count; }
    const T& operator[](uint32_t i) const { return i < n ? p[i] : zero; }
};

template <typename T>
struct RWStructuredBuffer {
    T* p = nullptr;
    uint32_t n = 0;
    T sink{};
    void bind(void* ptr, uint32_t count) { p = static_cast<T*>(ptr); n = count; }
    T& operator[](uint32_t i) {
        if (i < n) return p[i];
        memset(&sink, 0, sizeof sink);  // dropped write / zero read
        return sink;
    }
};

template <typename T>
using RWBuffer = RWStructuredBuffer<T>;

inline void InterlockedAdd(uint& dest, int value, uint& original) {
    original = dest;
    dest = uint(dest.v + (uint32_t)value);
}

// A mip chain of R32F texels.
struct MipChain {
    const float* data = nullptr;
    uint32_t width = 0, height = 0, mips = 0;
    uint32_t offset[16] = {};
};

template <typename T>
struct Texture2D {
    MipChain c;
    float4 Load(uint3 at) const {
        const uint32_t mip = at.z;
        if (mip >= c.mips) return float4(0.f, 0.f, 0.f, 0.f);
        uint32_t w = c.width >> mip, h = c.height >> mip;
        w = w ? w : 1u;
        h = h ? h : 1u;
        if ((uint32_t)at.x >= w || (uint32_t)at.y >= h) return float4(0.f, 0.f, 0.f, 0.f);
        const float v = c.data[c.offset[mip] + (uint64_t)(uint32_t)at.y * w + (uint32_t)at.x];
        return float4(v, v, v, v);
    }
};

struct TexelRef {
    float* p;
    TexelRef& operator=(float4 v) {
        if (p) *p = v.r;
        return *this;
    }
};

template <typename T>
struct RWTexture2D {
    float* data = nullptr;
    uint32_t width = 0, height = 0;
    TexelRef operator[](uint2 at) {
        if ((uint32_t)at.x >= width || (uint32_t)at.y >= height) return TexelRef{nullptr};
        return TexelRef{data + (uint64_t)(uint32_t)at.y * width + (uint32_t)at.x};
    }
};

// GetComputeShaderGroupSize (src/BlitzenMathLibrary/blitML.h:64-67): N / threads + 1 groups.
inline uint32_t group_count(uint32_t n, uint32_t threads) { return n / threads + 1; }
