// Minimal Slang builtins for compiling the reference shader source
// `src/volumetric_filter.slang` as C++ on the host.  TEST INFRASTRUCTURE ONLY.
//
// oracle/build.py strips the Slang-only constructs from the shader
// (`[shader("compute")]`, `[numthreads(8, 8, 1)]`, the `: SV_DispatchThreadID`
// semantic) and gives every unsuffixed floating literal an `f` suffix (Slang
// floating literals are 32-bit, C++ ones are double); the rest compiles
// unchanged against this header.  The types below provide what the shader
// uses: float2/3/4 (.xyz, .w), int3, uint2/uint3 (.xy), float4x4 with
// mul(M, v), dot / normalize / max / pow / log / floor / clamp / lerp, and
// RWTexture3D<float4> whose stores round to fp16 when the bound image is
// rgba16f (the reference's froxel images, `src/main.cpp:1918-1924`).
//
// float4x4 holds 16 floats in the reference's MathLib::Mat4 order (element
// (col, row) at index col * 4 + row, `libs/math/include/math/matrix.hpp:26-47`),
// and mul(M, v) is the column-vector product, its four column terms summed
// left to right.
#pragma once
#include <cmath>
#include <cstdint>

typedef unsigned int uint;

struct int3;

struct uint2 {
    uint x, y;
};

struct float2 {
    float x, y;
    float2() = default;
    float2(float a, float b) : x(a), y(b) {}
    explicit float2(uint2 v) : x(float(v.x)), y(float(v.y)) {}
};

struct float3 {
    float x, y, z;
    float3() = default;
    float3(float a, float b, float c) : x(a), y(b), z(c) {}
    explicit float3(const int3& v);
};

struct uint3 {
    union {
        struct { uint x, y, z; };
        struct { uint2 xy; uint z_pad_; };
    };
    uint3() = default;
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};

struct int3 {
    int x, y, z;
    int3() = default;
    int3(int a, int b, int c) : x(a), y(b), z(c) {}
    explicit int3(const float3& v) : x(int(v.x)), y(int(v.y)), z(int(v.z)) {}
};

inline float3::float3(const int3& v) : x(float(v.x)), y(float(v.y)), z(float(v.z)) {}

// float4's .xyz: plain data (a member of the anonymous union) that converts to float3
struct float3_view {
    float x, y, z;
    operator float3() const { return float3(x, y, z); }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        struct { float3_view xyz; float w_pad_; };
    };
    float4() = default;
    float4(float a, float b, float c, float d) : x(a), y(b), z(c), w(d) {}
    float4(float2 v, float c, float d) : x(v.x), y(v.y), z(c), w(d) {}
    float4(float3 v, float d) : x(v.x), y(v.y), z(v.z), w(d) {}
};

struct float4x4 {
    float m[16];
};

inline float2 operator+(float2 a, float s) { return float2(a.x + s, a.y + s); }
inline float2 operator/(float2 a, float2 b) { return float2(a.x / b.x, a.y / b.y); }

inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator-(float3 a, float3 b) { return float3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }

inline float4 operator+(float4 a, float4 b) { return float4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
inline float4 operator/(float4 a, float s) { return float4(a.x / s, a.y / s, a.z / s, a.w / s); }
inline float4& operator+=(float4& a, const float4& b)
{
    a = a + b;
    return a;
}

inline int3 operator+(int3 a, int s) { return int3(a.x + s, a.y + s, a.z + s); }

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 normalize(float3 v) { return v / std::sqrt(dot(v, v)); }
inline float max(float a, float b) { return a > b ? a : b; }
inline float pow(float a, float b) { return std::pow(a, b); }
inline float log(float a) { return std::log(a); }
inline float3 floor(float3 v) { return float3(std::floor(v.x), std::floor(v.y), std::floor(v.z)); }
inline int clamp1(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline int3 clamp(int3 v, int3 lo, int3 hi)
{
    return int3(clamp1(v.x, lo.x, hi.x), clamp1(v.y, lo.y, hi.y), clamp1(v.z, lo.z, hi.z));
}
inline float4 lerp(float4 a, float4 b, float t)
{
    return float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
}
inline float4 mul(const float4x4& M, float4 v)
{
    float o[4];
    for (int r = 0; r < 4; ++r) o[r] = M.m[0 * 4 + r] * v.x + M.m[1 * 4 + r] * v.y + M.m[2 * 4 + r] * v.z + M.m[3 * 4 + r] * v.w;
    return float4(o[0], o[1], o[2], o[3]);
}

// Whether image stores round to fp16 (the reference's rgba16f froxel images).
extern bool g_slang_fp16_store;

inline float slang_store_round(float v)
{
    return g_slang_fp16_store ? static_cast<float>(static_cast<_Float16>(v)) : v;
}

struct Texel3 : float4 {
    float4* dst;
    explicit Texel3(float4* p) : float4(*p), dst(p) {}
    Texel3& operator=(const float4& v)
    {
        *dst = float4(slang_store_round(v.x), slang_store_round(v.y), slang_store_round(v.z), slang_store_round(v.w));
        return *this;
    }
};

template <class V> struct RWTexture3D {
    V* data = nullptr;
    int width = 0, height = 0;
    Texel3 operator[](uint3 p) const
    {
        return Texel3(data + (static_cast<long>(p.z) * height + p.y) * width + p.x);
    }
};
