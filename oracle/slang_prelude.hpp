// Minimal Slang/HLSL builtins for compiling the reference shader source
// `src/svgf_denoise.slang` as C++ on the host.  TEST INFRASTRUCTURE ONLY.
//
// oracle/build.py strips the three Slang-only constructs from the shader
// (`[shader("compute")]`, `[numthreads(8, 8, 1)]` and the `: SV_DispatchThreadID`
// semantic) and compiles the rest unchanged against this header.  The types
// below provide exactly what the shader uses: float2/3/4 with the .rgb/.a/.r/.g
// swizzles, int2/uint2/uint3, dot/lerp/max/clamp/abs/exp/sqrt, and
// RWTexture2D<T> whose element stores round to fp16 when the bound image has an
// fp16 format (the reference binds rgba16f / rg16f images,
// `src/svgf_denoise.slang:61-94`).
#pragma once
#include <cmath>
#include <cstdint>

typedef unsigned int uint;

// An aggregate so that it may sit inside float4's anonymous union; the shader's
// `float3(a, b, c)` is then C++20 parenthesised aggregate initialisation.
struct float3 {
    float x, y, z;
};

inline float3 operator+(float3 a, float3 b) { return float3{a.x + b.x, a.y + b.y, a.z + b.z}; }
inline float3 operator*(float3 a, float s) { return float3{a.x * s, a.y * s, a.z * s}; }
inline float3 operator/(float3 a, float s) { return float3{a.x / s, a.y / s, a.z / s}; }
inline float3& operator+=(float3& a, float3 b)
{
    a = a + b;
    return a;
}

struct float2 {
    union {
        struct { float x, y; };
        struct { float r, g; };
    };
    float2() = default;
    float2(float a, float b) : x(a), y(b) {}
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        struct { float r, g, b, a; };
        struct { float3 rgb; float a_pad_; };
    };
    float4() = default;
    float4(float a0, float a1, float a2, float a3) : x(a0), y(a1), z(a2), w(a3) {}
    float4(float3 v, float a3) : x(v.x), y(v.y), z(v.z), w(a3) {}
};

struct uint2 {
    uint x, y;
};

struct uint3 {
    union {
        struct { uint x, y, z; };
        struct { uint2 xy; uint z_pad_; };
    };
};

struct int2 {
    int x, y;
    int2() = default;
    int2(int a, int b) : x(a), y(b) {}
    explicit int2(uint2 v) : x(int(v.x)), y(int(v.y)) {}
};

inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float lerp(float a, float b, float t) { return a + (b - a) * t; }
inline float max(float a, float b) { return a > b ? a : b; }
inline int clamp(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline float abs(float v) { return std::fabs(v); }
inline float exp(float v) { return std::exp(v); }
inline float sqrt(float v) { return std::sqrt(v); }

// Whether image stores round to fp16 (the reference's rgba16f / rg16f images).
extern bool g_slang_fp16_store;

inline float slang_store_round(float v)
{
    return g_slang_fp16_store ? static_cast<float>(static_cast<_Float16>(v)) : v;
}
inline float2 slang_store_round(float2 v) { return float2(slang_store_round(v.x), slang_store_round(v.y)); }
inline float4 slang_store_round(float4 v)
{
    return float4(slang_store_round(v.x), slang_store_round(v.y), slang_store_round(v.z), slang_store_round(v.w));
}

template <class V> struct Texel : V {
    V* dst;
    explicit Texel(V* p) : V(*p), dst(p) {}
    Texel& operator=(const V& v)
    {
        *dst = slang_store_round(v);
        return *this;
    }
};

template <class V> struct RWTexture2D {
    V* data = nullptr;
    int width = 0;
    Texel<V> operator[](int2 p) const { return Texel<V>(data + static_cast<long>(p.y) * width + p.x); }
};
