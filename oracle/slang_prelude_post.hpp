// Minimal Slang builtins for compiling the reference shader sources
// `src/bloom_downsample.slang` and `src/postprocess.slang` as C++ on the host.
// TEST INFRASTRUCTURE ONLY.
//
// oracle/build.py strips the Slang-only constructs from the shaders
// (`[shader("compute")]`, `[numthreads(8, 8, 1)]`, the `: SV_DispatchThreadID`
// semantics) and gives every unsuffixed floating literal an `f` suffix (Slang
// floating literals are 32-bit); the rest compiles unchanged against this
// header.  The types below provide what the two shaders use: float2/3/4 with
// .rgb / .r .g .b, int2 / uint2 / uint3 arithmetic, float3x3 built from its
// rows with mul(M, v), dot / max / min / clamp / step / saturate / pow / lerp,
// and RWTexture2D<float4> with GetDimensions and a per-image store conversion:
// none, binary16 (the reference's rgba16f HDR and bloom images) or 8-bit UNORM
// with round-to-nearest-even (the B8G8R8A8_UNORM swapchain image,
// `src/swapchain.cpp:26-40`).
#pragma once
#include <cmath>
#include <cstdint>

typedef unsigned int uint;

struct int2;
struct uint2;

struct float2 {
    float x, y;
    float2() = default;
    float2(float a, float b) : x(a), y(b) {}
    explicit float2(const uint2& v);
};

// plain-data views (members of anonymous unions) that convert to the vector types
struct float3_data {
    union {
        struct { float x, y, z; };
        struct { float r, g, b; };
    };
};
struct uint2_data {
    uint x, y;
};

struct float3 : float3_data {
    float3() = default;
    float3(float a, float b, float c) { x = a; y = b; z = c; }
    float3(const float3_data& v) { x = v.x; y = v.y; z = v.z; }
};

struct float4 {
    union {
        struct { float x, y, z, w; };
        struct { float3_data rgb; float a; };
    };
    float4() = default;
    float4(float a0, float a1, float a2, float a3) : x(a0), y(a1), z(a2), w(a3) {}
    float4(float3 v, float a3) : x(v.x), y(v.y), z(v.z), w(a3) {}
};

struct uint2 {
    uint x, y;
    uint2() = default;
    uint2(uint a, uint b) : x(a), y(b) {}
    uint2(const uint2_data& v) : x(v.x), y(v.y) {}
    explicit uint2(const int2& v);
};

struct int2 {
    int x, y;
    int2() = default;
    int2(int a, int b) : x(a), y(b) {}
    explicit int2(const uint2& v) : x(int(v.x)), y(int(v.y)) {}
    explicit int2(const float2& v) : x(int(v.x)), y(int(v.y)) {}
};

inline float2::float2(const uint2& v) : x(float(v.x)), y(float(v.y)) {}
inline uint2::uint2(const int2& v) : x(uint(v.x)), y(uint(v.y)) {}

struct uint3 {
    union {
        struct { uint x, y, z; };
        struct { uint2_data xy; uint z_pad_; };
    };
    uint3() = default;
    uint3(uint a, uint b, uint c) : x(a), y(b), z(c) {}
};

struct float3x3 {
    float m[3][3];  // rows
    float3x3(float a, float b, float c, float d, float e, float f, float g, float h, float i)
    {
        m[0][0] = a; m[0][1] = b; m[0][2] = c;
        m[1][0] = d; m[1][1] = e; m[1][2] = f;
        m[2][0] = g; m[2][1] = h; m[2][2] = i;
    }
};

// float2
inline float2 operator+(float2 a, float s) { return float2(a.x + s, a.y + s); }
inline float2 operator-(float2 a, float s) { return float2(a.x - s, a.y - s); }
inline float2 operator*(float2 a, float s) { return float2(a.x * s, a.y * s); }
inline float2 operator*(float2 a, float2 b) { return float2(a.x * b.x, a.y * b.y); }
inline float2 operator/(float2 a, float2 b) { return float2(a.x / b.x, a.y / b.y); }
inline float dot(float2 a, float2 b) { return a.x * b.x + a.y * b.y; }

// float3
inline float3 operator+(float3 a, float3 b) { return float3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline float3 operator+(float3 a, float s) { return float3(a.x + s, a.y + s, a.z + s); }
inline float3 operator-(float3 a, float s) { return float3(a.x - s, a.y - s, a.z - s); }
inline float3 operator*(float3 a, float3 b) { return float3(a.x * b.x, a.y * b.y, a.z * b.z); }
inline float3 operator*(float3 a, float s) { return float3(a.x * s, a.y * s, a.z * s); }
inline float3 operator*(float s, float3 a) { return float3(s * a.x, s * a.y, s * a.z); }
inline float3 operator/(float3 a, float3 b) { return float3(a.x / b.x, a.y / b.y, a.z / b.z); }
inline float3 operator/(float3 a, float s) { return float3(a.x / s, a.y / s, a.z / s); }
inline float3& operator+=(float3& a, float3 b)
{
    a = a + b;
    return a;
}
inline float3& operator*=(float3& a, float s)
{
    a = a * s;
    return a;
}
inline float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float3 max(float3 a, float3 b)
{
    return float3(a.x > b.x ? a.x : b.x, a.y > b.y ? a.y : b.y, a.z > b.z ? a.z : b.z);
}
inline float saturate(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
inline float3 saturate(float3 v) { return float3(saturate(v.x), saturate(v.y), saturate(v.z)); }
inline float3 lerp(float3 a, float3 b, float t) { return float3(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t); }
inline float3 mul(const float3x3& M, float3 v)
{
    return float3(M.m[0][0] * v.x + M.m[0][1] * v.y + M.m[0][2] * v.z, M.m[1][0] * v.x + M.m[1][1] * v.y + M.m[1][2] * v.z,
                  M.m[2][0] * v.x + M.m[2][1] * v.y + M.m[2][2] * v.z);
}

// scalars
inline float max(float a, float b) { return a > b ? a : b; }
inline float step(float edge, float x) { return x >= edge ? 1.0f : 0.0f; }
inline float pow(float a, float b) { return std::pow(a, b); }

// integer vectors
inline uint2 operator*(uint2 a, int s) { return uint2(a.x * uint(s), a.y * uint(s)); }
inline uint2 operator+(uint2 a, uint2 b) { return uint2(a.x + b.x, a.y + b.y); }
inline uint2 operator/(uint2 a, int s) { return uint2(a.x / uint(s), a.y / uint(s)); }
inline uint2 min(uint2 a, uint2 b) { return uint2(a.x < b.x ? a.x : b.x, a.y < b.y ? a.y : b.y); }
inline int2 operator+(int2 a, int2 b) { return int2(a.x + b.x, a.y + b.y); }
inline int2 operator-(int2 a, int2 b) { return int2(a.x - b.x, a.y - b.y); }
inline int2 operator/(int2 a, int s) { return int2(a.x / s, a.y / s); }
inline int clamp1(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }
inline int2 clamp(int2 v, int2 lo, int2 hi) { return int2(clamp1(v.x, lo.x, hi.x), clamp1(v.y, lo.y, hi.y)); }

// Store conversion of one image.
enum SlangStore { STORE_NONE = 0, STORE_FP16 = 1, STORE_UNORM8 = 2 };

inline float slang_store(float v, int mode)
{
    if (mode == STORE_FP16) return static_cast<float>(static_cast<_Float16>(v));
    if (mode == STORE_UNORM8) return std::nearbyint(saturate(v) * 255.0f) / 255.0f;
    return v;
}

struct Texel2 : float4 {
    float4* dst;
    int mode;
    Texel2(float4* p, int m) : float4(*p), dst(p), mode(m) {}
    Texel2& operator=(const float4& v)
    {
        *dst = float4(slang_store(v.x, mode), slang_store(v.y, mode), slang_store(v.z, mode), slang_store(v.w, mode));
        return *this;
    }
};

template <class V> struct RWTexture2D {
    V* data = nullptr;
    int width = 0, height = 0, store = STORE_NONE;
    void GetDimensions(uint& w, uint& h) const
    {
        w = uint(width);
        h = uint(height);
    }
    Texel2 operator[](uint2 p) const { return Texel2(data + static_cast<long>(p.y) * width + p.x, store); }
    Texel2 operator[](int2 p) const { return Texel2(data + static_cast<long>(p.y) * width + p.x, store); }
};
