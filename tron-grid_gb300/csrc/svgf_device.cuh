// Device-side building blocks of the SVGF kernels: image views, storage
// formats, luminance, octahedral normals, fp16 packing.
//
// Every comparison that decides a discrete outcome (history accepted or not,
// a tap inside the image, a 7x7 variance fallback) is evaluated with
// explicitly rounded, unfused operations (__fmul_rn / __fadd_rn), so that the
// decision is bit-identical to a CPU evaluation of the same expression.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "tg_svgf.h"

// Chain kernels are launched with programmatic stream serialization (PDL) when
// this is 1: a kernel's CTAs are scheduled while the previous kernel of the
// stream drains, and wait in pdl_begin() for its completion.
#ifndef TG_PDL
#define TG_PDL 1
#endif

namespace tg {

// First statement of every chain kernel.  griddepcontrol.wait holds the CTA
// until the previous kernel of the stream has completed and its writes are
// visible (it returns at once for a kernel launched without programmatic
// serialization); launch_dependents then allows the next kernel's CTAs to be
// scheduled once every CTA of this grid has started, so they never take an SM
// slot from a CTA of this grid that has not.
__device__ __forceinline__ void pdl_begin()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// Launches a chain kernel on `st`, with programmatic stream serialization when
// TG_PDL is set (the kernel must begin with pdl_begin()).
template <class... P, class... A>
inline cudaError_t launch_chain(void (*k)(P...), dim3 grid, dim3 block, cudaStream_t st, A&&... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = TG_PDL ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, k, static_cast<A&&>(args)...);
}

enum Storage : int { ST_FP32 = 0, ST_FP16 = 1 };

// Caller image as seen by a kernel.
struct Img {
    char* ptr;
    int64_t pitch;
    int32_t fmt;
    int32_t pad;
};

// Constants of the FULL algorithm.
constexpr float kEpsL = 1e-4f;     // luminance edge-stop denominator floor
constexpr float kEpsZ = 1e-3f;     // depth edge-stop denominator floor (metres)
constexpr float kDepthRel = 0.05f; // reprojection depth test: relative term
constexpr float kDepthGrad = 4.0f; // reprojection depth test: gradient term
constexpr float kDepthAbs = 0.1f;  // reprojection depth test: absolute term
constexpr float kNormalCos = 0.9f; // reprojection normal test: minimum cosine (tested squared: 0.81)
constexpr float kHalfMax = 65504.0f;
constexpr float kLog2eF = 1.4426950408889634f;

__device__ __forceinline__ float ex2_approx(float x)
{
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float lg2_approx(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float rcp_approx(float x)
{
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float sqrt_approx(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ float b3(int i)
{
    // B3-spline taps 1/16, 1/4, 3/8, 1/4, 1/16 (index 0..4).
    return i == 2 ? 0.375f : ((i == 1 || i == 3) ? 0.25f : 0.0625f);
}

// Rec.709 luminance (src/svgf_denoise.slang:109-112), unfused.
__device__ __forceinline__ float lum(float r, float g, float b)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(r, 0.2126f), __fmul_rn(g, 0.7152f)), __fmul_rn(b, 0.0722f));
}

__device__ __forceinline__ float dot3_rn(float ax, float ay, float az, float bx, float by, float bz)
{
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// Hint: bring the line holding p towards L2 (no register result; p must lie in an allocation).
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

__device__ __forceinline__ float q16(float v) { return __half2float(__float2half_rn(v)); }
__device__ __forceinline__ float sat16(float v) { return fminf(fmaxf(v, -kHalfMax), kHalfMax); }

__device__ __forceinline__ uint32_t pack_h2(float a, float b)
{
    __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ float2 unpack_h2(uint32_t u)
{
    __half2 h = *reinterpret_cast<__half2*>(&u);
    return __half22float2(h);
}

__device__ __forceinline__ float4 unpack_h4(uint2 u)
{
    float2 a = unpack_h2(u.x), b = unpack_h2(u.y);
    return make_float4(a.x, a.y, b.x, b.y);
}

__device__ __forceinline__ uint2 pack_h4(float4 v) { return make_uint2(pack_h2(v.x, v.y), pack_h2(v.z, v.w)); }

// Octahedral snorm16 codec (Meyer et al. 2010).  Same operation order as the
// CPU oracle so that encode/decode round trips agree bit for bit.
__device__ __forceinline__ float sgn_nz(float v) { return v >= 0.0f ? 1.0f : -1.0f; }

__device__ __forceinline__ uint32_t oct16_encode(float nx, float ny, float nz)
{
    float l1 = __fadd_rn(__fadd_rn(fabsf(nx), fabsf(ny)), fabsf(nz));
    float px = l1 > 0.0f ? __fdiv_rn(nx, l1) : 0.0f;
    float py = l1 > 0.0f ? __fdiv_rn(ny, l1) : 0.0f;
    if (nz < 0.0f) {
        float ox = __fmul_rn(__fsub_rn(1.0f, fabsf(py)), sgn_nz(px));
        float oy = __fmul_rn(__fsub_rn(1.0f, fabsf(px)), sgn_nz(py));
        px = ox;
        py = oy;
    }
    px = fminf(1.0f, fmaxf(-1.0f, px));
    py = fminf(1.0f, fmaxf(-1.0f, py));
    int ex = __float2int_rn(__fmul_rn(px, 32767.0f));
    int ey = __float2int_rn(__fmul_rn(py, 32767.0f));
    return (uint32_t(ex) & 0xffffu) | (uint32_t(ey) << 16);
}

__device__ __forceinline__ float3 oct16_decode(uint32_t u)
{
    int ex = int(int16_t(u & 0xffffu));
    int ey = int(int16_t(u >> 16));
    float px = fmaxf(-1.0f, __fdiv_rn(float(ex), 32767.0f));
    float py = fmaxf(-1.0f, __fdiv_rn(float(ey), 32767.0f));
    float vz = __fsub_rn(__fsub_rn(1.0f, fabsf(px)), fabsf(py));
    if (vz < 0.0f) {
        float ox = __fmul_rn(__fsub_rn(1.0f, fabsf(py)), sgn_nz(px));
        float oy = __fmul_rn(__fsub_rn(1.0f, fabsf(px)), sgn_nz(py));
        px = ox;
        py = oy;
    }
    float d = dot3_rn(px, py, vz, px, py, vz);
    float inv = __fdiv_rn(1.0f, __fsqrt_rn(d));
    return make_float3(__fmul_rn(px, inv), __fmul_rn(py, inv), __fmul_rn(vz, inv));
}

// Unnormalised octahedral decode (the point on the unit octahedron), the form
// in which FP16 storage keeps normals for the reprojection test.  Same
// operations as the CPU oracle, so the test decides identically.
__device__ __forceinline__ float3 oct16_decode_raw(uint32_t u)
{
    const float kInv = 1.0f / 32767.0f;
    float px = fmaxf(-1.0f, __fmul_rn(float(int(int16_t(u & 0xffffu))), kInv));
    float py = fmaxf(-1.0f, __fmul_rn(float(int(int16_t(u >> 16))), kInv));
    const float vz = __fsub_rn(__fsub_rn(1.0f, fabsf(px)), fabsf(py));
    if (vz < 0.0f) {
        const float ox = __fmul_rn(__fsub_rn(1.0f, fabsf(py)), sgn_nz(px));
        const float oy = __fmul_rn(__fsub_rn(1.0f, fabsf(px)), sgn_nz(py));
        px = ox;
        py = oy;
    }
    return make_float3(px, py, vz);
}

// Reprojection normal test, scale-free: the angle between a and b is at most
// acos(0.9) iff a.b >= 0 and (a.b)^2 >= 0.81 |a|^2 |b|^2 (unfused, as on the CPU).
__device__ __forceinline__ bool normal_close(float ax, float ay, float az, float bx, float by, float bz)
{
    const float d = dot3_rn(ax, ay, az, bx, by, bz);
    if (!(d >= 0.0f)) return false;
    const float aa = dot3_rn(ax, ay, az, ax, ay, az);
    const float bb = dot3_rn(bx, by, bz, bx, by, bz);
    return __fmul_rn(d, d) >= __fmul_rn(__fmul_rn(0.81f, aa), bb);
}

// Octahedral decode for edge-stopping weights only (never for a discrete
// decision): reciprocal-multiply and rsqrt instead of IEEE divisions.
__device__ __forceinline__ float3 oct16_decode_fast(uint32_t u)
{
    const float kInv = 1.0f / 32767.0f;
    float px = fmaxf(-1.0f, float(int(int16_t(u & 0xffffu))) * kInv);
    float py = fmaxf(-1.0f, float(int(int16_t(u >> 16))) * kInv);
    const float vz = 1.0f - fabsf(px) - fabsf(py);
    if (vz < 0.0f) {
        const float ox = (1.0f - fabsf(py)) * sgn_nz(px);
        const float oy = (1.0f - fabsf(px)) * sgn_nz(py);
        px = ox;
        py = oy;
    }
    const float inv = rsqrtf(fmaf(px, px, fmaf(py, py, vz * vz)));
    return make_float3(px * inv, py * inv, vz * inv);
}

// ---------------------------------------------------------- caller images ----

__device__ __forceinline__ const char* row_ptr(const Img& im, int y) { return im.ptr + int64_t(y) * im.pitch; }

__device__ __forceinline__ float4 ld_rgba(const Img& im, int x, int y)
{
    const char* r = row_ptr(im, y);
    if (im.fmt == TG_FMT_RGBA32F) return __ldg(reinterpret_cast<const float4*>(r) + x);
    uint2 u = __ldg(reinterpret_cast<const uint2*>(r) + x);
    return unpack_h4(u);
}

__device__ __forceinline__ void st_rgba(const Img& im, int x, int y, float4 v)
{
    char* r = im.ptr + int64_t(y) * im.pitch;
    if (im.fmt == TG_FMT_RGBA32F)
        reinterpret_cast<float4*>(r)[x] = v;
    else
        reinterpret_cast<uint2*>(r)[x] = pack_h4(v);
}

__device__ __forceinline__ float ld_depth(const Img& im, int x, int y)
{
    return __ldg(reinterpret_cast<const float*>(row_ptr(im, y)) + x);
}

// Unit normal; `enc` receives the octahedral code (input bits when the input
// is OCT16, else the encoding of the loaded vector).
__device__ __forceinline__ float3 ld_normal(const Img& im, int x, int y, bool want_enc, uint32_t& enc)
{
    const char* r = row_ptr(im, y);
    if (im.fmt == TG_FMT_OCT16) {
        enc = __ldg(reinterpret_cast<const uint32_t*>(r) + x);
        if (want_enc) return make_float3(0.f, 0.f, 0.f);  // the caller decodes the code itself
        return oct16_decode(enc);
    }
    float3 n;
    if (im.fmt == TG_FMT_RGBA32F) {
        float4 v = __ldg(reinterpret_cast<const float4*>(r) + x);
        n = make_float3(v.x, v.y, v.z);
    } else {
        const float* p = reinterpret_cast<const float*>(r) + 3 * x;
        n = make_float3(__ldg(p), __ldg(p + 1), __ldg(p + 2));
    }
    if (want_enc) enc = oct16_encode(n.x, n.y, n.z);
    return n;
}

__device__ __forceinline__ float2 ld_motion(const Img& im, int x, int y)
{
    const char* r = row_ptr(im, y);
    if (im.fmt == TG_FMT_RG32F) return __ldg(reinterpret_cast<const float2*>(r) + x);
    return unpack_h2(__ldg(reinterpret_cast<const uint32_t*>(r) + x));
}

// --------------------------------------------------------- handle storage ----
//
// FULL state per pixel
//   guide : unit normal + linear depth   FP32 float4(n, z)    FP16 uint2(oct16, z bits)
//   hist  : colour history + length      FP32 float4(rgb, len) FP16 4 x half
//   mom   : luminance mean + variance    FP32 float2           FP16 2 x half
// FULL scratch per pixel
//   tc    : temporally integrated colour + length   (as hist)
//   col   : a-trous colour + variance               (as hist)

template <int ST> struct Stor;

template <> struct Stor<ST_FP32> {
    typedef float4 guide_t;
    typedef float4 c4_t;
    typedef float2 mom_t;
    __device__ static float4 ld_guide_raw(const guide_t* p, size_t i) { return __ldg(p + i); }
    __device__ static float4 ld_guide_w(const guide_t* p, size_t i) { return __ldg(p + i); }
    __device__ static float ld_guide_z(const guide_t* p, size_t i) { return __ldg(reinterpret_cast<const float*>(p + i) + 3); }
    __device__ static guide_t mk_guide(float3 n, uint32_t, float z) { return make_float4(n.x, n.y, n.z, z); }
    // the guide as stored (FP32: unit normal and depth)
    typedef float4 graw_t;
    __device__ static graw_t ld_graw(const guide_t* p, size_t i) { return __ldg(p + i); }
    __device__ static float4 ld4(const c4_t* p, size_t i) { return __ldg(p + i); }
    __device__ static float ld4_w(const c4_t* p, size_t i) { return __ldg(reinterpret_cast<const float*>(p + i) + 3); }
    __device__ static void st4(c4_t* p, size_t i, float4 v) { p[i] = v; }
    __device__ static void st4_sat_w(c4_t* p, size_t i, float4 v) { p[i] = v; }
    __device__ static float2 ldm(const mom_t* p, size_t i) { return __ldg(p + i); }
    __device__ static void stm(mom_t* p, size_t i, float2 v) { p[i] = v; }
    // the value ld4 / ldm return after st4 / stm stored v
    __device__ static float4 rt4(float4 v) { return v; }
    __device__ static float2 rtm(float2 v) { return v; }
    __device__ static float qin(float v) { return v; }
};

template <> struct Stor<ST_FP16> {
    typedef uint2 guide_t;
    typedef uint2 c4_t;
    typedef uint32_t mom_t;
    // guide for the reprojection test: unnormalised octahedral normal
    __device__ static float4 ld_guide_raw(const guide_t* p, size_t i)
    {
        uint2 u = __ldg(p + i);
        float3 n = oct16_decode_raw(u.x);
        return make_float4(n.x, n.y, n.z, __uint_as_float(u.y));
    }
    // guide for edge-stopping weights (fast decode)
    __device__ static float4 ld_guide_w(const guide_t* p, size_t i)
    {
        uint2 u = __ldg(p + i);
        float3 n = oct16_decode_fast(u.x);
        return make_float4(n.x, n.y, n.z, __uint_as_float(u.y));
    }
    __device__ static float ld_guide_z(const guide_t* p, size_t i)
    {
        return __uint_as_float(__ldg(reinterpret_cast<const uint32_t*>(p + i) + 1));
    }
    __device__ static guide_t mk_guide(float3, uint32_t enc, float z) { return make_uint2(enc, __float_as_uint(z)); }
    // the guide as stored (FP16 storage: octahedral code and depth bits)
    typedef uint2 graw_t;
    __device__ static graw_t ld_graw(const guide_t* p, size_t i) { return __ldg(p + i); }
    __device__ static float4 ld4(const c4_t* p, size_t i) { return unpack_h4(__ldg(p + i)); }
    __device__ static float ld4_w(const c4_t* p, size_t i)
    {
        return unpack_h2(__ldg(reinterpret_cast<const uint32_t*>(p + i) + 1)).y;
    }
    __device__ static void st4(c4_t* p, size_t i, float4 v) { p[i] = pack_h4(v); }
    __device__ static void st4_sat_w(c4_t* p, size_t i, float4 v)
    {
        v.w = sat16(v.w);
        p[i] = pack_h4(v);
    }
    __device__ static float2 ldm(const mom_t* p, size_t i) { return unpack_h2(__ldg(p + i)); }
    __device__ static void stm(mom_t* p, size_t i, float2 v) { p[i] = pack_h2(sat16(v.x), sat16(v.y)); }
    // the value ld4 / ldm return after st4 / stm stored v
    __device__ static float4 rt4(float4 v) { return unpack_h4(pack_h4(v)); }
    __device__ static float2 rtm(float2 v) { return unpack_h2(pack_h2(sat16(v.x), sat16(v.y))); }
    __device__ static float qin(float v) { return q16(v); }
};

// A-trous scratch records, the same for both storage forms (binary16 records
// were the largest error term of the FP16 form against float64, so the
// scratch stays float32): float4 (r, g, b, var) in the colour half-plane at i,
// the guide float4 (unit normal, z) in the guide half-plane at gh + i; a tile
// row of either half is one contiguous run.  Beside the records, a plane of
// their variances (`off` bytes after the buffer start), 4 B per record.
struct Rec {
    typedef float4 rec_t;
    static constexpr int kRecBytes = 32;
    __device__ static void ld_rec(const rec_t* p, size_t i, float4& c, float4& g, size_t gh)
    {
        c = __ldg(p + i);
        g = __ldg(p + gh + i);
    }
    __device__ static void st_rec(rec_t* p, size_t i, float4 c, float4 g, size_t gh)
    {
        p[i] = c;
        p[gh + i] = g;
    }
    typedef float var_t;
    __device__ static const var_t* var_ptr(const void* buf, size_t off)
    {
        return reinterpret_cast<const float*>(static_cast<const char*>(buf) + off);
    }
    __device__ static float var_at(const var_t* p, int i) { return __ldg(p + i); }
    __device__ static float ld_var(const void* buf, size_t off, size_t i) { return __ldg(var_ptr(buf, off) + i); }
    __device__ static void st_var(void* buf, size_t off, size_t i, float v)
    {
        reinterpret_cast<float*>(static_cast<char*>(buf) + off)[i] = v;
    }
};

// One-sided depth difference with the smaller magnitude (0 for a 1-pixel axis).
__device__ __forceinline__ float grad1(float z, float zl, float zr, bool has_l, bool has_r)
{
    float dl = has_l ? __fsub_rn(z, zl) : 0.0f;
    float dr = has_r ? __fsub_rn(zr, z) : 0.0f;
    if (has_l && has_r) return fabsf(dl) <= fabsf(dr) ? dl : dr;
    if (has_l) return dl;
    if (has_r) return dr;
    return 0.0f;
}

// max(0, d)^sigma_n: `sq` squarings when sigma_n = 2^sq, else exp2(sigma_n log2 d).
__device__ __forceinline__ float normal_weight(float d, int sq, float sigma_n)
{
    if (!(d > 0.0f)) return 0.0f;
    if (sq >= 0) {
        float v = d;
        for (int i = 0; i < sq; ++i) v = v * v;
        return v;
    }
    return exp2f(sigma_n * log2f(d));
}

} // namespace tg
