// Bloom + post-process chain (include/tg_post.h) on sm_103a.
//
// The reference's bloomExtractMain / bloomDownsampleMain / bloomUpsampleMain
// (src/bloom_downsample.slang) and postprocessMain (src/postprocess.slang),
// in the reference host's order (src/main.cpp:306-430): extract into mip 0 and
// downsample into mips 1..N-1 (one launch builds mips 0..5: each CTA owns an
// aligned tile of every level), upsample mip N-2 .. 0 in place (each texel
// reads the next mip and its own value, so no texel is read after another
// thread writes it), then the post pass.  The bloom chain is one allocation of
// rgba16f mips (8 B per texel, as the reference's bloom image).
//
// All arithmetic is explicitly rounded IEEE single precision in the shaders'
// order (sums left to right, no contraction into FMA); only the sRGB curve's
// power (exp2f / log2f) is CUDA's.  One thread per output texel, 32 x 8
// threads per CTA.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <new>

#include "svgf_internal.h"
#include "tg_post.h"

namespace tg {
namespace {

constexpr int kPostTX = 32, kPostTY = 8;
constexpr int kMaxMips = 16;

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }

struct C3 {
    float r, g, b;
};

__device__ __forceinline__ float lum(C3 c) { return add(add(mul(c.r, 0.2126f), mul(c.g, 0.7152f)), mul(c.b, 0.0722f)); }

__device__ __forceinline__ C3 ld_h4(const uint2* p, long long i)
{
    const uint2 u = p[i];
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
    return {a.x, a.y, b.x};
}

__device__ __forceinline__ void st_h4(uint2* p, long long i, C3 c)
{
    const __half2 a = __floats2half2_rn(c.r, c.g), b = __floats2half2_rn(c.b, 1.0f);
    p[i] = make_uint2(*reinterpret_cast<const uint32_t*>(&a), *reinterpret_cast<const uint32_t*>(&b));
}

template <bool F16> __device__ __forceinline__ C3 ld_hdr(const char* base, long long pitch, int x, int y)
{
    const char* row = base + y * pitch;
    if constexpr (F16) {
        return ld_h4(reinterpret_cast<const uint2*>(row), x);
    } else {
        const float4 v = reinterpret_cast<const float4*>(row)[x];
        return {v.x, v.y, v.z};
    }
}

struct Mip {
    uint2* p;
    int w, h;
};

__device__ __forceinline__ C3 round16(C3 c)
{
    return {__half2float(__float2half_rn(c.r)), __half2float(__float2half_rn(c.g)), __half2float(__float2half_rn(c.b))};
}

// Mip-0 texel (x, y) of the extraction (bloomExtractMain), before the fp16 store.
template <bool HDR16> __device__ __forceinline__ C3 extract_texel(const char* hdr, long long pitch, int W, int H, int x, int y, float thr)
{
    C3 s[4];
    float w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        C3 c = ld_hdr<HDR16>(hdr, pitch, min(2 * x + (k & 1), W - 1), min(2 * y + (k >> 1), H - 1));
        c = {c.r > 0.f ? c.r : 0.f, c.g > 0.f ? c.g : 0.f, c.b > 0.f ? c.b : 0.f};
        const float keep = lum(c) >= thr ? 1.f : 0.f;
        c = {mul(c.r, keep), mul(c.g, keep), mul(c.b, keep)};
        s[k] = c;
        w[k] = dv(1.f, add(1.f, lum(c)));
    }
    const float ws = add(add(add(w[0], w[1]), w[2]), w[3]);
    const float den = ws > 1e-7f ? ws : 1e-7f;
    auto acc = [&](float C3::*m) {
        return dv(add(add(add(mul(s[0].*m, w[0]), mul(s[1].*m, w[1])), mul(s[2].*m, w[2])), mul(s[3].*m, w[3])), den);
    };
    return {acc(&C3::r), acc(&C3::g), acc(&C3::b)};
}

// Mip i of the box-downsample chain from the 2x2 block of mip i-1 (bloomDownsampleMain).
__device__ __forceinline__ C3 box4(const C3 (&c)[4])
{
    return {mul(add(add(add(c[0].r, c[1].r), c[2].r), c[3].r), 0.25f), mul(add(add(add(c[0].g, c[1].g), c[2].g), c[3].g), 0.25f),
            mul(add(add(add(c[0].b, c[1].b), c[2].b), c[3].b), 0.25f)};
}

// Extraction and the downsample pyramid in one launch.  Mip i texel (x, y) reads exactly the 2x2 block
// (2x, 2y) .. (2x+1, 2y+1) of mip i-1 (clamped, and the clamp never leaves the block's aligned tile because
// mip i is floor(mip i-1 / 2) wide, or 1 wide when mip i-1 is), so a CTA that owns an aligned 32x32 tile of
// mip 0 owns the (32 >> i)-square tile of every mip i <= 5 and builds it from shared memory, with the values
// as the fp16 image stores them.
constexpr int kPyrT = 32;
constexpr int kPyrLevels = 6;
struct MipSet {
    Mip m[kPyrLevels];
    int n;  // levels built here, 1 .. kPyrLevels
};

template <bool HDR16>
__global__ void __launch_bounds__(256) k_bloom_pyramid(const char* hdr, long long pitch, int W, int H, MipSet ms, float thr)
{
    __shared__ float sa[3][kPyrT * kPyrT];  // ping-pong tiles of one mip level, one plane per channel
    __shared__ float sb[3][kPyrT * kPyrT];
    const int tid = threadIdx.x;
    const int X0 = blockIdx.x * kPyrT, Y0 = blockIdx.y * kPyrT;
    for (int k = tid; k < kPyrT * kPyrT; k += 256) {
        const int x = X0 + k % kPyrT, y = Y0 + k / kPyrT;
        if (x >= ms.m[0].w || y >= ms.m[0].h) continue;
        const C3 c = round16(extract_texel<HDR16>(hdr, pitch, W, H, x, y, thr));
        st_h4(ms.m[0].p, (long long)y * ms.m[0].w + x, c);
        sa[0][k] = c.r;
        sa[1][k] = c.g;
        sa[2][k] = c.b;
    }
    float(*cur)[kPyrT * kPyrT] = sa;
    float(*nxt)[kPyrT * kPyrT] = sb;
    int side = kPyrT;
    for (int i = 1; i < ms.n; ++i) {
        __syncthreads();
        const Mip s = ms.m[i - 1], d = ms.m[i];
        const int ns = side >> 1, sx0 = X0 >> (i - 1), sy0 = Y0 >> (i - 1), dx0 = X0 >> i, dy0 = Y0 >> i;
        for (int k = tid; k < ns * ns; k += 256) {
            const int x = dx0 + k % ns, y = dy0 + k / ns;
            if (x >= d.w || y >= d.h) continue;
            C3 c[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int j = (min(2 * y + (q >> 1), s.h - 1) - sy0) * side + (min(2 * x + (q & 1), s.w - 1) - sx0);
                c[q] = {cur[0][j], cur[1][j], cur[2][j]};
            }
            const C3 v = round16(box4(c));
            st_h4(d.p, (long long)y * d.w + x, v);
            nxt[0][k] = v.r;
            nxt[1][k] = v.g;
            nxt[2][k] = v.b;
        }
        float(*t)[kPyrT * kPyrT] = cur;
        cur = nxt;
        nxt = t;
        side = ns;
    }
}

__global__ void __launch_bounds__(kPostTX* kPostTY) k_bloom_down(Mip s, Mip d)
{
    const int x = blockIdx.x * kPostTX + threadIdx.x, y = blockIdx.y * kPostTY + threadIdx.y;
    if (x >= d.w || y >= d.h) return;
    C3 c[4];
#pragma unroll
    for (int k = 0; k < 4; ++k)
        c[k] = ld_h4(s.p, (long long)min(2 * y + (k >> 1), s.h - 1) * s.w + min(2 * x + (k & 1), s.w - 1));
    st_h4(d.p, (long long)y * d.w + x, box4(c));
}

__global__ void __launch_bounds__(kPostTX* kPostTY) k_bloom_up(Mip s, Mip d)
{
    const int x = blockIdx.x * kPostTX + threadIdx.x, y = blockIdx.y * kPostTY + threadIdx.y;
    if (x >= d.w || y >= d.h) return;
    const int bx = x / 2, by = y / 2;
    C3 sum = {0.f, 0.f, 0.f};
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            const float wk = float((dx == 0 ? 2 : 1) * (dy == 0 ? 2 : 1)) * 0.0625f;
            const C3 c = ld_h4(s.p, (long long)min(max(by + dy, 0), s.h - 1) * s.w + min(max(bx + dx, 0), s.w - 1));
            sum = {add(sum.r, mul(wk, c.r)), add(sum.g, mul(wk, c.g)), add(sum.b, mul(wk, c.b))};
        }
    const long long i = (long long)y * d.w + x;
    const C3 e = ld_h4(d.p, i);
    st_h4(d.p, i, {add(e.r, sum.r), add(e.g, sum.g), add(e.b, sum.b)});
}

__device__ __forceinline__ float sat(float v) { return v < 0.f ? 0.f : (v > 1.f ? 1.f : v); }

// c^(1/2.4) for c in (0.0031308, 1] as exp2f(log2f(c) / 2.4): full-precision library calls (a few ulp),
// far cheaper than the general powf; the 8-bit output absorbs the difference almost everywhere.
__device__ __forceinline__ float srgb(float c)
{
    constexpr float kExp = 1.0f / 2.4f;
    c = c > 0.f ? c : 0.f;
    if (c <= 0.0031308f) return mul(c, 12.92f);
    return sub(mul(1.055f, exp2f(mul(log2f(c), kExp))), 0.055f);
}

__device__ __forceinline__ float fit(float v)
{
    const float a = sub(mul(v, add(v, 0.0245786f)), 0.000090537f);
    const float b = add(mul(v, add(mul(0.983729f, v), 0.4329510f)), 0.238081f);
    return dv(a, b);
}

__device__ __forceinline__ C3 mat3(const float (&m)[9], C3 v)
{
    return {add(add(mul(m[0], v.r), mul(m[1], v.g)), mul(m[2], v.b)), add(add(mul(m[3], v.r), mul(m[4], v.g)), mul(m[5], v.b)),
            add(add(mul(m[6], v.r), mul(m[7], v.g)), mul(m[8], v.b))};
}

__constant__ float kAcesIn[9] = {0.59719f, 0.35458f, 0.04823f, 0.07600f, 0.90834f, 0.01566f, 0.02840f, 0.13383f, 0.83777f};
__constant__ float kAcesOut[9] = {1.60475f, -0.53108f, -0.07367f, -0.10208f, 1.10813f, -0.00605f, -0.00327f, -0.07276f, 1.07602f};

enum OutFmt { OUT_BGRA8 = 0, OUT_RGBA8 = 1, OUT_RGBA32F = 2 };

template <bool HDR16, int OUT>
__global__ void __launch_bounds__(kPostTX* kPostTY)
    k_post(const char* hdr, long long hpitch, char* out, long long opitch, int W, int H, Mip bl, float strength)
{
    const int x = blockIdx.x * kPostTX + threadIdx.x, y = blockIdx.y * kPostTY + threadIdx.y;
    if (x >= W || y >= H) return;
    const float u = dv(add(float(x), 0.5f), float(W)), v = dv(add(float(y), 0.5f), float(H));
    const float ox = sub(u, 0.5f), oy = sub(v, 0.5f);
    const float d2 = add(mul(ox, ox), mul(oy, oy));
    const int px = int(mul(mul(mul(ox, d2), 0.0015f), float(W))), py = int(mul(mul(mul(oy, d2), 0.0015f), float(H)));
    auto sample = [&](int cx, int cy) {
        cx = min(cx, W - 1);
        cy = min(cy, H - 1);
        const C3 h = ld_hdr<HDR16>(hdr, hpitch, cx, cy);
        const C3 b = ld_h4(bl.p, (long long)min(cy / 2, bl.h - 1) * bl.w + min(cx / 2, bl.w - 1));
        return C3{add(h.r, mul(strength, b.r)), add(h.g, mul(strength, b.g)), add(h.b, mul(strength, b.b))};
    };
    C3 c;
    c.r = sample(min(max(x + px, 0), W - 1), min(max(y + py, 0), H - 1)).r;
    c.g = sample(x, y).g;
    c.b = sample(min(max(x - px, 0), W - 1), min(max(y - py, 0), H - 1)).b;
    c = mat3(kAcesIn, c);
    c = {fit(c.r), fit(c.g), fit(c.b)};
    c = mat3(kAcesOut, c);
    c = {srgb(sat(c.r)), srgb(sat(c.g)), srgb(sat(c.b))};
    const float l = lum(c);
    const C3 cool = {mul(l, 0.9f), mul(l, 0.95f), mul(l, 1.1f)};
    c = {add(c.r, mul(sub(cool.r, c.r), 0.15f)), add(c.g, mul(sub(cool.g, c.g), 0.15f)), add(c.b, mul(sub(cool.b, c.b), 0.15f))};
    const float vig = sat(sub(1.f, mul(add(mul(ox, ox), mul(oy, oy)), 1.5f)));
    c = {mul(c.r, vig), mul(c.g, vig), mul(c.b, vig)};
    char* row = out + y * opitch;
    if constexpr (OUT == OUT_RGBA32F) {
        reinterpret_cast<float4*>(row)[x] = make_float4(c.r, c.g, c.b, 1.f);
    } else {
        auto q = [](float f) { return __float2uint_rn(__fmul_rn(sat(f), 255.0f)); };
        const uint32_t r = q(c.r), g = q(c.g), b = q(c.b);
        reinterpret_cast<uint32_t*>(row)[x] = OUT == OUT_BGRA8 ? (b | (g << 8) | (r << 16) | (255u << 24))
                                                                : (r | (g << 8) | (b << 16) | (255u << 24));
    }
}

} // namespace
} // namespace tg

using namespace tg;

struct tg_post {
    int device = 0;
    uint32_t w = 0, h = 0;
    tg_post_params p{};
    char* buf = nullptr;
    size_t bytes = 0;
    int n = 0;
    Mip mip[kMaxMips];
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

int alloc_chain(tg_post* s)
{
    const uint32_t bw = std::max(s->w / 2, 1u), bh = std::max(s->h / 2, 1u);
    const uint32_t levels = uint32_t(std::floor(std::log2(float(std::max(bw, bh))))) + 1;
    s->n = int(std::min(std::min(levels, s->p.max_mips), uint32_t(kMaxMips)));
    size_t off[kMaxMips], total = 0;
    for (int i = 0; i < s->n; ++i) {
        s->mip[i].w = int(std::max(bw >> i, 1u));
        s->mip[i].h = int(std::max(bh >> i, 1u));
        off[i] = total;
        total += (size_t(s->mip[i].w) * s->mip[i].h * 8 + 255) / 256 * 256;
    }
    if (cudaMalloc(&s->buf, total) != cudaSuccess) {
        cudaGetLastError();
        s->buf = nullptr;
        return fail(TG_ERR_OOM, "cudaMalloc of %zu bloom bytes failed", total);
    }
    s->bytes = total;
    for (int i = 0; i < s->n; ++i) s->mip[i].p = reinterpret_cast<uint2*>(s->buf + off[i]);
    return TG_OK;
}

int check_img(const char* what, const tg_image* im, uint32_t w, const int* fmts, int nf, long long& pitch)
{
    if (!im || !im->ptr) return fail(TG_ERR_INVALID, "%s: null image", what);
    bool ok = false;
    for (int k = 0; k < nf; ++k) ok |= im->format == fmts[k];
    if (!ok) return fail(TG_ERR_INVALID, "%s: unsupported format %d", what, im ? im->format : -1);
    const long long tb = fmt_bytes(im->format);
    pitch = im->pitch_bytes ? im->pitch_bytes : tb * w;
    if (pitch < tb * (long long)w || pitch % tb || reinterpret_cast<uintptr_t>(im->ptr) % tb)
        return fail(TG_ERR_INVALID, "%s: address and pitch must be multiples of %lld bytes and cover a row", what, tb);
    return TG_OK;
}

} // namespace

int tg_post_params_default(tg_post_params* p)
{
    if (!p) return fail(TG_ERR_INVALID, "null params");
    *p = tg_post_params{1.0f, 0.095f, 6u, 0u};
    return TG_OK;
}

int tg_post_create(uint32_t width, uint32_t height, const tg_post_params* params, int device, tg_post** out)
{
    if (!out) return fail(TG_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(TG_ERR_INVALID, "size %ux%u outside 1..32768", width, height);
    tg_post_params p;
    tg_post_params_default(&p);
    if (params) p = *params;
    if (p.max_mips < 1 || !std::isfinite(p.bloom_threshold) || !std::isfinite(p.bloom_strength))
        return fail(TG_ERR_INVALID, "max_mips must be >= 1 and threshold / strength finite");
    if (device < 0 && cudaGetDevice(&device) != cudaSuccess) return fail(TG_ERR_CUDA, "no current CUDA device");
    DeviceGuard g(device);
    tg_post* s = new (std::nothrow) tg_post();
    if (!s) return fail(TG_ERR_OOM, "host allocation failed");
    s->device = device;
    s->w = width;
    s->h = height;
    s->p = p;
    const int st = alloc_chain(s);
    if (st) {
        delete s;
        return st;
    }
    *out = s;
    return TG_OK;
}

int tg_post_process(tg_post* s, const tg_image* hdr, const tg_image* out, void* stream)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    static const int kHdr[] = {TG_FMT_RGBA16F, TG_FMT_RGBA32F};
    static const int kOut[] = {TG_FMT_BGRA8, TG_FMT_RGBA8, TG_FMT_RGBA32F};
    long long hp = 0, op = 0;
    int st;
    if ((st = check_img("hdr", hdr, s->w, kHdr, 2, hp))) return st;
    if ((st = check_img("out", out, s->w, kOut, 3, op))) return st;
    DeviceGuard g(s->device);
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    const dim3 blk(kPostTX, kPostTY);
    auto grid = [](int w, int h) { return dim3((w + kPostTX - 1) / kPostTX, (h + kPostTY - 1) / kPostTY); };
    const char* hb = static_cast<const char*>(hdr->ptr);
    const bool h16 = hdr->format == TG_FMT_RGBA16F;
    const int W = int(s->w), H = int(s->h);
    // extraction + mips 1..5 in one launch; mips beyond the sixth (max_mips > 6) one launch each
    MipSet ms;
    ms.n = std::min(s->n, kPyrLevels);
    for (int i = 0; i < ms.n; ++i) ms.m[i] = s->mip[i];
    const dim3 pgrid((s->mip[0].w + kPyrT - 1) / kPyrT, (s->mip[0].h + kPyrT - 1) / kPyrT);
    if (h16)
        k_bloom_pyramid<true><<<pgrid, 256, 0, cs>>>(hb, hp, W, H, ms, s->p.bloom_threshold);
    else
        k_bloom_pyramid<false><<<pgrid, 256, 0, cs>>>(hb, hp, W, H, ms, s->p.bloom_threshold);
    for (int i = kPyrLevels; i < s->n; ++i) k_bloom_down<<<grid(s->mip[i].w, s->mip[i].h), blk, 0, cs>>>(s->mip[i - 1], s->mip[i]);
    for (int i = s->n - 2; i >= 0; --i) k_bloom_up<<<grid(s->mip[i].w, s->mip[i].h), blk, 0, cs>>>(s->mip[i + 1], s->mip[i]);
    char* ob = static_cast<char*>(out->ptr);
    const float str = s->p.bloom_strength;
    const dim3 pg = grid(W, H);
    switch ((h16 ? 10 : 0) + (out->format == TG_FMT_BGRA8 ? 0 : out->format == TG_FMT_RGBA8 ? 1 : 2)) {
    case 10: k_post<true, OUT_BGRA8><<<pg, blk, 0, cs>>>(hb, hp, ob, op, W, H, s->mip[0], str); break;
    case 11: k_post<true, OUT_RGBA8><<<pg, blk, 0, cs>>>(hb, hp, ob, op, W, H, s->mip[0], str); break;
    case 12: k_post<true, OUT_RGBA32F><<<pg, blk, 0, cs>>>(hb, hp, ob, op, W, H, s->mip[0], str); break;
    case 0: k_post<false, OUT_BGRA8><<<pg, blk, 0, cs>>>(hb, hp, ob, op, W, H, s->mip[0], str); break;
    case 1: k_post<false, OUT_RGBA8><<<pg, blk, 0, cs>>>(hb, hp, ob, op, W, H, s->mip[0], str); break;
    default: k_post<false, OUT_RGBA32F><<<pg, blk, 0, cs>>>(hb, hp, ob, op, W, H, s->mip[0], str); break;
    }
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "post-process launch failed: %s", cudaGetErrorString(e));
    return TG_OK;
}

int tg_post_resize(tg_post* s, uint32_t width, uint32_t height)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(TG_ERR_INVALID, "size %ux%u outside 1..32768", width, height);
    DeviceGuard g(s->device);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(TG_ERR_CUDA, "synchronize failed");
    cudaFree(s->buf);
    s->buf = nullptr;
    s->w = width;
    s->h = height;
    return alloc_chain(s);
}

int tg_post_get_info(const tg_post* s, tg_post_info* info)
{
    if (!s || !info) return fail(TG_ERR_INVALID, "null handle or info");
    *info = tg_post_info{};
    info->width = s->w;
    info->height = s->h;
    info->mip_count = uint32_t(s->n);
    info->bloom_bytes = s->bytes;
    for (int i = 0; i < s->n; ++i) {
        info->mip_width[i] = uint32_t(s->mip[i].w);
        info->mip_height[i] = uint32_t(s->mip[i].h);
        info->mip_ptr[i] = s->mip[i].p;
    }
    return TG_OK;
}

void tg_post_destroy(tg_post* s)
{
    if (!s) return;
    {
        DeviceGuard g(s->device);
        cudaFree(s->buf);
    }
    delete s;
}
