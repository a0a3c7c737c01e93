// Volumetric-fog froxel filter (include/tg_fog.h) on sm_103a.
//
// The reference's filterMain (src/volumetric_filter.slang:142-226).  A CTA
// covers 32 x 4 columns of 8 consecutive slices, one thread per column: the
// column's camera ray and the slices' view depths are computed once (they are
// the same for every froxel of a column / slice), then for each slice the CTA
// stages the 34 x 6 halo of injected texels in shared memory with coalesced
// loads (the 3x3 mean reads shared memory; a texel is read from L2 once per CTA
// instead of nine times) and each thread places its froxel centre on its ray,
// projects it into the previous frame and fetches the history trilinearly.
//
// Every add, multiply, divide and square root on the projection path is an
// explicitly rounded IEEE operation (no contraction into FMA), in the order
// the reference writes them, so the froxel coordinates that decide the
// rejection tests and the trilinear weights are the reference's own float
// arithmetic; only powf / logf (slice depth, its inverse) are CUDA's.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "svgf_internal.h"
#include "tg_fog.h"

namespace tg {
namespace {

// 128-thread CTAs: 4.6% faster per pass at 320x180x64 than 32 x 8 columns.
constexpr int kFogTX = 32, kFogTY = 4;
constexpr int kFogSW = kFogTX + 2, kFogSH = kFogTY + 2;
constexpr int kFogZC = 8;  // slices per CTA

struct FogArgs {
    float ivp[16], pvp[16], cam[3];
    float alpha, znear, zfar;
    int W, H, D, valid;
    const char* raw;
    const char* hist;
    char* out;
    long long raw_row, raw_slice, hist_row, hist_slice, out_row, out_slice;
};

template <bool F16> __device__ __forceinline__ float4 ld_texel(const char* base, long long off)
{
    if constexpr (F16) {
        const uint2 u = __ldg(reinterpret_cast<const uint2*>(base + off));
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&u.y));
        return make_float4(a.x, a.y, b.x, b.y);
    } else {
        return __ldg(reinterpret_cast<const float4*>(base + off));
    }
}

template <bool F16> __device__ __forceinline__ void st_texel(char* base, long long off, float4 v)
{
    if constexpr (F16) {
        const __half2 a = __floats2half2_rn(v.x, v.y), b = __floats2half2_rn(v.z, v.w);
        uint2 u;
        u.x = *reinterpret_cast<const uint32_t*>(&a);
        u.y = *reinterpret_cast<const uint32_t*>(&b);
        *reinterpret_cast<uint2*>(base + off) = u;
    } else {
        *reinterpret_cast<float4*>(base + off) = v;
    }
}

__device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float dv(float a, float b) { return __fdiv_rn(a, b); }

// clip = M (x, y, z, w), M column-major, the four column terms summed left to right
__device__ __forceinline__ void mat_vec(const float* m, float x, float y, float z, float w, float o[4])
{
#pragma unroll
    for (int r = 0; r < 4; ++r) o[r] = add(add(add(mul(m[r], x), mul(m[4 + r], y)), mul(m[8 + r], z)), mul(m[12 + r], w));
}

__device__ __forceinline__ float lerp1(float a, float b, float t) { return add(a, mul(sub(b, a), t)); }

__device__ __forceinline__ float4 lerp4(float4 a, float4 b, float t)
{
    return make_float4(lerp1(a.x, b.x, t), lerp1(a.y, b.y, t), lerp1(a.z, b.z, t), lerp1(a.w, b.w, t));
}

template <bool RAW16, bool OUT16>
__global__ void __launch_bounds__(kFogTX* kFogTY) k_fog_filter(const FogArgs a)
{
    __shared__ float4 tile[kFogSH * kFogSW];
    __shared__ float view_z[kFogZC];
    const int x0 = blockIdx.x * kFogTX, y0 = blockIdx.y * kFogTY, z0 = blockIdx.z * kFogZC;
    const int tid = threadIdx.y * kFogTX + threadIdx.x;
    const int x = x0 + threadIdx.x, y = y0 + threadIdx.y;
    const bool inside = x < a.W && y < a.H;
    const int nz = min(kFogZC, a.D - z0);
    const float ratio = dv(a.zfar, a.znear);

    // Per slice of the chunk: its view depth (:74-78).
    if (tid < nz) {
        const float tz = dv(add(float(z0 + tid), 0.5f), float(a.D));
        view_z[tid] = mul(a.znear, powf(ratio, tz));
    }
    // Per column: the normalised camera ray through the column's NDC and its cosine to the camera axis (:83-106).
    float ray[3], rdf = 1.f, lnr = 1.f;
    if (a.valid && inside) {
        const float u = dv(add(float(x), 0.5f), float(a.W)), v = dv(add(float(y), 0.5f), float(a.H));
        const float nx = sub(mul(u, 2.f), 1.f), ny = sub(1.f, mul(v, 2.f));
        float nh[4], fh[4], fwd[3];
        mat_vec(a.ivp, nx, ny, 0.f, 1.f, nh);
        mat_vec(a.ivp, 0.f, 0.f, 0.f, 1.f, fh);
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ray[k] = sub(dv(nh[k], nh[3]), a.cam[k]);
            fwd[k] = sub(dv(fh[k], fh[3]), a.cam[k]);
        }
        const float rl = __fsqrt_rn(add(add(mul(ray[0], ray[0]), mul(ray[1], ray[1])), mul(ray[2], ray[2])));
        const float fl = __fsqrt_rn(add(add(mul(fwd[0], fwd[0]), mul(fwd[1], fwd[1])), mul(fwd[2], fwd[2])));
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            ray[k] = dv(ray[k], rl);
            fwd[k] = dv(fwd[k], fl);
        }
        rdf = add(add(mul(ray[0], fwd[0]), mul(ray[1], fwd[1])), mul(ray[2], fwd[2]));
        rdf = rdf > 1e-4f ? rdf : 1e-4f;
        lnr = logf(ratio);
    }
    // In-grid members of the column's 3x3 box.
    float n = 0.f;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx)
            if (x + dx >= 0 && x + dx <= a.W - 1 && y + dy >= 0 && y + dy <= a.H - 1) n = add(n, 1.f);
    const float cnt = fmaxf(n, 1.f);

    for (int zi = 0; zi < nz; ++zi) {
        const int z = z0 + zi;
        const char* rs = a.raw + z * a.raw_slice;
        __syncthreads();  // the previous slice's tile is consumed (and view_z is written before the first use)
        for (int k = tid; k < kFogSH * kFogSW; k += kFogTX * kFogTY) {
            const int qy = y0 - 1 + k / kFogSW, qx = x0 - 1 + k % kFogSW;
            float4 q = make_float4(0.f, 0.f, 0.f, 0.f);
            if (qx >= 0 && qy >= 0 && qx < a.W && qy < a.H) q = ld_texel<RAW16>(rs, qy * a.raw_row + qx * (RAW16 ? 8LL : 16LL));
            tile[k] = q;
        }
        __syncthreads();
        if (!inside) continue;

        // 1. 3x3 mean over the in-grid neighbours of the slice (:152-166).  Cells outside the grid are staged
        // as +0 and summed without a test: the running sum starts at +0 and so is never -0, which makes adding
        // +0 an exact no-op, the same sums as the reference's skipped taps.
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int dy = -1; dy <= 1; ++dy)
#pragma unroll
            for (int dx = -1; dx <= 1; ++dx) {
                const float4 q = tile[(threadIdx.y + 1 + dy) * kFogSW + threadIdx.x + 1 + dx];
                s = make_float4(add(s.x, q.x), add(s.y, q.y), add(s.z, q.z), add(s.w, q.w));
            }
        const float4 sp = make_float4(dv(s.x, cnt), dv(s.y, cnt), dv(s.z, cnt), dv(s.w, cnt));
        char* op = a.out + z * a.out_slice + y * a.out_row + x * (OUT16 ? 8LL : 16LL);
        if (!a.valid) {
            st_texel<OUT16>(op, 0, sp);
            continue;
        }

        // 2. froxel centre on the column's ray at the slice's view depth (:100-106)
        const float t = dv(view_z[zi], rdf);
        const float wx = add(a.cam[0], mul(ray[0], t)), wy = add(a.cam[1], mul(ray[1], t)),
                    wz = add(a.cam[2], mul(ray[2], t));

        // 3. previous-frame froxel coordinates and rejections (:177-213)
        float pc[4];
        mat_vec(a.pvp, wx, wy, wz, 1.f, pc);
        if (pc[3] <= 1e-4f) {
            st_texel<OUT16>(op, 0, sp);
            continue;
        }
        const float ndx = dv(pc[0], pc[3]), ndy = dv(pc[1], pc[3]);
        const float fx = mul(add(mul(ndx, 0.5f), 0.5f), float(a.W));
        const float fy = mul(add(mul(-ndy, 0.5f), 0.5f), float(a.H));
        const float pz = pc[3];
        if (pz < a.znear || pz > a.zfar) {
            st_texel<OUT16>(op, 0, sp);
            continue;
        }
        const float lt = dv(logf(dv(pz, a.znear)), lnr);
        const float fz = sub(mul(lt, float(a.D)), 0.5f);
        if (fx < 0.f || fx >= float(a.W) || fy < 0.f || fy >= float(a.H) || fz < 0.f || fz >= float(a.D)) {
            st_texel<OUT16>(op, 0, sp);
            continue;
        }

        // 4. trilinear history, clamp-to-edge (:111-140), then the EMA (:216-225)
        const int ix = int(floorf(fx)), iy = int(floorf(fy)), iz = int(floorf(fz));
        const float ax = sub(fx, float(ix)), ay = sub(fy, float(iy)), az = sub(fz, float(iz));
        const int xa = min(max(ix, 0), a.W - 1), xb = min(max(ix + 1, 0), a.W - 1);
        const int ya = min(max(iy, 0), a.H - 1), yb = min(max(iy + 1, 0), a.H - 1);
        const int za = min(max(iz, 0), a.D - 1), zb = min(max(iz + 1, 0), a.D - 1);
        const long long tb = OUT16 ? 8LL : 16LL;
        const long long oxa = xa * tb, oxb = xb * tb, oya = ya * a.hist_row, oyb = yb * a.hist_row;
        const char* ha = a.hist + za * a.hist_slice;
        const char* hb = a.hist + zb * a.hist_slice;
        const float4 c000 = ld_texel<OUT16>(ha, oya + oxa), c100 = ld_texel<OUT16>(ha, oya + oxb);
        const float4 c010 = ld_texel<OUT16>(ha, oyb + oxa), c110 = ld_texel<OUT16>(ha, oyb + oxb);
        const float4 c001 = ld_texel<OUT16>(hb, oya + oxa), c101 = ld_texel<OUT16>(hb, oya + oxb);
        const float4 c011 = ld_texel<OUT16>(hb, oyb + oxa), c111 = ld_texel<OUT16>(hb, oyb + oxb);
        const float4 c0 = lerp4(lerp4(c000, c100, ax), lerp4(c010, c110, ax), ay);
        const float4 c1 = lerp4(lerp4(c001, c101, ax), lerp4(c011, c111, ax), ay);
        const float4 h = lerp4(c0, c1, az);
        st_texel<OUT16>(op, 0, lerp4(h, sp, a.alpha));
    }
}

struct VolGeom {
    long long row, slice, bytes;
    int texel;
};

int check_volume(const char* what, const tg_volume* v, int W, int H, int D, VolGeom& g)
{
    if (!v || !v->ptr) return fail(TG_ERR_INVALID, "%s: null volume", what);
    if (v->format != TG_FMT_RGBA16F && v->format != TG_FMT_RGBA32F)
        return fail(TG_ERR_INVALID, "%s: format %d is not RGBA16F or RGBA32F", what, v->format);
    g.texel = v->format == TG_FMT_RGBA16F ? 8 : 16;
    g.row = v->row_pitch_bytes ? v->row_pitch_bytes : (long long)W * g.texel;
    g.slice = v->slice_pitch_bytes ? v->slice_pitch_bytes : (long long)H * g.row;
    if (g.row < (long long)W * g.texel || g.row % g.texel) return fail(TG_ERR_INVALID, "%s: bad row pitch %lld", what, g.row);
    if (g.slice < (long long)H * g.row || g.slice % g.texel)
        return fail(TG_ERR_INVALID, "%s: bad slice pitch %lld", what, g.slice);
    if (reinterpret_cast<uintptr_t>(v->ptr) % g.texel)
        return fail(TG_ERR_INVALID, "%s: address must be a multiple of %d bytes", what, g.texel);
    g.bytes = (long long)(D - 1) * g.slice + (long long)(H - 1) * g.row + (long long)W * g.texel;
    return TG_OK;
}

bool overlap(const void* a, long long na, const void* b, long long nb)
{
    const uintptr_t pa = reinterpret_cast<uintptr_t>(a), pb = reinterpret_cast<uintptr_t>(b);
    return pa < pb + uintptr_t(nb) && pb < pa + uintptr_t(na);
}

} // namespace
} // namespace tg

using namespace tg;

int tg_fog_filter(const tg_fog_filter_params* p, const tg_volume* raw, const tg_volume* hist, const tg_volume* out,
                  void* stream)
{
    if (!p) return fail(TG_ERR_INVALID, "null parameters");
    const uint32_t W = p->froxel_width, H = p->froxel_height, D = p->froxel_depth;
    if (W == 0 || H == 0 || D == 0 || W > 65535u * kFogTX || H > 65535u * kFogTY || D > 65535u)
        return fail(TG_ERR_INVALID, "froxel grid %ux%ux%u outside 1..(2097120, 524280, 65535)", W, H, D);
    if (!(p->near_plane > 0.f) || !(p->far_plane > p->near_plane))
        return fail(TG_ERR_INVALID, "depth range needs 0 < near_plane < far_plane");
    VolGeom gr, gh, go;
    int st;
    if ((st = check_volume("inject_raw", raw, W, H, D, gr))) return st;
    if ((st = check_volume("history", hist, W, H, D, gh))) return st;
    if ((st = check_volume("output", out, W, H, D, go))) return st;
    if (hist->format != out->format) return fail(TG_ERR_INVALID, "history and output formats differ");
    if (overlap(out->ptr, go.bytes, raw->ptr, gr.bytes) || overlap(out->ptr, go.bytes, hist->ptr, gh.bytes))
        return fail(TG_ERR_INVALID, "output overlaps inject_raw or history");
    FogArgs a;
    for (int k = 0; k < 16; ++k) {
        a.ivp[k] = p->inv_view_projection[k];
        a.pvp[k] = p->prev_view_projection[k];
    }
    for (int k = 0; k < 3; ++k) a.cam[k] = p->camera_pos[k];
    a.alpha = p->alpha;
    a.znear = p->near_plane;
    a.zfar = p->far_plane;
    a.W = int(W);
    a.H = int(H);
    a.D = int(D);
    a.valid = p->history_valid != 0;
    a.raw = static_cast<const char*>(raw->ptr);
    a.hist = static_cast<const char*>(hist->ptr);
    a.out = static_cast<char*>(out->ptr);
    a.raw_row = gr.row;
    a.raw_slice = gr.slice;
    a.hist_row = gh.row;
    a.hist_slice = gh.slice;
    a.out_row = go.row;
    a.out_slice = go.slice;
    const dim3 grid((W + kFogTX - 1) / kFogTX, (H + kFogTY - 1) / kFogTY, (D + kFogZC - 1) / kFogZC),
        block(kFogTX, kFogTY);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const bool r16 = raw->format == TG_FMT_RGBA16F, o16 = out->format == TG_FMT_RGBA16F;
    if (r16 && o16)
        k_fog_filter<true, true><<<grid, block, 0, s>>>(a);
    else if (r16)
        k_fog_filter<true, false><<<grid, block, 0, s>>>(a);
    else if (o16)
        k_fog_filter<false, true><<<grid, block, 0, s>>>(a);
    else
        k_fog_filter<false, false><<<grid, block, 0, s>>>(a);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "fog filter launch failed: %s", cudaGetErrorString(e));
    return TG_OK;
}
