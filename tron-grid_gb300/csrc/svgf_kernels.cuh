// SVGF kernels for sm_103a: the reference-exact chain and the FULL chain.
//
// One thread per pixel over 2-D blocks of 32 x 8: a warp covers 32 adjacent
// pixels of one row, so every image access of a warp is one contiguous,
// coalesced segment (16 B/px float4 or 8 B/px half4 per lane).  The a-trous
// taps re-read neighbours through the read-only (L1) path.
#pragma once

#include "svgf_device.cuh"

namespace tg {

constexpr int kBlockX = 32;
constexpr int kBlockY = 8;

// ------------------------------------------------------------- REF-EXACT ----
// src/svgf_denoise.slang:152-275, one kernel per pass.

struct RefArgs {
    int w, h;
    Img raw;  // lighting_raw (b0)
    Img out;  // denoised_indirect (b3)
    const void* mom_prev; // moments_prev (b4)
    void* mom_curr;       // moments_curr (b5)
    const void* src;      // wavelet source (b1 or b2)
    void* dst;            // wavelet destination (b2 or b1)
    float phi;            // SIGMA_COLOR_BASE
    float alpha_m;        // ALPHA_MOMENTS
    float var_eps;        // VARIANCE_EPSILON
    int stride;
    int final_pass;
};

// Pass 0 (src/svgf_denoise.slang:176-191): luminance moments EMA, sqrt-variance.
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY) k_ref_init(RefArgs a)
{
    typedef Stor<ST> S;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.w || y >= a.h) return;
    const size_t i = size_t(y) * a.w + x;
    float4 c = ld_rgba(a.raw, x, y);
    float l = lum(c.x, c.y, c.z);
    float2 mp = S::ldm(static_cast<const typename S::mom_t*>(a.mom_prev), i);
    float m1 = __fadd_rn(mp.x, __fmul_rn(__fsub_rn(l, mp.x), a.alpha_m));
    float m2 = __fadd_rn(mp.y, __fmul_rn(__fsub_rn(__fmul_rn(l, l), mp.y), a.alpha_m));
    float var = fmaxf(__fsub_rn(m2, __fmul_rn(m1, m1)), 0.0f);
    float sd = __fsqrt_rn(__fadd_rn(var, a.var_eps));
    typename S::mom_t* mc = static_cast<typename S::mom_t*>(a.mom_curr);
    if (ST == ST_FP16) {
        // rg16f store: plain round-to-nearest (overflows to inf as the reference does).
        reinterpret_cast<uint32_t*>(mc)[i] = pack_h2(m1, m2);
    } else {
        S::stm(mc, i, make_float2(m1, m2));
    }
    S::st4(static_cast<typename S::c4_t*>(a.dst), i, make_float4(c.x, c.y, c.z, sd));
}

// Passes 1..3 (src/svgf_denoise.slang:209-274): 5x5 B3 taps at `stride`,
// clamp-to-edge, luminance edge stop exp(-|dl| / max(phi * sqrt_var, eps)).
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY) k_ref_level(RefArgs a)
{
    typedef Stor<ST> S;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.w || y >= a.h) return;
    const typename S::c4_t* src = static_cast<const typename S::c4_t*>(a.src);
    const size_t i = size_t(y) * a.w + x;
    const float4 c = S::ld4(src, i);
    const float cl = lum(c.x, c.y, c.z);
    const float sigma = fmaxf(__fmul_rn(a.phi, c.w), a.var_eps);
    const float nis = -1.0f / sigma;
    const int mx = a.w - 1, my = a.h - 1, s = a.stride;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f, ws = 0.0f;
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
        const int sy = min(max(y + dy * s, 0), my);
        const size_t row = size_t(sy) * a.w;
#pragma unroll
        for (int dx = -2; dx <= 2; ++dx) {
            const int sx = min(max(x + dx * s, 0), mx);
            const float4 q = S::ld4(src, row + sx);
            const float ql = lum(q.x, q.y, q.z);
            const float kw = b3(dx + 2) * b3(dy + 2);
            const float tw = kw * __expf(fabsf(ql - cl) * nis);
            sr = fmaf(q.x, tw, sr);
            sg = fmaf(q.y, tw, sg);
            sb = fmaf(q.z, tw, sb);
            ws += tw;
        }
    }
    float4 o;
    if (ws > 1e-6f) {
        o = make_float4(__fdiv_rn(sr, ws), __fdiv_rn(sg, ws), __fdiv_rn(sb, ws), c.w);
    } else {
        o = make_float4(c.x, c.y, c.z, c.w);
    }
    if (a.final_pass) {
        o.w = 1.0f;
        if (ST == ST_FP16) o = make_float4(q16(o.x), q16(o.y), q16(o.z), 1.0f);
        st_rgba(a.out, x, y, o);
    } else {
        S::st4(static_cast<typename S::c4_t*>(a.dst), i, o);
    }
}

// ------------------------------------------------------------------ FULL ----

struct FullArgs {
    int w, h;
    Img radiance, depth, normal, motion, out;
    const void* guide_prev;
    const void* hist_prev;
    const void* mom_prev;
    void* guide_cur;
    void* hist_cur;
    void* mom_cur;
    void* tc;
    const void* col_src;
    void* col_dst;
    float alpha, alpha_m, sigma_l, sigma_n, sigma_z;
    int sq_n; // squarings for sigma_n = 2^sq_n, -1 otherwise
    int max_history, fallback_frames;
    int level, stride, last;
};

template <int ST> __device__ __forceinline__ float guide_z(const FullArgs& a, int x, int y)
{
    return Stor<ST>::ld_guide_z(static_cast<const typename Stor<ST>::guide_t*>(a.guide_cur), size_t(y) * a.w + x);
}

template <int ST> __device__ __forceinline__ void guide_grad(const FullArgs& a, int x, int y, float z, float& gx,
                                                             float& gy)
{
    const bool hl = x > 0, hr = x < a.w - 1, hu = y > 0, hd = y < a.h - 1;
    float zl = hl ? guide_z<ST>(a, x - 1, y) : 0.0f;
    float zr = hr ? guide_z<ST>(a, x + 1, y) : 0.0f;
    float zu = hu ? guide_z<ST>(a, x, y - 1) : 0.0f;
    float zd = hd ? guide_z<ST>(a, x, y + 1) : 0.0f;
    gx = grad1(z, zl, zr, hl, hr);
    gy = grad1(z, zu, zd, hu, hd);
}

// K1: guide write, reprojection (bilinear 2x2 with depth/normal test), history
// length, colour EMA and mean-centred moment EMA.
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY) k_full_temporal(FullArgs a)
{
    typedef Stor<ST> S;
    typedef typename S::guide_t G;
    typedef typename S::c4_t C4;
    typedef typename S::mom_t M;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.w || y >= a.h) return;
    const size_t i = size_t(y) * a.w + x;

    uint32_t enc = 0;
    float3 n = ld_normal(a.normal, x, y, ST == ST_FP16, enc);
    if (ST == ST_FP16 && a.normal.fmt != TG_FMT_OCT16) n = oct16_decode(enc);
    const float z = ld_depth(a.depth, x, y);
    static_cast<G*>(a.guide_cur)[i] = S::mk_guide(n, enc, z);

    const bool hl = x > 0, hr = x < a.w - 1, hu = y > 0, hd = y < a.h - 1;
    const float gx = grad1(z, hl ? ld_depth(a.depth, x - 1, y) : 0.0f, hr ? ld_depth(a.depth, x + 1, y) : 0.0f, hl, hr);
    const float gy = grad1(z, hu ? ld_depth(a.depth, x, y - 1) : 0.0f, hd ? ld_depth(a.depth, x, y + 1) : 0.0f, hu, hd);

    const float4 c4 = ld_rgba(a.radiance, x, y);
    const float cr = S::qin(c4.x), cg = S::qin(c4.y), cb = S::qin(c4.z);
    const float gsum = __fadd_rn(fabsf(gx), fabsf(gy));
    const float ztol = __fadd_rn(__fadd_rn(__fmul_rn(kDepthRel, z), __fmul_rn(kDepthGrad, gsum)), kDepthAbs);
    const float2 mv = ld_motion(a.motion, x, y);
    const float px = __fadd_rn(float(x), mv.x);
    const float py = __fadd_rn(float(y), mv.y);
    const float fx0 = floorf(px), fy0 = floorf(py);
    const float fx = __fsub_rn(px, fx0), fy = __fsub_rn(py, fy0);
    const float lim = 1073741824.0f;
    const int x0 = int(fmaxf(-lim, fminf(lim, fx0)));
    const int y0 = int(fmaxf(-lim, fminf(lim, fy0)));
    const float ofx = __fsub_rn(1.0f, fx), ofy = __fsub_rn(1.0f, fy);
    const float bw[4] = {__fmul_rn(ofx, ofy), __fmul_rn(fx, ofy), __fmul_rn(ofx, fy), __fmul_rn(fx, fy)};

    const G* gp = static_cast<const G*>(a.guide_prev);
    const C4* hp = static_cast<const C4*>(a.hist_prev);
    const M* mp = static_cast<const M*>(a.mom_prev);
    float sw = 0.0f, hr_ = 0.0f, hg = 0.0f, hb = 0.0f, hmu = 0.0f;
    float tmu[4], tvar[4], tw[4];
    int lmax = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        tw[k] = 0.0f;
        tmu[k] = 0.0f;
        tvar[k] = 0.0f;
        const int tx = x0 + (k & 1), ty = y0 + (k >> 1);
        if (tx < 0 || ty < 0 || tx >= a.w || ty >= a.h) continue;
        const size_t j = size_t(ty) * a.w + tx;
        const float4 hv = S::ld4(hp, j);
        if (!(hv.w > 0.0f)) continue;
        const float4 g = S::ld_guide(gp, j);
        if (!(fabsf(__fsub_rn(g.w, z)) <= ztol)) continue;
        const float d = dot3_rn(g.x, g.y, g.z, n.x, n.y, n.z);
        if (!(d >= kNormalCos)) continue;
        const float2 m = S::ldm(mp, j);
        tw[k] = bw[k];
        tmu[k] = m.x;
        tvar[k] = m.y;
        sw = __fadd_rn(sw, bw[k]);
        hr_ += bw[k] * hv.x;
        hg += bw[k] * hv.y;
        hb += bw[k] * hv.z;
        hmu += bw[k] * m.x;
        lmax = max(lmax, int(hv.w));
    }
    const float l = lum(cr, cg, cb);
    float orr, og, ob, mu, var;
    int len;
    if (sw > 0.0f) {
        const float inv = 1.0f / sw;
        hr_ *= inv;
        hg *= inv;
        hb *= inv;
        hmu *= inv;
        float hvv = 0.0f;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float dm = tmu[k] - hmu;
            hvv += tw[k] * (tvar[k] + dm * dm);
        }
        hvv *= inv;
        len = min(lmax + 1, a.max_history);
        const float ac = fmaxf(a.alpha, 1.0f / float(len));
        const float am = fmaxf(a.alpha_m, 1.0f / float(len));
        orr = hr_ + ac * (cr - hr_);
        og = hg + ac * (cg - hg);
        ob = hb + ac * (cb - hb);
        const float dl = l - hmu;
        mu = hmu + am * dl;
        var = (1.0f - am) * (hvv + am * dl * dl);
    } else {
        len = 1;
        orr = cr;
        og = cg;
        ob = cb;
        mu = l;
        var = 0.0f;
    }
    S::st4(static_cast<C4*>(a.tc), i, make_float4(orr, og, ob, float(len)));
    S::stm(static_cast<M*>(a.mom_cur), i, make_float2(mu, var));
}

// K2: variance per pixel: the temporal moment variance, or for histories
// shorter than `fallback_frames` a 7x7 depth/normal-weighted spatial estimate
// from the neighbours' moments.  Writes col = (colour, variance).
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY) k_full_variance(FullArgs a)
{
    typedef Stor<ST> S;
    typedef typename S::guide_t G;
    typedef typename S::c4_t C4;
    typedef typename S::mom_t M;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.w || y >= a.h) return;
    const size_t i = size_t(y) * a.w + x;
    const C4* tc = static_cast<const C4*>(a.tc);
    const M* mc = static_cast<const M*>(a.mom_cur);
    const G* gc = static_cast<const G*>(a.guide_cur);
    const float4 t = S::ld4(tc, i);
    const int len = int(t.w);
    const float2 mom = S::ldm(mc, i);
    float var = mom.y;
    if (len < a.fallback_frames) {
        const float4 g = S::ld_guide(gc, i);
        float gx, gy;
        guide_grad<ST>(a, x, y, g.w, gx, gy);
        float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
        for (int dy = -3; dy <= 3; ++dy) {
            const int qy = y + dy;
            if (qy < 0 || qy >= a.h) continue;
            for (int dx = -3; dx <= 3; ++dx) {
                const int qx = x + dx;
                if (qx < 0 || qx >= a.w) continue;
                const size_t j = size_t(qy) * a.w + qx;
                const float4 q = S::ld_guide(gc, j);
                const float d = dot3_rn(q.x, q.y, q.z, g.x, g.y, g.z);
                const float wn = normal_weight(d, a.sq_n, a.sigma_n);
                if (!(wn > 0.0f)) continue;
                const float den = a.sigma_z * fabsf(float(dx) * gx + float(dy) * gy) + kEpsZ;
                const float ez = fabsf(q.w - g.w) / den;
                const float wgt = wn * __expf(-ez);
                const float2 m = S::ldm(mc, j);
                const float dm = m.x - mom.x;
                s0 += wgt;
                s1 += wgt * dm;
                s2 += wgt * (dm * dm + m.y);
            }
        }
        if (s0 > 0.0f) {
            const float m1 = s1 / s0;
            var = fmaxf(0.0f, s2 / s0 - m1 * m1);
        }
    }
    S::st4_sat_w(static_cast<C4*>(a.col_dst), i, make_float4(t.x, t.y, t.z, var));
}

// K3: one a-trous level at stride 2^level.  Edge stops: luminance
// exp(-|dl| / (sigma_l sqrt(g3x3 var) + eps)), normal max(0, n.n')^sigma_n,
// depth exp(-|dz| / (sigma_z |grad z . offset| + eps)).  Taps outside the image
// are skipped.  Variance is propagated with squared weights.  Level 0 writes
// the colour history; the last level writes the caller's output.
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY) k_full_level(FullArgs a)
{
    typedef Stor<ST> S;
    typedef typename S::guide_t G;
    typedef typename S::c4_t C4;
    const int x = blockIdx.x * kBlockX + threadIdx.x;
    const int y = blockIdx.y * kBlockY + threadIdx.y;
    if (x >= a.w || y >= a.h) return;
    const size_t i = size_t(y) * a.w + x;
    const C4* src = static_cast<const C4*>(a.col_src);
    const G* gc = static_cast<const G*>(a.guide_cur);
    const float4 c = S::ld4(src, i);
    const float cl = lum(c.x, c.y, c.z);
    const float4 g = S::ld_guide(gc, i);
    float gx, gy;
    guide_grad<ST>(a, x, y, g.w, gx, gy);

    float gv = 0.0f, gw = 0.0f;
#pragma unroll
    for (int dy = -1; dy <= 1; ++dy) {
        const int qy = y + dy;
        if (qy < 0 || qy >= a.h) continue;
#pragma unroll
        for (int dx = -1; dx <= 1; ++dx) {
            const int qx = x + dx;
            if (qx < 0 || qx >= a.w) continue;
            const float k = (dy == 0 ? 0.5f : 0.25f) * (dx == 0 ? 0.5f : 0.25f);
            gv += k * S::ld4_w(src, size_t(qy) * a.w + qx);
            gw += k;
        }
    }
    gv = __fdiv_rn(gv, gw);
    const float inv_l = 1.0f / (a.sigma_l * sqrtf(fmaxf(gv, 0.0f)) + kEpsL);
    const int s = a.stride;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f, sw = 0.0f, sv = 0.0f;
#pragma unroll
    for (int dy = -2; dy <= 2; ++dy) {
        const int qy = y + dy * s;
        if (qy < 0 || qy >= a.h) continue;
#pragma unroll
        for (int dx = -2; dx <= 2; ++dx) {
            const int qx = x + dx * s;
            if (qx < 0 || qx >= a.w) continue;
            const size_t j = size_t(qy) * a.w + qx;
            const float4 q = S::ld_guide(gc, j);
            const float d = dot3_rn(q.x, q.y, q.z, g.x, g.y, g.z);
            const float wn = normal_weight(d, a.sq_n, a.sigma_n);
            if (!(wn > 0.0f)) continue;
            const float4 v = S::ld4(src, j);
            const float ql = lum(v.x, v.y, v.z);
            const float el = fabsf(cl - ql) * inv_l;
            const float den = a.sigma_z * fabsf(float(s) * (float(dx) * gx + float(dy) * gy)) + kEpsZ;
            const float ez = __fdividef(fabsf(g.w - q.w), den);
            const float wgt = b3(dx + 2) * b3(dy + 2) * wn * __expf(-(el + ez));
            sr = fmaf(wgt, v.x, sr);
            sg = fmaf(wgt, v.y, sg);
            sb = fmaf(wgt, v.z, sb);
            sw += wgt;
            sv = fmaf(wgt * wgt, v.w, sv);
        }
    }
    float4 o;
    if (sw > 0.0f) {
        const float inv = 1.0f / sw;
        o = make_float4(sr * inv, sg * inv, sb * inv, sv * (inv * inv));
    } else {
        o = c;
    }
    if (a.level == 0) {
        const float len = S::ld4_w(static_cast<const C4*>(a.tc), i);
        S::st4(static_cast<C4*>(a.hist_cur), i, make_float4(o.x, o.y, o.z, len));
    }
    if (a.last) {
        st_rgba(a.out, x, y, make_float4(S::qin(o.x), S::qin(o.y), S::qin(o.z), 1.0f));
    } else {
        S::st4_sat_w(static_cast<C4*>(a.col_dst), i, o);
    }
}

} // namespace tg
