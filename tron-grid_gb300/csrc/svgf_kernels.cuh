// SVGF kernels for sm_103a: the reference-exact chain and the FULL chain.
//
// One thread per pixel over 2-D blocks of 32 x 4: a warp covers 32 adjacent
// pixels of one row, so every image access of a warp is one contiguous,
// coalesced segment (16 B/px float4 or 8 B/px half4 per lane).  The a-trous
// taps re-read neighbours through the read-only (L1) path.
#pragma once

#include "svgf_device.cuh"

namespace tg {

constexpr int kBlockX = 32;
constexpr int kBlockY = 4;

// Residue-major layout of the a-trous scratch for stride s = 2^lg: pixel
// (x, y) lives in plane (y mod s) * s + (x mod s) at position (x / s, y / s),
// each plane pw x ph.  For s = 1 this is the ordinary row-major image.  Level
// L reads its input in the layout of its own stride and writes its output in
// the layout of the next level's stride, so every tile a level stages and
// every 3x3 neighbourhood it reads is a contiguous run of memory.
struct ResLayout {
    int lg, pw, ph;
};

__device__ __forceinline__ size_t res_idx(const ResLayout& L, int x, int y)
{
    const int m = (1 << L.lg) - 1;
    return (size_t(((y & m) << L.lg) + (x & m)) * L.ph + (y >> L.lg)) * L.pw + (x >> L.lg);
}

__host__ __device__ inline ResLayout res_layout(int w, int h, int lg)
{
    ResLayout L;
    L.lg = lg;
    L.pw = (w + (1 << lg) - 1) >> lg;
    L.ph = (h + (1 << lg) - 1) >> lg;
    return L;
}

// ------------------------------------------------------------- REF-EXACT ----
// src/svgf_denoise.slang:152-275: the arguments of the REF_EXACT kernels
// (svgf_level.cuh; the init pass runs inside the first wavelet pass).

struct RefArgs {
    int w, h;
    Img raw;  // lighting_raw (b0)
    Img out;  // denoised_indirect (b3)
    const void* mom_prev; // moments_prev (b4)
    void* mom_curr;       // moments_curr (b5)
    const void* src;      // wavelet source (b1 or b2)
    void* dst;            // wavelet destination (b2 or b1)
    ResLayout lin, lout;  // scratch layouts of src and dst
    float phi;            // SIGMA_COLOR_BASE
    float alpha_m;        // ALPHA_MOMENTS
    float var_eps;        // VARIANCE_EPSILON
    int stride;
    int final_pass;
    int* err;             // device error word of bounded waits (may be null)
};

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
    size_t var_off;         // byte offset of the variance plane in col_src / col_dst
    size_t ghalf;           // FP32 records: index of the guide half-plane (16-byte units)
    float2* grad;           // per-pixel depth gradient (written by the temporal kernel)
    int* fb_flags;          // per 32x4 pixel block: 1 if a pixel needs the spatial variance fallback
    int* err;               // device error word (bounded waits that gave up); may be null
    ResLayout lin, lout;    // scratch layouts of col_src and col_dst
    float alpha, alpha_m, sigma_l, sigma_n, sigma_z;
    int sq_n; // squarings for sigma_n = 2^sq_n, -1 otherwise
    int max_history, fallback_frames;
    int level, stride, last;
};

// K1: guide write, reprojection (bilinear 2x2 with depth/normal test), history
// length, colour EMA and mean-centred moment EMA.  A pixel whose history is at
// least `fallback_frames` long also gets its level-0 variance-plane entry (the
// temporal variance as stored) here; the function returns true for the
// others, whose variance needs the neighbours' moments (K2).  Level 0 stages
// its input from tc, guide_cur and that plane, so no level-0 record is written.
template <int ST> __device__ __forceinline__ bool full_temporal_px(const FullArgs& a, int x, int y)
{
    typedef Stor<ST> S;
    typedef typename S::guide_t G;
    typedef typename S::c4_t C4;
    typedef typename S::mom_t M;
    const size_t i = size_t(y) * a.w + x;
    // The reprojection taps land next to (x, y) under small motion: start their lines towards L2 now, so the
    // gathers that depend on the motion load find them there instead of paying a second DRAM round trip.
    prefetch_l2(static_cast<const C4*>(a.hist_prev) + i);
    prefetch_l2(static_cast<const G*>(a.guide_prev) + i);
    prefetch_l2(static_cast<const M*>(a.mom_prev) + i);

    // Every load of this pixel is issued before its first store (the motion first: the reprojection gathers
    // depend on it), and the gathers before the guide and gradient work, which runs while they are in flight.
    const float2 mv = ld_motion(a.motion, x, y);
    const float4 c4 = ld_rgba(a.radiance, x, y);
    uint32_t enc = 0;
    float3 n = ld_normal(a.normal, x, y, ST == ST_FP16, enc);
    const float z = ld_depth(a.depth, x, y);
    const bool hl = x > 0, hr = x < a.w - 1, hu = y > 0, hd = y < a.h - 1;
    const float zl = hl ? ld_depth(a.depth, x - 1, y) : 0.0f, zr = hr ? ld_depth(a.depth, x + 1, y) : 0.0f;
    const float zu = hu ? ld_depth(a.depth, x, y - 1) : 0.0f, zd = hd ? ld_depth(a.depth, x, y + 1) : 0.0f;

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
    // All four taps' history, guide and moments are loaded before any of them
    // is tested, so the gathers overlap instead of forming a dependent chain.
    size_t tj[4];
    bool tin[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int tx = x0 + (k & 1), ty = y0 + (k >> 1);
        tin[k] = tx >= 0 && ty >= 0 && tx < a.w && ty < a.h;
        tj[k] = tin[k] ? size_t(ty) * a.w + tx : 0;
    }
    float4 thv[4], tg[4];
    float2 tm[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (tin[k]) {
            thv[k] = S::ld4(hp, tj[k]);
            tg[k] = S::ld_guide_raw(gp, tj[k]);
            tm[k] = S::ldm(mp, tj[k]);
        } else {
            thv[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            tg[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            tm[k] = make_float2(0.f, 0.f);
        }
    }

    if (ST == ST_FP16) n = oct16_decode_raw(enc);  // FP16 storage keeps the octahedral code
    const G gv = S::mk_guide(n, enc, z);
    static_cast<G*>(a.guide_cur)[i] = gv;
    const float gx = grad1(z, zl, zr, hl, hr);
    const float gy = grad1(z, zu, zd, hu, hd);
    a.grad[i] = make_float2(gx, gy);
    const float cr = S::qin(c4.x), cg = S::qin(c4.y), cb = S::qin(c4.z);
    const float gsum = __fadd_rn(fabsf(gx), fabsf(gy));
    const float ztol = __fadd_rn(__fadd_rn(__fmul_rn(kDepthRel, z), __fmul_rn(kDepthGrad, gsum)), kDepthAbs);
    float sw = 0.0f, hr_ = 0.0f, hg = 0.0f, hb = 0.0f, hmu = 0.0f;
    float tw[4];
    int lmax = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        tw[k] = 0.0f;
        if (!tin[k] || !(thv[k].w > 0.0f)) continue;
        if (!(fabsf(__fsub_rn(tg[k].w, z)) <= ztol)) continue;
        if (!normal_close(tg[k].x, tg[k].y, tg[k].z, n.x, n.y, n.z)) continue;
        tw[k] = bw[k];
        sw = __fadd_rn(sw, bw[k]);
        hr_ += bw[k] * thv[k].x;
        hg += bw[k] * thv[k].y;
        hb += bw[k] * thv[k].z;
        hmu += bw[k] * tm[k].x;
        lmax = max(lmax, int(thv[k].w));
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
            if (!(tw[k] > 0.0f)) continue;  // rejected taps never enter the sums
            const float dm = tm[k].x - hmu;
            hvv += tw[k] * (tm[k].y + dm * dm);
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
    const float4 tcv = make_float4(orr, og, ob, float(len));
    const float2 mom = make_float2(mu, var);
    S::st4(static_cast<C4*>(a.tc), i, tcv);
    S::stm(static_cast<M*>(a.mom_cur), i, mom);
    const float4 t = S::rt4(tcv);
    if (int(t.w) < a.fallback_frames) return true;
    Rec::st_var(a.col_dst, a.var_off, i, S::rtm(mom).y);
    return false;
}

// K2: for histories shorter than `fallback_frames`, the variance is a 7x7
// depth/normal-weighted spatial estimate from the neighbours' moments; writes
// the level-0 variance-plane entry of such a pixel.  The other pixels' entries
// come from K1.
//
// A CTA stages the guides (decoded) and moments of its pixel block plus a
// 3-pixel halo in shared memory.  Cells outside the image hold a zero normal,
// whose weight max(0, n.n')^sigma_n = 2^(sigma_n lg2 0) is exactly 0, so the
// sums equal those over the inside neighbours only.
constexpr int kVarHalo = 3;
constexpr int kVarTW = kBlockX + 2 * kVarHalo;
constexpr int kVarTH = kBlockY + 2 * kVarHalo;
struct VarTile {
    float4 g[kVarTH * kVarTW];  // unit normal, depth
    float2 m[kVarTH * kVarTW];  // luminance mean, variance
};

// `t` (the pixel's temporal colour and length) and `gr` (its depth gradient)
// are loaded by the caller before it stages the tile.
template <int ST>
__device__ __forceinline__ void full_variance_px(const FullArgs& a, int x, int y, int cell, const VarTile& vt, float4 t,
                                                 float2 gr)
{
    typedef Stor<ST> S;
    const size_t i = size_t(y) * a.w + x;
    const int len = int(t.w);
    if (len >= a.fallback_frames) return;
    const float2 mom = vt.m[cell];
    const float4 g = vt.g[cell];
    // w = max(0, n.n')^sigma_n exp(-|dz| / (sigma_z |grad z . off| + eps_z)), as one ex2;
    // offsets (dx, dy) and (-dx, -dy) share the depth scale kz
    const float A_ = a.sigma_z * gr.x * (1.0f / kLog2eF), B_ = a.sigma_z * gr.y * (1.0f / kLog2eF);
    const float ez = kEpsZ * (1.0f / kLog2eF);
    float kz[25];
#pragma unroll
    for (int q = 0; q < 25; ++q) {
        // q enumerates the offsets with dy < 0, or dy == 0 and dx <= 0 (the centre is q = 24)
        const int dy = q < 21 ? q / 7 - 3 : 0;
        const int dx = q < 21 ? q % 7 - 3 : q - 24;
        kz[q] = rcp_approx(fabsf(fmaf(float(dx), A_, float(dy) * B_)) + ez);
    }
    float s0 = 0.0f, s1 = 0.0f, s2 = 0.0f;
#pragma unroll
    for (int dy = -kVarHalo; dy <= kVarHalo; ++dy) {
#pragma unroll
        for (int dx = -kVarHalo; dx <= kVarHalo; ++dx) {
            const bool neg = dy < 0 || (dy == 0 && dx <= 0);
            const int ex = neg ? dx : -dx, ey = neg ? dy : -dy;
            const int q = ey < 0 ? (ey + 3) * 7 + (ex + 3) : 24 + ex;
            const int c = cell + dy * kVarTW + dx;
            const float4 n = vt.g[c];
            const float d = fmaf(n.z, g.z, fmaf(n.y, g.y, n.x * g.x));
            float e = -fabsf(n.w - g.w) * kz[q];
            e = fmaf(a.sigma_n, lg2_approx(fmaxf(d, 0.0f)), e);
            const float wgt = ex2_approx(e);
            const float2 m = vt.m[c];
            const float dm = m.x - mom.x;
            s0 += wgt;
            s1 = fmaf(wgt, dm, s1);
            s2 = fmaf(wgt, fmaf(dm, dm, m.y), s2);
        }
    }
    float var = mom.y;
    if (s0 > 0.0f) {
        const float m1 = s1 / s0;
        var = fmaxf(0.0f, s2 / s0 - m1 * m1);
    }
    Rec::st_var(a.col_dst, a.var_off, i, var);
}

// One kBlockX x kBlockY pixel block `blk` (row-major over the image's blocks)
// of K1 and K2.  K1 records in fb_flags[blk] whether any pixel of the block
// needs the spatial fallback; K2 skips the blocks that need none.  Every thread
// of the CTA calls these (K1 synchronises the CTA).
template <int ST> __device__ __forceinline__ void full_temporal_block(const FullArgs& a, int blk, int x, int y)
{
    const bool fb = (x < a.w && y < a.h) ? full_temporal_px<ST>(a, x, y) : false;
    const int any = __syncthreads_or(fb);
    if (threadIdx.x == 0 && threadIdx.y == 0) a.fb_flags[blk] = any;
}

// K2 on one flagged pixel block; (x, y) is this thread's pixel of the block.
template <int ST> __device__ __forceinline__ void full_variance_tile(const FullArgs& a, int x, int y, VarTile& vt)
{
    typedef Stor<ST> S;
    const int x0 = x - int(threadIdx.x) - kVarHalo, y0 = y - int(threadIdx.y) - kVarHalo;
    const typename S::guide_t* gc = static_cast<const typename S::guide_t*>(a.guide_cur);
    const typename S::mom_t* mc = static_cast<const typename S::mom_t*>(a.mom_cur);
    // this thread's own pixel inputs, loaded before the staging so that their latency overlaps it
    const bool own = x < a.w && y < a.h;
    const size_t i = own ? size_t(y) * a.w + x : 0;
    const float4 t = own ? S::ld4(static_cast<const typename S::c4_t*>(a.tc), i) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 gr = own ? a.grad[i] : make_float2(0.f, 0.f);
    for (int k = threadIdx.y * kBlockX + threadIdx.x; k < kVarTH * kVarTW; k += kBlockX * kBlockY) {
        const int qy = y0 + k / kVarTW, qx = x0 + k % kVarTW;
        float4 g = make_float4(0.f, 0.f, 0.f, 0.f);
        float2 m = make_float2(0.f, 0.f);
        if (qx >= 0 && qy >= 0 && qx < a.w && qy < a.h) {
            const size_t j = size_t(qy) * a.w + qx;
            g = S::ld_guide_w(gc, j);
            m = S::ldm(mc, j);
        }
        vt.g[k] = g;
        vt.m[k] = m;
    }
    __syncthreads();
    if (own) full_variance_px<ST>(a, x, y, (int(threadIdx.y) + kVarHalo) * kVarTW + int(threadIdx.x) + kVarHalo, vt, t, gr);
    __syncthreads();  // the tile's storage is reused by the caller's next block
}

// K2 grids: a CTA takes the pixel blocks base + t * stride (t < kVarPerCta) of
// its chunk, compacts the flagged ones into a shared list and runs only those,
// so that the mostly unflagged blocks of a frame cost one parallel flag read
// per chunk instead of one CTA each.
constexpr int kVarPerCta = 32;

__host__ __device__ inline int variance_grid(int items, int sms)
{
    const int lo = (items + kVarPerCta - 1) / kVarPerCta, hi = items < 6 * sms ? items : 6 * sms;
    return lo > hi ? lo : hi;
}

struct VarList {
    int item[kVarPerCta];
    int n;
};

// Fills `l` with the flagged items of the chunk at `base`; `flag(item)` reads an item's flag.
template <class Flag>
__device__ __forceinline__ void variance_compact(int base, int stride, int items, Flag flag, VarList& l)
{
    const int tid = threadIdx.y * kBlockX + threadIdx.x;
    if (tid == 0) l.n = 0;
    __syncthreads();
    if (tid < kVarPerCta) {
        const int item = base + tid * stride;
        if (item < items && flag(item)) l.item[atomicAdd(&l.n, 1)] = item;
    }
    __syncthreads();
}

// 8 CTAs of 128 threads per SM (64 registers a thread): 3% faster than 4 of 256.
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY, 8) k_full_temporal(FullArgs a)
{
    pdl_begin();
    full_temporal_block<ST>(a, blockIdx.y * gridDim.x + blockIdx.x, blockIdx.x * kBlockX + threadIdx.x,
                            blockIdx.y * kBlockY + threadIdx.y);
}

// One chunk per CTA: gridDim.x = variance_grid(blocks, SMs) covers every block.
template <int ST> __global__ void __launch_bounds__(kBlockX* kBlockY) k_full_variance(FullArgs a)
{
    __shared__ VarTile vt;
    __shared__ VarList l;
    pdl_begin();
    const int tx = (a.w + kBlockX - 1) / kBlockX, items = tx * ((a.h + kBlockY - 1) / kBlockY);
    const int* flags = a.fb_flags;
    variance_compact(int(blockIdx.x), int(gridDim.x), items, [flags](int b) { return __ldcg(flags + b) != 0; }, l);
    const int n = l.n;
    for (int e = 0; e < n; ++e) {
        const int b = l.item[e];
        full_variance_tile<ST>(a, (b % tx) * kBlockX + threadIdx.x, (b / tx) * kBlockY + threadIdx.y, vt);
    }
}

} // namespace tg
