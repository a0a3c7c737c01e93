// A-trous level kernels, shared-memory tiled on the stride sub-lattice.
//
// At stride s a 5x5 tap footprint spans 4s+1 pixels, but the taps of a pixel
// all lie on its residue class {(x, y) : x = a (mod s), y = b (mod s)}.  A CTA
// therefore works on one residue class (a, b): it stages a dense
// (TX + 4) x (TY + 4) tile of that class (the TX x TY outputs plus a 2-pixel
// halo in sub-lattice units) in shared memory, and every tap of every output is
// a shared-memory neighbour.  Block ids enumerate the s*s residue classes
// fastest, so the CTAs that share DRAM sectors run back to back and meet in L2.
//
// Staged records carry what every tap needs, decoded once per staged pixel:
//   A = (r, g, b, luminance)   N = (nx, ny, nz, z)   V = variance
// A pixel outside the image is staged as an all-zero record: its normal is the
// zero vector, so its normal weight max(0, n.n')^sigma_n is exactly 0 and it
// drops out of every sum without a branch (FULL mode skips outside taps).
// In REF_EXACT mode the staged coordinates are clamped to the image instead,
// which reproduces the reference's clamp-to-edge taps
// (src/svgf_denoise.slang:231-232) exactly.
//
// Every weight is folded into one base-2 exponent per tap:
//   w = 2^( log2 h  -  log2e |dz| / (sigma_z |grad z . off| + eps_z)
//                   -  log2e |dl| / (sigma_l sqrt(g3x3 var) + eps_l)
//                   +  sigma_n log2 max(0, n.n') )
// so a tap costs one lg2 and one ex2 on the SFU plus ~15 FP32 operations.
// Each thread computes R outputs of one sub-lattice column, so a staged tap
// record is read from shared memory once for up to R outputs.
#pragma once

#include "svgf_device.cuh"

namespace tg {

constexpr int kLvTX = 32;      // outputs per tile row (one warp)
constexpr int kLvRows = 8;     // thread rows per CTA
constexpr float kLog2e = kLog2eF;
// log2 of the B3 taps 1/16, 1/4, 3/8, 1/4, 1/16.
__device__ __forceinline__ constexpr float log2_b3(int i)
{
    return i == 2 ? -1.4150374992788438f : ((i == 1 || i == 3) ? -2.0f : -4.0f);
}

struct LevelGeom {
    int s;        // stride
    int sub_w;    // ceil(W / s): sub-lattice columns of residue 0
    int sub_h;    // ceil(H / s)
    int tiles_x;  // ceil(sub_w / TX)
    int tiles_y;  // ceil(sub_h / TY)
};

template <int R> struct LevelTile {
    static constexpr int TX = kLvTX;
    static constexpr int TY = kLvRows * R;
    static constexpr int SW = TX + 4;
    static constexpr int SH = TY + 4;
    static constexpr int N = SW * SH;
};

template <int R> struct LevelSmem {
    float4 A[LevelTile<R>::N];
    float4 N[LevelTile<R>::N];
    float V[LevelTile<R>::N];
};

// Maps tile `bid` to (residue a, b) and its tile origin in sub-lattice units.
__device__ __forceinline__ void level_block(const LevelGeom& g, int bid, int TX, int TY, int& ra, int& rb, int& i0,
                                            int& j0)
{
    const int ss = g.s * g.s;
    const int res = bid % ss;
    const int tile = bid / ss;
    ra = res % g.s;
    rb = res / g.s;
    i0 = (tile % g.tiles_x) * TX;
    j0 = (tile / g.tiles_x) * TY;
}

// ------------------------------------------------------------------ FULL ----

// Per-level arguments of an a-trous level (the rest comes from FullArgs).
struct LevelArgs {
    const void* col_src;
    void* col_dst;
    int level, last;
    ResLayout lin, lout;
};

__host__ __device__ inline LevelArgs level_args_of(const FullArgs& a)
{
    LevelArgs l;
    l.col_src = a.col_src;
    l.col_dst = a.col_dst;
    l.level = a.level;
    l.last = a.last;
    l.lin = a.lin;
    l.lout = a.lout;
    return l;
}

// One tile of one level.  The caller synchronises the CTA before reusing `sm`.
template <int ST, int R>
__device__ __forceinline__ void full_level_tile(const FullArgs& a, const LevelArgs& lv, const LevelGeom& g, int bid,
                                                LevelSmem<R>& sm)
{
    typedef Stor<ST> S;
    typedef typename S::guide_t G;
    typedef typename S::c4_t C4;
    typedef LevelTile<R> T;
    float4* sA = sm.A;
    float4* sN = sm.N;
    float* sV = sm.V;

    int ra, rb, i0, j0;
    level_block(g, bid, T::TX, T::TY, ra, rb, i0, j0);
    const int s = g.s, lg = lv.lin.lg, m = s - 1;
    const int pw = lv.lin.pw;
    const int P = lv.lin.pw * lv.lin.ph;  // elements per residue plane (< 2^31)
    const C4* src = static_cast<const C4*>(lv.col_src);
    const G* gc = static_cast<const G*>(a.guide_cur);
    const int ci = threadIdx.x;         // tile column of this thread's outputs
    const int cj0 = threadIdx.y * R;    // first tile row of this thread's outputs
    const int cx = ra + s * (i0 + ci);

    // ---- per-centre global reads first, so that their latency overlaps the
    // staging below: the depth gradient and the 3x3 variance neighbourhood.
    // In the residue-major layout the index of (qx, qy) separates into a
    // column term and a row term, and a warp's 32 reads are contiguous.
    int cxo[3];
    bool cxv[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int qx = cx + e - 1;
        cxv[e] = unsigned(qx) < unsigned(a.w);
        cxo[e] = (qx & m) * P + (qx >> lg);
    }
    const float kx_sum = (cxv[0] ? 0.25f : 0.f) + (cxv[1] ? 0.5f : 0.f) + (cxv[2] ? 0.25f : 0.f);
    float vn9[R][9];
    float2 gr[R];
    bool valid[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int y = rb + s * (j0 + cj0 + k);
        valid[k] = cx < a.w && y < a.h;
        gr[k] = valid[k] ? a.grad[y * a.w + cx] : make_float2(0.f, 0.f);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const int qy = y + f - 1;
            const bool oy = valid[k] && unsigned(qy) < unsigned(a.h);
            const int ro = ((qy & m) << lg) * P + (qy >> lg) * pw;
#pragma unroll
            for (int e = 0; e < 3; ++e) vn9[k][f * 3 + e] = (oy && cxv[e]) ? S::ld4_w(src, ro + cxo[e]) : 0.f;
        }
    }

    // ---- stage the tile: (TX+4) x (TY+4) sub-lattice pixels, zero outside.
    const int plane = ((rb << lg) + ra) * P;
    for (int k = threadIdx.y * kLvTX + threadIdx.x; k < T::N; k += kLvTX * kLvRows) {
        const int sj = k / T::SW, si = k - sj * T::SW;
        const int j = j0 + sj - 2, i = i0 + si - 2;
        const int y = rb + s * j, x = ra + s * i;
        float4 va = make_float4(0.f, 0.f, 0.f, 0.f), vn = make_float4(0.f, 0.f, 0.f, 0.f);
        float vv = 0.f;
        if (j >= 0 && i >= 0 && y < a.h && x < a.w) {
            const float4 c = S::ld4(src, plane + j * pw + i);
            va = make_float4(c.x, c.y, c.z, lum(c.x, c.y, c.z));
            vv = c.w;
            vn = S::ld_guide_w(gc, y * a.w + x);
        }
        sA[k] = va;
        sN[k] = vn;
        sV[k] = vv;
    }
    __syncthreads();

    // ---- per-centre set-up.  Exponent factors are pre-scaled by log2(e).
    float lp[R], kl[R], zp[R], nx[R], ny[R], nz[R], kz[R][13];
    float ar[R], ag[R], ab[R], aw[R], av[R];
    const float zs = a.sigma_z * float(s) * (1.0f / kLog2e);
    const float ez = kEpsZ * (1.0f / kLog2e);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int c = (cj0 + k + 2) * T::SW + ci + 2;
        const float4 A = sA[c], N = sN[c];
        lp[k] = A.w;
        zp[k] = N.w;
        nx[k] = N.x;
        ny[k] = N.y;
        nz[k] = N.z;
        ar[k] = ag[k] = ab[k] = aw[k] = av[k] = 0.f;
        // 3x3 Gaussian (1 2 1)x(1 2 1)/16 of the variance over inside pixels
        const int y = rb + s * (j0 + cj0 + k);
        const float ky_sum = (unsigned(y - 1) < unsigned(a.h) ? 0.25f : 0.f) + 0.5f +
                             (unsigned(y + 1) < unsigned(a.h) ? 0.25f : 0.f);
        float sv = 0.f;
#pragma unroll
        for (int q = 0; q < 9; ++q) sv = fmaf((q / 3 == 1 ? 0.5f : 0.25f) * (q % 3 == 1 ? 0.5f : 0.25f), vn9[k][q], sv);
        const float gv = sv * rcp_approx(ky_sum * kx_sum);
        kl[k] = kLog2e * rcp_approx(a.sigma_l * sqrt_approx(fmaxf(gv, 0.f)) + kEpsL);
        const float A_ = zs * gr[k].x, B_ = zs * gr[k].y;
        // kz for the 13 offsets (dx, dy) with dy > 0 or (dy == 0 and dx >= 0);
        // the other 12 offsets are their negations and share the value.
#pragma unroll
        for (int q = 0; q < 13; ++q) {
            const int dx = (q < 3) ? q : ((q - 3) % 5) - 2;
            const int dy = (q < 3) ? 0 : 1 + (q - 3) / 5;
            kz[k][q] = rcp_approx(fabsf(float(dx) * A_ + float(dy) * B_) + ez);
        }
    }

    // ---- taps: rows r = 0 .. R+3 of this thread's strip, 5 columns each.
    // A warp (one strip row of 32 columns) whose outputs all lie outside the
    // sub-lattice skips the taps.
    bool any_valid = false;
#pragma unroll
    for (int k = 0; k < R; ++k) any_valid |= valid[k];
    const float sn = a.sigma_n;
    if (__any_sync(0xffffffffu, any_valid)) {
#pragma unroll
        for (int r = 0; r < R + 4; ++r) {
#pragma unroll
            for (int dx = -2; dx <= 2; ++dx) {
                const int q = (cj0 + r) * T::SW + ci + 2 + dx;
                const float4 A = sA[q], N = sN[q];
                const float V = sV[q];
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int dy = r - 2 - k;
                    if (dy < -2 || dy > 2) continue;
                    const int ddx = (dy > 0 || (dy == 0 && dx >= 0)) ? dx : -dx;
                    const int ddy = dy >= 0 ? dy : -dy;
                    const int qi = ddy == 0 ? ddx : 3 + (ddy - 1) * 5 + (ddx + 2);
                    const float d = fmaf(nz[k], N.z, fmaf(ny[k], N.y, nx[k] * N.x));
                    float t = fmaf(-fabsf(zp[k] - N.w), kz[k][qi], log2_b3(dx + 2) + log2_b3(dy + 2));
                    t = fmaf(-fabsf(lp[k] - A.w), kl[k], t);
                    t = fmaf(sn, lg2_approx(fmaxf(d, 0.f)), t);
                    const float w = ex2_approx(t);
                    ar[k] = fmaf(w, A.x, ar[k]);
                    ag[k] = fmaf(w, A.y, ag[k]);
                    ab[k] = fmaf(w, A.z, ab[k]);
                    aw[k] += w;
                    av[k] = fmaf(w * w, V, av[k]);
                }
            }
        }
    }

    // ---- outputs.
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!valid[k]) continue;
        const int y = rb + s * (j0 + cj0 + k);
        const int i = y * a.w + cx;
        float4 o;
        if (aw[k] > 0.f) {
            const float inv = rcp_approx(aw[k]);
            o = make_float4(ar[k] * inv, ag[k] * inv, ab[k] * inv, av[k] * (inv * inv));
        } else {
            const int c = (cj0 + k + 2) * T::SW + ci + 2;
            o = make_float4(sA[c].x, sA[c].y, sA[c].z, sV[c]);
        }
        if (lv.level == 0) {
            const float len = S::ld4_w(static_cast<const C4*>(a.tc), i);
            S::st4(static_cast<C4*>(a.hist_cur), i, make_float4(o.x, o.y, o.z, len));
        }
        if (lv.last)
            st_rgba(a.out, cx, y, make_float4(S::qin(o.x), S::qin(o.y), S::qin(o.z), 1.0f));
        else
            S::st4_sat_w(static_cast<C4*>(lv.col_dst), res_idx(lv.lout, cx, y), o);
    }
}

template <int ST, int R> __global__ void __launch_bounds__(kLvTX* kLvRows, 3) k_full_level_tiled(FullArgs a, LevelGeom g)
{
    __shared__ LevelSmem<R> sm;
    full_level_tile<ST, R>(a, level_args_of(a), g, blockIdx.x, sm);
}

// ------------------------------------------------------------- REF-EXACT ----
// src/svgf_denoise.slang:209-274 on the same tiling; staged coordinates are
// clamped to the image (the reference's clamp-to-edge taps).

template <int ST, int R> __global__ void __launch_bounds__(kLvTX* kLvRows) k_ref_level_tiled(RefArgs a, LevelGeom g)
{
    typedef Stor<ST> S;
    typedef typename S::c4_t C4;
    typedef LevelTile<R> T;
    __shared__ float4 sA[T::N];

    int ra, rb, i0, j0;
    level_block(g, blockIdx.x, T::TX, T::TY, ra, rb, i0, j0);
    const int s = g.s;
    const C4* src = static_cast<const C4*>(a.src);
    const int tid = threadIdx.y * kLvTX + threadIdx.x;
    for (int k = tid; k < T::N; k += kLvTX * kLvRows) {
        const int si = k % T::SW, sj = k / T::SW;
        const int x = min(max(ra + s * (i0 + si - 2), 0), a.w - 1);
        const int y = min(max(rb + s * (j0 + sj - 2), 0), a.h - 1);
        const float4 c = S::ld4(src, res_idx(a.lin, x, y));
        sA[k] = make_float4(c.x, c.y, c.z, lum(c.x, c.y, c.z));
    }
    __syncthreads();

    const int ci = threadIdx.x, cj0 = threadIdx.y * R;
    float lp[R], nk[R], ca[R], ar[R], ag[R], ab[R], aw[R];
    bool valid[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int x = ra + s * (i0 + ci);
        const int y = rb + s * (j0 + cj0 + k);
        valid[k] = x < a.w && y < a.h;
        lp[k] = sA[(cj0 + k + 2) * T::SW + ci + 2].w;
        ca[k] = valid[k] ? S::ld4_w(src, res_idx(a.lin, x, y)) : 0.f;
        const float sigma = fmaxf(__fmul_rn(a.phi, ca[k]), a.var_eps);
        nk[k] = -kLog2e / sigma;
        ar[k] = ag[k] = ab[k] = aw[k] = 0.f;
    }
#pragma unroll
    for (int r = 0; r < R + 4; ++r) {
#pragma unroll
        for (int dx = -2; dx <= 2; ++dx) {
            const float4 A = sA[(cj0 + r) * T::SW + ci + 2 + dx];
#pragma unroll
            for (int k = 0; k < R; ++k) {
                const int dy = r - 2 - k;
                if (dy < -2 || dy > 2) continue;
                const float w = ex2_approx(fmaf(fabsf(A.w - lp[k]), nk[k], log2_b3(dx + 2) + log2_b3(dy + 2)));
                ar[k] = fmaf(A.x, w, ar[k]);
                ag[k] = fmaf(A.y, w, ag[k]);
                ab[k] = fmaf(A.z, w, ab[k]);
                aw[k] += w;
            }
        }
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!valid[k]) continue;
        const int x = ra + s * (i0 + ci);
        const int y = rb + s * (j0 + cj0 + k);
        const int c = (cj0 + k + 2) * T::SW + ci + 2;
        float4 o;
        if (aw[k] > 1e-6f)
            o = make_float4(__fdiv_rn(ar[k], aw[k]), __fdiv_rn(ag[k], aw[k]), __fdiv_rn(ab[k], aw[k]), ca[k]);
        else
            o = make_float4(sA[c].x, sA[c].y, sA[c].z, ca[k]);
        if (a.final_pass) {
            if (ST == ST_FP16) o = make_float4(q16(o.x), q16(o.y), q16(o.z), 1.0f);
            o.w = 1.0f;
            st_rgba(a.out, x, y, o);
        } else {
            S::st4(static_cast<C4*>(a.dst), res_idx(a.lout, x, y), o);
        }
    }
}

__host__ __device__ inline LevelGeom level_geom(int w, int h, int s, int R)
{
    LevelGeom g;
    g.s = s;
    g.sub_w = (w + s - 1) / s;
    g.sub_h = (h + s - 1) / s;
    g.tiles_x = (g.sub_w + kLvTX - 1) / kLvTX;
    g.tiles_y = (g.sub_h + kLvRows * R - 1) / (kLvRows * R);
    return g;
}

__host__ __device__ inline unsigned level_blocks(const LevelGeom& g)
{
    return unsigned(g.s * g.s) * g.tiles_x * g.tiles_y;
}

} // namespace tg
