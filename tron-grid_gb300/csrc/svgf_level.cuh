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

#include <cuda.h>

#include <type_traits>

#include "svgf_device.cuh"

namespace tg {

constexpr int kLvTX = 32;      // outputs per tile row (one warp)
constexpr int kLvRows = 4;     // thread rows per CTA
constexpr float kLog2e = kLog2eF;
// log2 of the B3 taps 1/16, 1/4, 3/8, 1/4, 1/16.
__device__ __forceinline__ constexpr float log2_b3(int i)
{
    return i == 2 ? -1.4150374992788438f : ((i == 1 || i == 3) ? -2.0f : -4.0f);
}

struct LevelGeom {
    int s;        // stride, a power of two
    int lg;       // log2(s)
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

// CTAs per SM the level kernels are compiled for: at R = 2 eight CTAs of 128
// threads (32 warps, 64 registers a thread) hide the tap loop's latencies and
// the tile waits better than four of 256 threads (2% slower per level), two of
// 512 (15% slower) or 256-thread CTAs at 80 registers.
template <int R> struct LevelOcc {
    static constexpr int kCtas = R <= 2 ? 8 : 4;
};

// Staged tile of one level: X0 = (r, g, b, variance), X1 = (unit normal, depth),
// XL = luminance.  A TMA box must land on a 128-byte boundary: X0 and X1 start
// on one (N * 16 bytes is a multiple of 128), and so does the second half of
// X1, where a binary16 level-0 tile lands its guide box (N * 8 bytes in).
template <int R> struct __align__(128) LevelSmem {
    static_assert((LevelTile<R>::N * 8) % 128 == 0,
                  "every TMA destination in a level tile must start on a 128-byte boundary");
    float4 X0[LevelTile<R>::N];
    float4 X1[LevelTile<R>::N];
    float XL[LevelTile<R>::N];
};

// Maps tile `bid` to (residue a, b) and its tile origin in sub-lattice units.
// The residue is the low 2 lg bits of the id (s is a power of two), so only
// the tile row needs a division.
__device__ __forceinline__ void level_block(const LevelGeom& g, int bid, int TX, int TY, int& ra, int& rb, int& i0,
                                            int& j0)
{
    const unsigned u = unsigned(bid);
    const unsigned res = u & ((1u << (2 * g.lg)) - 1u);
    const unsigned tile = u >> (2 * g.lg);
    ra = int(res & unsigned(g.s - 1));
    rb = int(res >> g.lg);
    const unsigned ty = tile / unsigned(g.tiles_x);
    i0 = int(tile - ty * unsigned(g.tiles_x)) * TX;
    j0 = int(ty) * TY;
}

// ------------------------------------------------------------------ FULL ----

// Per-level arguments of an a-trous level (the rest comes from FullArgs).
struct LevelArgs {
    const void* col_src;
    void* col_dst;
    size_t var_off;  // byte offset of the variance plane in col_src / col_dst
    size_t ghalf;    // FP32 records: index of the guide half-plane (16-byte units)
    int level, last;
    ResLayout lin, lout;
};

__host__ __device__ inline LevelArgs level_args_of(const FullArgs& a)
{
    LevelArgs l;
    l.col_src = a.col_src;
    l.col_dst = a.col_dst;
    l.var_off = a.var_off;
    l.ghalf = a.ghalf;
    l.level = a.level;
    l.last = a.last;
    l.lin = a.lin;
    l.lout = a.lout;
    return l;
}

// Per-centre values read from global memory before the tile is staged, so
// that their latency overlaps the staging: the depth gradient, the 3x3
// variance neighbourhood (contiguous in the residue-major layout: the index of
// (qx, qy) separates into a column and a row term).
template <int ST, int R> struct CentrePre {
    float vn9[R][9];
    float2 gr[R];
    bool valid[R];
    float kx_sum;
};

// IN: the CTA's tile, its halo and every centre's 3x3 neighbourhood lie inside
// the image (tile_interior), so no access needs a bounds test.
template <int ST, int R, bool IN>
__device__ __forceinline__ void level_prefetch(const FullArgs& a, const LevelArgs& lv, int s, int ra, int rb, int i0,
                                               int j0, CentrePre<ST, R>& pre)
{
    typedef Stor<ST> S;
    const int lg = lv.lin.lg, m = s - 1, pw = lv.lin.pw, P = lv.lin.pw * lv.lin.ph;
    const int cx = ra + s * (i0 + int(threadIdx.x));
    int cxo[3];
    bool cxv[3];
#pragma unroll
    for (int e = 0; e < 3; ++e) {
        const int qx = cx + e - 1;
        cxv[e] = IN || unsigned(qx) < unsigned(a.w);
        cxo[e] = (qx & m) * P + (qx >> lg);
    }
    pre.kx_sum = IN ? 1.f : (cxv[0] ? 0.25f : 0.f) + (cxv[1] ? 0.5f : 0.f) + (cxv[2] ? 0.25f : 0.f);
    // Every output row y = rb + s jj of this thread has residue rb, so neighbour row y + f - 1 lies in plane row
    // (rb + f - 1) mod s at position jj + floor((rb + f - 1) / s): its offset is a per-thread constant plus jj pw.
    const int j_base = (j0 + int(threadIdx.y) * R) * pw;
    int rowf[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        const int t = rb + f - 1;
        rowf[f] = ((t & m) << lg) * P + (t >> lg) * pw + j_base;
    }
    const Rec::var_t* vp = Rec::var_ptr(lv.col_src, lv.var_off);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int y = rb + s * (j0 + int(threadIdx.y) * R + k);
        pre.valid[k] = IN || (cx < a.w && y < a.h);
        pre.gr[k] = pre.valid[k] ? a.grad[y * a.w + cx] : make_float2(0.f, 0.f);
#pragma unroll
        for (int f = 0; f < 3; ++f) {
            const bool oy = pre.valid[k] && (IN || unsigned(y + f - 1) < unsigned(a.h));
#pragma unroll
            for (int e = 0; e < 3; ++e)
                pre.vn9[k][f * 3 + e] = (oy && cxv[e]) ? Rec::var_at(vp, rowf[f] + k * pw + cxo[e]) : 0.f;
        }
    }
}

// Whether staged tile cell k (sub-lattice coordinates relative to the tile) is
// a pixel of the image; cells outside are zero records with weight 0.
template <int R>
__device__ __forceinline__ bool staged_inside(const FullArgs& a, int s, int ra, int rb, int i0, int j0, int k)
{
    typedef LevelTile<R> T;
    const int sj = k / T::SW, si = k - sj * T::SW;
    const int j = j0 + sj - 2, i = i0 + si - 2;
    return j >= 0 && i >= 0 && rb + s * j < a.h && ra + s * i < a.w;
}

// Whether the tile at (i0, j0) of residue (ra, rb), with its 2-cell halo, lies
// inside the image; then so do its centres and their 3x3 neighbourhoods.
template <int R>
__device__ __forceinline__ bool tile_interior(const FullArgs& a, int s, int ra, int rb, int i0, int j0)
{
    typedef LevelTile<R> T;
    return i0 >= 2 && j0 >= 2 && ra + s * (i0 + T::TX + 1) < a.w && rb + s * (j0 + T::TY + 1) < a.h;
}

// Everything after staging: per-centre set-up, the taps, the output records.
// VAR = false leaves out the variance propagation (sum of w^2 var): the last
// level writes only colour.
template <int ST, int R, bool VAR, bool IN>
__device__ __forceinline__ void level_compute(const FullArgs& a, const LevelArgs& lv, const LevelGeom& g, int ra,
                                              int rb, int i0, int j0, const CentrePre<ST, R>& pre,
                                              const LevelSmem<R>& sm)
{
    typedef Stor<ST> S;
    typedef typename S::c4_t C4;
    typedef LevelTile<R> T;
    const int s = g.s;
    const int ci = threadIdx.x, cj0 = threadIdx.y * R;
    const int cx = ra + s * (i0 + ci);
    // A warp (one strip row of 32 columns) whose outputs all lie outside the
    // sub-lattice has nothing to compute or write.
    bool any_valid = false;
#pragma unroll
    for (int k = 0; k < R; ++k) any_valid |= pre.valid[k];
    if (!__any_sync(0xffffffffu, any_valid)) return;
    float lp[R], kl[R], zp[R], nx[R], ny[R], nz[R], kz[R][13];
    float ar[R], ag[R], ab[R], aw[R], av[R];
    const float zs = a.sigma_z * float(s) * (1.0f / kLog2e);
    const float ez = kEpsZ * (1.0f / kLog2e);
    const float kz_centre = rcp_approx(ez);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int c = (cj0 + k + 2) * T::SW + ci + 2;
        const float4 N = sm.X1[c];
        lp[k] = sm.XL[c];
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
        for (int q = 0; q < 9; ++q)
            sv = fmaf((q / 3 == 1 ? 0.5f : 0.25f) * (q % 3 == 1 ? 0.5f : 0.25f), pre.vn9[k][q], sv);
        // (an inside pixel's weights sum to 1: its blur is sv itself on either path)
        const float kk = ky_sum * pre.kx_sum;
        const float gv = (IN || kk == 1.0f) ? sv : sv * rcp_approx(kk);
        kl[k] = kLog2e * rcp_approx(a.sigma_l * sqrt_approx(fmaxf(gv, 0.f)) + kEpsL);
        const float A_ = zs * pre.gr[k].x, B_ = zs * pre.gr[k].y, B2 = B_ + B_;
        // kz for the 13 offsets (dx, dy) with dy > 0 or (dy == 0 and dx >= 0);
        // the other 12 offsets are their negations and share the value.  The
        // projections dx A + dy B are built from A, B and 2B (exact) with one
        // operation each; offset (0, 0) has the constant 1 / eps.
        kz[k][0] = kz_centre;
#pragma unroll
        for (int q = 1; q < 13; ++q) {
            const int dx = (q < 3) ? q : ((q - 3) % 5) - 2;
            const int dy = (q < 3) ? 0 : 1 + (q - 3) / 5;
            const float by = dy == 1 ? B_ : B2;
            const float v = dy == 0 ? (dx == 1 ? A_ : A_ + A_) : (dx == 0 ? by : fmaf(float(dx), A_, by));
            kz[k][q] = rcp_approx(fabsf(v) + ez);
        }
    }

    // Taps: rows r = 0 .. R+3 of this thread's strip, 5 columns each.
    const float sn = a.sigma_n;
    {
#pragma unroll
        for (int r = 0; r < R + 4; ++r) {
#pragma unroll
            for (int dx = -2; dx <= 2; ++dx) {
                const int q = (cj0 + r) * T::SW + ci + 2 + dx;
                const float4 A = sm.X0[q], N = sm.X1[q];
                const float L = sm.XL[q];
#pragma unroll
                for (int k = 0; k < R; ++k) {
                    const int dy = r - 2 - k;
                    if (dy < -2 || dy > 2) continue;
                    const int ddx = (dy > 0 || (dy == 0 && dx >= 0)) ? dx : -dx;
                    const int ddy = dy >= 0 ? dy : -dy;
                    const int qi = ddy == 0 ? ddx : 3 + (ddy - 1) * 5 + (ddx + 2);
                    const float d = fmaf(nz[k], N.z, fmaf(ny[k], N.y, nx[k] * N.x));
                    float t = fmaf(-fabsf(zp[k] - N.w), kz[k][qi], log2_b3(dx + 2) + log2_b3(dy + 2));
                    t = fmaf(-fabsf(lp[k] - L), kl[k], t);
                    t = fmaf(sn, lg2_approx(fmaxf(d, 0.f)), t);
                    const float w = ex2_approx(t);
                    ar[k] = fmaf(w, A.x, ar[k]);
                    ag[k] = fmaf(w, A.y, ag[k]);
                    ab[k] = fmaf(w, A.z, ab[k]);
                    aw[k] += w;
                    if constexpr (VAR) av[k] = fmaf(w * w, A.w, av[k]);
                }
            }
        }
    }

    // Outputs: the next level's record (colour, variance, the centre's guide),
    // the colour history at level 0, the caller's image at the last level.  At
    // level 0 the history lengths of all outputs are loaded before any store.
    float len[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int y = rb + s * (j0 + cj0 + k);
        len[k] = (lv.level == 0 && pre.valid[k]) ? S::ld4_w(static_cast<const C4*>(a.tc), y * a.w + cx) : 0.f;
    }
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!pre.valid[k]) continue;
        const int y = rb + s * (j0 + cj0 + k);
        const int i = y * a.w + cx;
        const int c = (cj0 + k + 2) * T::SW + ci + 2;
        float4 o;
        if (aw[k] > 0.f) {
            const float inv = rcp_approx(aw[k]);
            o = make_float4(ar[k] * inv, ag[k] * inv, ab[k] * inv, av[k] * (inv * inv));
        } else {
            o = sm.X0[c];
        }
        if (lv.level == 0) S::st4(static_cast<C4*>(a.hist_cur), i, make_float4(o.x, o.y, o.z, len[k]));
        if (lv.last) {
            st_rgba(a.out, cx, y, make_float4(o.x, o.y, o.z, 1.0f));
        } else {
            const size_t oi = res_idx(lv.lout, cx, y);
            Rec::st_rec(static_cast<Rec::rec_t*>(lv.col_dst), oi, o, sm.X1[c], lv.ghalf);
            Rec::st_var(lv.col_dst, lv.var_off, oi, o.w);
        }
    }
}

// Level 0 reads the planes K1 writes instead of records: the staged cell's
// colour from tc, its variance from the variance plane, its guide from
// guide_cur (FP16 storage: decoded from the octahedral code).  Every FULL path
// stages level 0 this way (PL); K1 and K2 write no level-0 records.
template <int ST>
__device__ __forceinline__ void plane_cell(const FullArgs& a, const LevelArgs& lv, size_t j, float4& c, float4& n)
{
    typedef Stor<ST> S;
    const float4 t = S::ld4(static_cast<const typename S::c4_t*>(a.tc), j);
    c = make_float4(t.x, t.y, t.z, Rec::ld_var(lv.col_src, lv.var_off, j));
    if constexpr (ST == ST_FP16) {
        const uint2 u = S::ld_graw(static_cast<const typename S::guide_t*>(a.guide_cur), j);
        const float3 v = oct16_decode_fast(u.x);
        n = make_float4(v.x, v.y, v.z, __uint_as_float(u.y));
    } else {
        n = S::ld_graw(static_cast<const typename S::guide_t*>(a.guide_cur), j);
    }
}

// One tile of one level, staged with plain coalesced loads (the residue-major
// records of a tile row are contiguous; PL: level 0 from the planes).  The
// caller synchronises the CTA before reusing `sm`.
template <int ST, int R, bool VAR, bool PL, bool IN>
__device__ __forceinline__ void level_tile_body(const FullArgs& a, const LevelArgs& lv, const LevelGeom& g, int ra,
                                                int rb, int i0, int j0, LevelSmem<R>& sm)
{
    typedef LevelTile<R> T;
    const int s = g.s;
    CentrePre<ST, R> pre;
    level_prefetch<ST, R, IN>(a, lv, s, ra, rb, i0, j0, pre);
    const Rec::rec_t* src = static_cast<const Rec::rec_t*>(lv.col_src);
    const int pw = lv.lin.pw, P = lv.lin.pw * lv.lin.ph;
    const int plane = ((rb << lv.lin.lg) + ra) * P;
    for (int k = threadIdx.y * kLvTX + threadIdx.x; k < T::N; k += kLvTX * kLvRows) {
        float4 c = make_float4(0.f, 0.f, 0.f, 0.f), n = make_float4(0.f, 0.f, 0.f, 0.f);
        if (IN || staged_inside<R>(a, s, ra, rb, i0, j0, k)) {
            const int sj = k / T::SW, si = k - sj * T::SW;
            const size_t ri = plane + (j0 + sj - 2) * pw + (i0 + si - 2);
            if constexpr (PL)
                plane_cell<ST>(a, lv, ri, c, n);
            else
                Rec::ld_rec(src, ri, c, n, lv.ghalf);
        }
        sm.X0[k] = c;
        sm.X1[k] = n;
        sm.XL[k] = lum(c.x, c.y, c.z);
    }
    __syncthreads();
    level_compute<ST, R, VAR, IN>(a, lv, g, ra, rb, i0, j0, pre, sm);
}

template <int ST, int R, bool VAR = true, bool PL = false>
__device__ __forceinline__ void full_level_tile(const FullArgs& a, const LevelArgs& lv, const LevelGeom& g, int bid,
                                                LevelSmem<R>& sm)
{
    int ra, rb, i0, j0;
    level_block(g, bid, LevelTile<R>::TX, LevelTile<R>::TY, ra, rb, i0, j0);
    if (tile_interior<R>(a, g.s, ra, rb, i0, j0))
        level_tile_body<ST, R, VAR, PL, true>(a, lv, g, ra, rb, i0, j0, sm);
    else
        level_tile_body<ST, R, VAR, PL, false>(a, lv, g, ra, rb, i0, j0, sm);
}

template <int ST, int R, bool VAR, bool PL = false>
__global__ void __launch_bounds__(kLvTX* kLvRows, LevelOcc<R>::kCtas) k_full_level_tiled(FullArgs a, LevelGeom g)
{
    __shared__ LevelSmem<R> sm;
    pdl_begin();
    full_level_tile<ST, R, VAR, PL>(a, level_args_of(a), g, blockIdx.x, sm);
}

// ------------------------------------------------------- TMA-staged level ----
//
// The same level with the halo tile staged by the tensor-memory accelerator:
// one elected thread issues cp.async.bulk.tensor for the tile's box of
// residue-major records (a 4-D map {float, row, plane, half-plane}, so that the
// box of each half lands as one dense float4 array and each tile row is one
// contiguous line of 36 records); level 0 reads two 2-D maps over the tc and guide
// planes instead.  Completion is tracked by an mbarrier transaction count and
// cells outside the plane array arrive zero-filled.  The wait is bounded: a box
// that has not landed after about a second sets a->err, the CTA waits (bounded)
// once more for the copy to retire, and returns.

constexpr long long kTmaWaitCycles = 2000000000LL;

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return uint32_t(__cvta_generic_to_shared(p)); }

__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t phase)
{
    const long long t0 = clock64();
    for (;;) {
        uint32_t ok;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(ok)
                     : "r"(bar), "r"(phase)
                     : "memory");
        if (ok) return true;
        if (clock64() - t0 > kTmaWaitCycles) return false;
    }
}

// Issues the halo box of the tile at (ra, rb, i0, j0) into `sm` (one thread).
// Level 0 with FP16 storage lands its two 8-byte-texel boxes in X1 (tc in the
// first N * 8 bytes, the guide in the next), to be decoded into X0 / X1.
template <int ST, int R, bool PL>
__device__ __forceinline__ void tma_issue(const LevelGeom& g, int ra, int rb, int i0, int j0, LevelSmem<R>& sm,
                                          uint32_t ubar, const CUtensorMap* tm, const CUtensorMap* tm2)
{
    typedef LevelTile<R> T;
    const uint64_t map = reinterpret_cast<uint64_t>(tm);
    if constexpr (PL) {
        const uint64_t map2 = reinterpret_cast<uint64_t>(tm2);
        const uint32_t bytes = 2u * T::N * (ST == ST_FP16 ? 8u : 16u);
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ubar), "r"(bytes) : "memory");
        if constexpr (ST == ST_FP16) {
            // 8-byte texels: x = i0 - 2 texels is even (i0 is a multiple of 32), so the box starts on 16 bytes
            const uint32_t d = smem_u32(sm.X1);
#pragma unroll
            for (int h = 0; h < 2; ++h)
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                    "[%4];" ::"r"(d + h * T::N * 8u),
                    "l"(h == 0 ? map : map2), "r"(i0 - 2), "r"(j0 - 2), "r"(ubar)
                    : "memory");
        } else {
            // x = 4 (i0 - 2) floats: the box starts on a 16-byte boundary
#pragma unroll
            for (int h = 0; h < 2; ++h)
                asm volatile(
                    "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                    "[%4];" ::"r"(smem_u32(h == 0 ? sm.X0 : sm.X1)),
                    "l"(h == 0 ? map : map2), "r"(4 * (i0 - 2)), "r"(j0 - 2), "r"(ubar)
                    : "memory");
        }
    } else {
        const int plane = (rb << g.lg) + ra;
        const uint32_t bytes = 2u * T::N * 16u;
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ubar), "r"(bytes) : "memory");
        // x = 4 (i0 - 2) floats: the box starts on a 16-byte boundary
#pragma unroll
        for (int half = 0; half < 2; ++half)
            asm volatile(
                "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
                "[%6];" ::"r"(smem_u32(half == 0 ? sm.X0 : sm.X1)),
                "l"(map), "r"(4 * (i0 - 2)), "r"(j0 - 2), "r"(plane), "r"(half), "r"(ubar)
                : "memory");
    }
}

// The TMA kernel after its copy is issued: prefetch, bounded wait, fix-up,
// compute.  IN: the tile is interior (tile_interior), so no cell needs a test.
template <int ST, int R, bool VAR, bool PL, bool IN>
__device__ __forceinline__ void tma_tile_body(const FullArgs& a, const LevelArgs& lv, const LevelGeom& g, int ra, int rb,
                                              int i0, int j0, int tid, uint32_t ubar, LevelSmem<R>& sm)
{
    typedef LevelTile<R> T;
    constexpr int kThreads = kLvTX * kLvRows;
    constexpr int kCells = (T::N + kThreads - 1) / kThreads;
    const int s = g.s;
    CentrePre<ST, R> pre;
    level_prefetch<ST, R, IN>(a, lv, s, ra, rb, i0, j0, pre);
    // PL: the staged cells' variances (the plane is row-major at level 0)
    float cv[PL ? kCells : 1];
    if constexpr (PL) {
#pragma unroll
        for (int e = 0; e < kCells; ++e) {
            const int k = tid + e * kThreads;
            cv[e] = 0.f;
            if (k < T::N && (IN || staged_inside<R>(a, s, ra, rb, i0, j0, k))) {
                const int sj = k / T::SW, si = k - sj * T::SW;
                cv[e] = Rec::ld_var(lv.col_src, lv.var_off, size_t(j0 + sj - 2) * a.w + (i0 + si - 2));
            }
        }
    }
    const bool landed = mbar_wait_bounded(ubar, 0);
    if (__syncthreads_or(!landed)) {
        if (tid == 0) {
            if (a.err) atomicExch(a.err, 1);
            mbar_wait_bounded(ubar, 0);  // give the copy a second bounded chance to retire
        }
        return;
    }
    if constexpr (PL && ST == ST_FP16) {
        // the raw texels of this thread's cells, read before any thread overwrites X1 with decoded guides
        const uint2* rc = reinterpret_cast<const uint2*>(sm.X1);
        const uint2* rg = rc + T::N;
        uint2 tc[kCells], gd[kCells];
#pragma unroll
        for (int e = 0; e < kCells; ++e) {
            const int k = tid + e * kThreads;
            tc[e] = k < T::N ? rc[k] : make_uint2(0u, 0u);
            gd[e] = k < T::N ? rg[k] : make_uint2(0u, 0u);
        }
        __syncthreads();
#pragma unroll
        for (int e = 0; e < kCells; ++e) {
            const int k = tid + e * kThreads;
            if (k >= T::N) break;
            const bool in = IN || staged_inside<R>(a, s, ra, rb, i0, j0, k);
            const float4 t = unpack_h4(tc[e]);
            const float3 v = oct16_decode_fast(gd[e].x);
            float4 c = make_float4(t.x, t.y, t.z, cv[e]);
            float4 n = make_float4(v.x, v.y, v.z, __uint_as_float(gd[e].y));
            if (!in) {
                c = make_float4(0.f, 0.f, 0.f, 0.f);
                n = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            sm.X0[k] = c;
            sm.X1[k] = n;
            sm.XL[k] = lum(c.x, c.y, c.z);
        }
    } else {
        // zero the cells outside the image, compute luminance
#pragma unroll
        for (int e = 0; e < kCells; ++e) {
            const int k = tid + e * kThreads;
            if (k >= T::N) break;
            const bool in = IN || staged_inside<R>(a, s, ra, rb, i0, j0, k);
            float4 c = sm.X0[k];
            if constexpr (PL) c.w = cv[e];
            if (!in) {
                c = make_float4(0.f, 0.f, 0.f, 0.f);
                sm.X1[k] = make_float4(0.f, 0.f, 0.f, 0.f);
            }
            if (PL || !in) sm.X0[k] = c;
            sm.XL[k] = lum(c.x, c.y, c.z);
        }
    }
    __syncthreads();
    level_compute<ST, R, VAR, IN>(a, lv, g, ra, rb, i0, j0, pre, sm);
}

// One level with its tile staged by TMA.  VAR = false at the last level (colour
// only).  PL (level 0): the box comes from two row-major images instead of the
// records, tc through `tm` and guide_cur through `tm2`, and each staged cell's
// variance comes from the variance plane, loaded before the wait.  Other levels
// read `tm` only.
// One tile `bid` of a level staged by TMA through maps `tm` / `tm2` (kernel
// parameters).
template <int ST, int R, bool VAR, bool PL>
__device__ __forceinline__ void full_level_tile_tma(const FullArgs& a, const LevelArgs& lv, const LevelGeom& g, int bid,
                                                    LevelSmem<R>& sm, uint64_t& bar, const CUtensorMap* tm,
                                                    const CUtensorMap* tm2)
{
    typedef LevelTile<R> T;
    int ra, rb, i0, j0;
    level_block(g, bid, T::TX, T::TY, ra, rb, i0, j0);
    const int tid = threadIdx.y * kLvTX + threadIdx.x;
    const uint32_t ubar = smem_u32(&bar);
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0) tma_issue<ST, R, PL>(g, ra, rb, i0, j0, sm, ubar, tm, tm2);
    if (tile_interior<R>(a, g.s, ra, rb, i0, j0))
        tma_tile_body<ST, R, VAR, PL, true>(a, lv, g, ra, rb, i0, j0, tid, ubar, sm);
    else
        tma_tile_body<ST, R, VAR, PL, false>(a, lv, g, ra, rb, i0, j0, tid, ubar, sm);
}

template <int ST, int R, bool VAR, bool PL>
__global__ void __launch_bounds__(kLvTX* kLvRows, LevelOcc<R>::kCtas)
    k_full_level_tma(FullArgs a, LevelArgs lv, LevelGeom g, const __grid_constant__ CUtensorMap tm,
                     const __grid_constant__ CUtensorMap tm2)
{
    __shared__ LevelSmem<R> sm;
    __shared__ __align__(8) uint64_t bar;
    pdl_begin();
    full_level_tile_tma<ST, R, VAR, PL>(a, lv, g, blockIdx.x, sm, bar, &tm, &tm2);
}

// ------------------------------------------------------------- REF-EXACT ----
// src/svgf_denoise.slang:176-274 on the same tiling; staged coordinates are
// clamped to the image (the reference's clamp-to-edge taps).  The init pass
// (src/svgf_denoise.slang:176-191) is pointwise, so it runs inside the first
// a-trous pass: that kernel stages the caller's radiance as the init pass would
// have stored it in wavelet_a (rounded to the storage format) and each centre
// computes its own moments and sqrt-variance, so wavelet_a is never written
// and read back.  Dispatches replaced: src/main.cpp:929-944 (one init and
// three wavelet passes become three kernels).

// Whether the tile at (i0, j0) of residue (ra, rb), with its 2-cell halo, lies
// inside a w x h image: then no staged coordinate needs clamping.
template <int R> __device__ __forceinline__ bool ref_tile_interior(int w, int h, int s, int ra, int rb, int i0, int j0)
{
    typedef LevelTile<R> T;
    return i0 >= 2 && j0 >= 2 && ra + s * (i0 + T::TX + 1) < w && rb + s * (j0 + T::TY + 1) < h;
}

// The 25 taps of this thread's R centres over the staged tile sA (r, g, b,
// luminance) and the outputs.  ca: each centre's alpha (sqrt-variance as
// stored), valid: the centre is a pixel of the image.  (Accumulating the sums
// in paired FMAs, fma.rn.f32x2, was measured 1% slower: the broadcast of each
// weight to both halves costs a move.)
template <int ST, int R>
__device__ __forceinline__ void ref_taps_out(const RefArgs& a, int s, int ra, int rb, int i0, int j0, const float* ca,
                                             const bool* valid, const float4* sA)
{
    typedef Stor<ST> S;
    typedef typename S::c4_t C4;
    typedef LevelTile<R> T;
    const int ci = threadIdx.x, cj0 = threadIdx.y * R;
    float lp[R], nk[R];
    float2 rg[R], bw[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        lp[k] = sA[(cj0 + k + 2) * T::SW + ci + 2].w;
        const float sigma = fmaxf(__fmul_rn(a.phi, ca[k]), a.var_eps);
        nk[k] = -kLog2e * rcp_approx(sigma);
        rg[k] = bw[k] = make_float2(0.f, 0.f);
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
                rg[k].x = fmaf(A.x, w, rg[k].x);
                rg[k].y = fmaf(A.y, w, rg[k].y);
                bw[k].x = fmaf(A.z, w, bw[k].x);
                bw[k].y += w;
            }
        }
    }
    const int x = ra + s * (i0 + ci);
#pragma unroll
    for (int k = 0; k < R; ++k) {
        if (!valid[k]) continue;
        const int y = rb + s * (j0 + cj0 + k);
        float4 o;
        if (bw[k].y > 1e-6f) {
            const float inv = rcp_approx(bw[k].y);
            o = make_float4(rg[k].x * inv, rg[k].y * inv, bw[k].x * inv, ca[k]);
        } else {
            const float4 c = sA[(cj0 + k + 2) * T::SW + ci + 2];
            o = make_float4(c.x, c.y, c.z, ca[k]);
        }
        if (a.final_pass) {
            // fp16 images round to binary16 (an RGBA16F output's store does the same rounding itself)
            if (ST == ST_FP16 && a.out.fmt != TG_FMT_RGBA16F) o = make_float4(q16(o.x), q16(o.y), q16(o.z), 1.0f);
            o.w = 1.0f;
            st_rgba(a.out, x, y, o);
        } else {
            S::st4(static_cast<C4*>(a.dst), res_idx(a.lout, x, y), o);
        }
    }
}

// TMA staging of a REF_EXACT tile (interior tiles only: no clamping needed).
// One thread issues the halo box of 8- or 16-byte texels into `land`; the
// others wait (bounded), then each cell is converted into sA as
// (r, g, b, luminance) of the colour rounded to the storage format.  Returns
// false (every thread) if the box did not land in time, after recording the
// timeout in a.err.
template <int ST, int R>
__device__ __forceinline__ bool ref_tma_land(const RefArgs& a, uint32_t ubar, bool f16_texels, const float4* land,
                                             float4* sA)
{
    typedef LevelTile<R> T;
    const int tid = threadIdx.y * kLvTX + threadIdx.x;
    const bool landed = mbar_wait_bounded(ubar, 0);
    if (__syncthreads_or(!landed)) {
        if (tid == 0) {
            if (a.err) atomicExch(a.err, 1);
            mbar_wait_bounded(ubar, 0);  // give the copy a second bounded chance to retire
        }
        return false;
    }
    constexpr int kThreads = kLvTX * kLvRows;
#pragma unroll
    for (int e = 0; e < (T::N + kThreads - 1) / kThreads; ++e) {
        const int k = tid + e * kThreads;
        if (k >= T::N) break;
        // binary16 texels are already in every storage format; fp32 texels are rounded to it
        const float4 c = f16_texels ? unpack_h4(reinterpret_cast<const uint2*>(land)[k]) : Stor<ST>::rt4(land[k]);
        sA[k] = make_float4(c.x, c.y, c.z, lum(c.x, c.y, c.z));
    }
    return true;
}

// Issues the box (one thread): `dims` 2 (x, row) or 3 (x, row, plane); x in
// elements of the map (texels for 8-byte texels, floats for 16-byte ones).
__device__ __forceinline__ void ref_tma_issue(const CUtensorMap* tm, uint32_t ubar, void* land, uint32_t bytes, int dims,
                                              int x, int y, int z)
{
    const uint64_t map = reinterpret_cast<uint64_t>(tm);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(ubar), "r"(bytes) : "memory");
    if (dims == 2)
        asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], "
                     "[%4];" ::"r"(smem_u32(land)),
                     "l"(map), "r"(x), "r"(y), "r"(ubar)
                     : "memory");
    else
        asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
                     "[%5];" ::"r"(smem_u32(land)),
                     "l"(map), "r"(x), "r"(y), "r"(z), "r"(ubar)
                     : "memory");
}

__device__ __forceinline__ void mbar_init_cta(uint32_t ubar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(ubar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Init and the first wavelet pass (stride 1) in one kernel: reads the caller's
// radiance and moments_prev, writes moments_curr and the pass's output (the
// next pass's input, or the caller's image when it is the only pass).  TM: the
// tile (interior) is staged by TMA from the caller's radiance through `tm`.
template <int ST, int R, bool IN, bool TM>
__device__ __forceinline__ void ref_first_tile(const RefArgs& a, int i0, int j0, float4* sA, const CUtensorMap* tm,
                                               float4* land, uint32_t ubar)
{
    typedef Stor<ST> S;
    typedef typename S::mom_t M;
    typedef LevelTile<R> T;
    const int tid = threadIdx.y * kLvTX + threadIdx.x;
    const int ci = threadIdx.x, cj0 = threadIdx.y * R;
    float ca[R];
    bool valid[R];
    float4 craw[R];
    float2 mp[R];
    // each centre's radiance and previous moments, loaded before the staging so that their latency overlaps it
    // (a TMA-staged tile takes the radiance from the landed texels instead)
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int x = i0 + ci, y = j0 + cj0 + k;
        valid[k] = IN || (x < a.w && y < a.h);
        craw[k] = (!TM && valid[k]) ? ld_rgba(a.raw, x, y) : make_float4(0.f, 0.f, 0.f, 0.f);
        mp[k] = valid[k] ? S::ldm(static_cast<const M*>(a.mom_prev), size_t(y) * a.w + x) : make_float2(0.f, 0.f);
    }
    if constexpr (TM) {
        // wavelet_a's colour as the init pass stores it: the radiance in the storage format
        const bool h = a.raw.fmt == TG_FMT_RGBA16F;
        if (!ref_tma_land<ST, R>(a, ubar, h, land, sA)) return;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int c = (cj0 + k + 2) * T::SW + ci + 2;
            craw[k] = h ? unpack_h4(reinterpret_cast<const uint2*>(land)[c]) : land[c];
        }
    } else {
        for (int k = tid; k < T::N; k += kLvTX * kLvRows) {
            const int sj = k / T::SW, si = k - sj * T::SW;
            int x = i0 + si - 2, y = j0 + sj - 2;
            if (!IN) {
                x = min(max(x, 0), a.w - 1);
                y = min(max(y, 0), a.h - 1);
            }
            // wavelet_a's colour as the init pass stores it: the radiance in the storage format
            const float4 c = S::rt4(ld_rgba(a.raw, x, y));
            sA[k] = make_float4(c.x, c.y, c.z, lum(c.x, c.y, c.z));
        }
    }
    // src/svgf_denoise.slang:177-190: moments EMA and sqrt-variance (the alpha wavelet_a would carry)
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const float l = lum(craw[k].x, craw[k].y, craw[k].z);
        const float m1 = __fadd_rn(mp[k].x, __fmul_rn(__fsub_rn(l, mp[k].x), a.alpha_m));
        const float m2 = __fadd_rn(mp[k].y, __fmul_rn(__fsub_rn(__fmul_rn(l, l), mp[k].y), a.alpha_m));
        const float var = fmaxf(__fsub_rn(m2, __fmul_rn(m1, m1)), 0.0f);
        const float sd = __fsqrt_rn(__fadd_rn(var, a.var_eps));
        ca[k] = ST == ST_FP16 ? q16(sd) : sd;
        if (valid[k]) {
            const size_t i = size_t(j0 + cj0 + k) * a.w + (i0 + ci);
            if (ST == ST_FP16)
                // rg16f store: plain round-to-nearest (overflows to inf as the reference's image store does)
                reinterpret_cast<uint32_t*>(a.mom_curr)[i] = pack_h2(m1, m2);
            else
                S::stm(static_cast<M*>(a.mom_curr), i, make_float2(m1, m2));
        }
    }
    __syncthreads();
    ref_taps_out<ST, R>(a, 1, 0, 0, i0, j0, ca, valid, sA);
}

// CTAs per SM the REF_EXACT kernels are compiled for: 12 of 128 threads (40
// registers a thread, 48 warps).  48 warps measured 14% faster per 4K frame
// than the 40 that 42 registers allowed; 12 CTAs of 128 threads ran as fast as
// 6 of 256; 3 rows per thread was slower.
#ifndef TG_REF_CTAS
#define TG_REF_CTAS 12
#endif
#ifndef TG_REF_FIRST_CTAS
#define TG_REF_FIRST_CTAS TG_REF_CTAS
#endif

// use_tma: interior tiles are staged through `tm`, a 2-D map over the caller's
// radiance ({8-byte texel, row} for RGBA16F, {float, row} for RGBA32F);
// border tiles (clamped taps) and use_tma == 0 stage with plain loads.
template <int ST, int R>
__global__ void __launch_bounds__(kLvTX* kLvRows, TG_REF_FIRST_CTAS)
    k_ref_first(RefArgs a, LevelGeom g, const __grid_constant__ CUtensorMap tm, int use_tma)
{
    typedef LevelTile<R> T;
    __shared__ float4 sA[T::N];
    __shared__ __align__(128) float4 land[T::N];
    __shared__ __align__(8) uint64_t bar;
    pdl_begin();
    const int i0 = int(blockIdx.x % unsigned(g.tiles_x)) * T::TX;
    const int j0 = int(blockIdx.x / unsigned(g.tiles_x)) * T::TY;
    const bool in = ref_tile_interior<R>(a.w, a.h, 1, 0, 0, i0, j0);
    if (in && use_tma) {
        const uint32_t ubar = smem_u32(&bar);
        if (threadIdx.x == 0 && threadIdx.y == 0) mbar_init_cta(ubar);
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            const bool h = a.raw.fmt == TG_FMT_RGBA16F;
            // x = i0 - 2 texels: even, so the box starts on a 16-byte boundary for 8-byte texels
            ref_tma_issue(&tm, ubar, land, T::N * (h ? 8u : 16u), 2, h ? i0 - 2 : 4 * (i0 - 2), j0 - 2, 0);
        }
        ref_first_tile<ST, R, true, true>(a, i0, j0, sA, &tm, land, ubar);
    } else if (in) {
        ref_first_tile<ST, R, true, false>(a, i0, j0, sA, &tm, land, 0);
    } else {
        ref_first_tile<ST, R, false, false>(a, i0, j0, sA, &tm, land, 0);
    }
}

// One wavelet pass at stride s >= 2 over residue-major scratch.  TM: the tile
// (interior) is staged by TMA (the box already issued into `land`).
template <int ST, int R, bool IN, bool TM>
__device__ __forceinline__ void ref_level_tile(const RefArgs& a, int s, int ra, int rb, int i0, int j0, float4* sA,
                                               const float4* land, uint32_t ubar)
{
    typedef Stor<ST> S;
    typedef typename S::c4_t C4;
    typedef LevelTile<R> T;
    const C4* src = static_cast<const C4*>(a.src);
    const int tid = threadIdx.y * kLvTX + threadIdx.x;
    const int ci = threadIdx.x, cj0 = threadIdx.y * R;
    const int pw = a.lin.pw;
    // each centre's alpha (the sigma of its luminance weight), loaded before the staging so that its latency
    // overlaps it
    // (a TMA-staged tile takes them from the landed texels instead)
    float ca[R];
    bool valid[R];
#pragma unroll
    for (int k = 0; k < R; ++k) {
        const int x = ra + s * (i0 + ci);
        const int y = rb + s * (j0 + cj0 + k);
        valid[k] = IN || (x < a.w && y < a.h);
        ca[k] = (!TM && valid[k]) ? S::ld4_w(src, res_idx(a.lin, x, y)) : 0.f;
    }
    if constexpr (TM) {
        if (!ref_tma_land<ST, R>(a, ubar, ST == ST_FP16, land, sA)) return;
#pragma unroll
        for (int k = 0; k < R; ++k) {
            const int c = (cj0 + k + 2) * T::SW + ci + 2;
            ca[k] = ST == ST_FP16 ? unpack_h2(reinterpret_cast<const uint2*>(land)[c].y).y : land[c].w;
        }
    } else if (IN) {
        // the tile's plane rows are contiguous runs of the residue-major layout
        const int base = ((rb << a.lin.lg) + ra) * a.lin.ph * pw + (j0 - 2) * pw + (i0 - 2);
        for (int k = tid; k < T::N; k += kLvTX * kLvRows) {
            const int sj = k / T::SW, si = k - sj * T::SW;
            const float4 c = S::ld4(src, base + sj * pw + si);
            sA[k] = make_float4(c.x, c.y, c.z, lum(c.x, c.y, c.z));
        }
    } else {
        for (int k = tid; k < T::N; k += kLvTX * kLvRows) {
            const int sj = k / T::SW, si = k - sj * T::SW;
            const int x = min(max(ra + s * (i0 + si - 2), 0), a.w - 1);
            const int y = min(max(rb + s * (j0 + sj - 2), 0), a.h - 1);
            const float4 c = S::ld4(src, res_idx(a.lin, x, y));
            sA[k] = make_float4(c.x, c.y, c.z, lum(c.x, c.y, c.z));
        }
    }
    __syncthreads();
    ref_taps_out<ST, R>(a, s, ra, rb, i0, j0, ca, valid, sA);
}

// use_tma: interior tiles are staged through `tm`, a 3-D map over the input's
// residue planes ({8-byte texel, row, plane} for fp16 images, {float, row,
// plane} for fp32 ones); border tiles and use_tma == 0 stage with plain loads.
template <int ST, int R>
__global__ void __launch_bounds__(kLvTX* kLvRows, TG_REF_CTAS)
    k_ref_level(RefArgs a, LevelGeom g, const __grid_constant__ CUtensorMap tm, int use_tma)
{
    typedef LevelTile<R> T;
    __shared__ float4 sA[T::N];
    __shared__ __align__(128) float4 land[T::N];
    __shared__ __align__(8) uint64_t bar;
    pdl_begin();
    int ra, rb, i0, j0;
    level_block(g, blockIdx.x, T::TX, T::TY, ra, rb, i0, j0);
    const bool in = ref_tile_interior<R>(a.w, a.h, g.s, ra, rb, i0, j0);
    if (in && use_tma) {
        const uint32_t ubar = smem_u32(&bar);
        if (threadIdx.x == 0 && threadIdx.y == 0) mbar_init_cta(ubar);
        __syncthreads();
        if (threadIdx.x == 0 && threadIdx.y == 0) {
            constexpr bool h = ST == ST_FP16;
            // x = i0 - 2 texels: even, so the box starts on a 16-byte boundary for 8-byte texels
            ref_tma_issue(&tm, ubar, land, T::N * (h ? 8u : 16u), 3, h ? i0 - 2 : 4 * (i0 - 2), j0 - 2,
                          (rb << g.lg) + ra);
        }
        ref_level_tile<ST, R, true, true>(a, g.s, ra, rb, i0, j0, sA, land, ubar);
    } else if (in) {
        ref_level_tile<ST, R, true, false>(a, g.s, ra, rb, i0, j0, sA, land, 0);
    } else {
        ref_level_tile<ST, R, false, false>(a, g.s, ra, rb, i0, j0, sA, land, 0);
    }
}

__host__ __device__ inline LevelGeom level_geom(int w, int h, int s, int R)
{
    LevelGeom g;
    g.s = s;
    g.lg = 0;
    while ((1 << g.lg) < s) ++g.lg;
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

// Tensor maps for TMA staging of the REF_EXACT chain (null: plain loads).
// first: over the caller's radiance; level[L]: over pass L's input planes.
struct RefMaps {
    const CUtensorMap* first = nullptr;
    const CUtensorMap* level[10] = {};
};

// Enqueues one REF_EXACT frame on `stream`: the init fused into the first pass
// (stride 1, output to `wb`), then passes at strides 2, 4, ... alternating
// wb -> wa -> wb; the last pass writes the caller's image.  `a` carries the
// images and constants.  hook(first, body) runs each launch body (first: the
// fused pass), so that a caller can bracket it with events.
template <int R, class Hook>
void enqueue_ref_chain(RefArgs a, void* wa, void* wb, int levels, bool f16, cudaStream_t stream, const RefMaps& maps,
                       Hook hook)
{
    const dim3 blk(kLvTX, kLvRows);
    const CUtensorMap none{};
    a.src = nullptr;
    a.dst = wb;
    a.stride = 1;
    a.final_pass = levels == 1;
    a.lin = res_layout(a.w, a.h, 0);
    a.lout = res_layout(a.w, a.h, 1);
    const LevelGeom g0 = level_geom(a.w, a.h, 1, R);
    hook(true, [&] {
        const CUtensorMap& m = maps.first ? *maps.first : none;
        const int t = maps.first != nullptr;
        launch_chain(f16 ? k_ref_first<ST_FP16, R> : k_ref_first<ST_FP32, R>, dim3(level_blocks(g0)), blk, stream, a, g0,
                     m, t);
    });
    void* src = wb;
    void* oth = wa;
    for (int lv = 1; lv < levels; ++lv) {
        a.src = src;
        a.dst = oth;
        a.stride = 1 << lv;
        a.final_pass = lv == levels - 1;
        a.lin = res_layout(a.w, a.h, lv);
        a.lout = res_layout(a.w, a.h, lv + 1);
        const LevelGeom g = level_geom(a.w, a.h, a.stride, R);
        hook(false, [&] {
            const CUtensorMap& m = maps.level[lv] ? *maps.level[lv] : none;
            const int t = maps.level[lv] != nullptr;
            launch_chain(f16 ? k_ref_level<ST_FP16, R> : k_ref_level<ST_FP32, R>, dim3(level_blocks(g)), blk, stream, a,
                         g, m, t);
        });
        void* t = src;
        src = oth;
        oth = t;
    }
}

} // namespace tg
