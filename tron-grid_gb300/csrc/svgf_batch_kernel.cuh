// The persistent multi-stream step kernel, its work table and its bounded
// grid barrier: shared by the batched form (svgf_batch.cu) and the serving
// loop (svgf_serve.cu).
//
// Work-list.  A step has 2 + L stages (temporal, variance, L a-trous levels).
// Stage k of stream j is cut into tiles (32 x 4 pixels for the pixel stages, a
// residue-class tile for the levels, exactly as in the single-stream kernels);
// the work table holds, per stage, the exclusive prefix sum of the tile counts
// over the active streams.  Every CTA of the persistent grid takes items
// blockIdx.x, blockIdx.x + gridDim.x, ... of the stage, finds its stream by a
// binary search in the prefix sums, runs the tile, and meets the other CTAs at
// a grid barrier before the next stage.  The launch is cooperative, so all
// CTAs are co-resident and the barrier cannot deadlock; its spin is still
// bounded, after which it records an error and every CTA returns.
#pragma once

#include "svgf_kernels.cuh"
#include "svgf_level.cuh"

namespace tg {

struct BarrierState {
    unsigned count;
    unsigned gen;
    int err;
    int pad;
};

struct BatchHeader {
    int n;        // active streams
    int levels;
    int n_stages; // 2 + levels
    int pad;
};

struct BatchEntry {
    FullArgs fa;  // stream-level arguments (col_dst = colA for the variance stage)
    void* colA;
    void* colB;
    // TMA staging of the stream's levels in the batch's stage kernels (k_ms_level_tma): its slot in the
    // launch's StageMaps (-1: plain loads), bit L of tma_mask set when level L's maps were encoded, guide_k
    // the parity of this step's guide
    int tma_slot;
    unsigned tma_mask;
    int guide_k;
    int pad;
};

// Tensor maps of one a-trous stage for the streams of a batch, passed as a
// kernel parameter (so that, like the single-stream kernels' maps, they need no
// proxy fence and cannot go stale): level 0 holds each stream's tc, guide[0]
// and guide[1] plane maps at 3 slot .. 3 slot + 2, level L >= 1 its records' map
// at slot.  The slot is the stream's id, so the maps do not depend on which
// streams a step runs, and a captured graph stays valid for any subset.
constexpr int kTmaStreams = 80;
struct StageMaps {
    CUtensorMap m[3 * kTmaStreams];
};
static_assert(sizeof(StageMaps) + 64 <= 32764, "stage maps must fit the kernel parameter space");

constexpr int kStages = 2 + 10;
constexpr long long kBarrierSpinCycles = 2000000000LL;  // default limit, ~1 s at 2 GHz

__host__ __device__ inline size_t table_prefix_offset() { return sizeof(BatchHeader); }
__host__ __device__ inline size_t table_entries_offset(int cap)
{
    const size_t p = sizeof(BatchHeader) + size_t(kStages) * (cap + 1) * sizeof(int);
    return (p + 15) / 16 * 16;
}
inline size_t table_bytes(int cap) { return table_entries_offset(cap) + size_t(cap) * sizeof(BatchEntry); }

// Grid-wide barrier with a bounded wait.  Returns false when this or any other
// CTA gave up; the caller then returns.
__device__ __forceinline__ bool grid_barrier(BarrierState* b, unsigned nblocks, long long spin_cycles)
{
    __shared__ int ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        ok = 1;
        volatile unsigned* vgen = &b->gen;
        volatile int* verr = &b->err;
        const unsigned g0 = *vgen;
        __threadfence();
        if (atomicAdd(&b->count, 1u) == nblocks - 1) {
            atomicExch(&b->count, 0u);
            __threadfence();
            atomicAdd(&b->gen, 1u);
        } else {
            const long long t0 = clock64();
            while (*vgen == g0) {
                if (*verr || clock64() - t0 > spin_cycles) {
                    atomicExch(&b->err, 1);
                    ok = 0;
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
    return ok != 0;
}

// Stream of work item `item` in a stage's prefix sums pf[0..n].
__device__ __forceinline__ int find_stream(const int* pf, int n, int item)
{
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (pf[mid] <= item)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// The persistent kernel runs the pixel stages on its level-shaped CTAs, and
// K2 stages its tile in the level tile's shared memory.
static_assert(kLvTX == kBlockX && kLvRows == kBlockY, "pixel and level CTAs must have the same shape");
static_assert(sizeof(VarTile) <= sizeof(LevelSmem<1>), "K2 tile must fit the level tile");

template <int ST, int R>
__global__ void __launch_bounds__(kLvTX* kLvRows, 6) k_batch_step(const char* __restrict__ table, int cap,
                                                                   BarrierState* bar, unsigned expect_blocks,
                                                                   long long spin_cycles)
{
    __shared__ LevelSmem<R> sm;
    __shared__ VarList vl;
    const BatchHeader hd = *reinterpret_cast<const BatchHeader*>(table);
    const int* prefix = reinterpret_cast<const int*>(table + table_prefix_offset());
    const BatchEntry* ent = reinterpret_cast<const BatchEntry*>(table + table_entries_offset(cap));
    for (int stage = 0; stage < hd.n_stages; ++stage) {
        const int* pf = prefix + stage * (cap + 1);
        const int items = pf[hd.n];
        if (stage == 1) {
            // K2: only the flagged pixel blocks, compacted a chunk at a time
            for (int base = blockIdx.x; base < items; base += gridDim.x * kVarPerCta) {
                variance_compact(
                    base, int(gridDim.x), items,
                    [&](int it) {
                        const int j = find_stream(pf, hd.n, it);
                        return __ldcg(ent[j].fa.fb_flags + (it - pf[j])) != 0;
                    },
                    vl);
                const int n = vl.n;
                for (int e = 0; e < n; ++e) {
                    const int it = vl.item[e];
                    const int j = find_stream(pf, hd.n, it), local = it - pf[j];
                    const FullArgs& a = ent[j].fa;
                    const int tx = (a.w + kBlockX - 1) / kBlockX;
                    full_variance_tile<ST>(a, (local % tx) * kBlockX + threadIdx.x, (local / tx) * kBlockY + threadIdx.y,
                                           *reinterpret_cast<VarTile*>(&sm));
                }
                __syncthreads();  // vl is refilled by the next chunk
            }
            if (stage + 1 < hd.n_stages && !grid_barrier(bar, expect_blocks, spin_cycles)) return;
            continue;
        }
        for (int item = blockIdx.x; item < items; item += gridDim.x) {
            const int lo = find_stream(pf, hd.n, item);
            const int local = item - pf[lo];
            const BatchEntry& e = ent[lo];
            const FullArgs& a = e.fa;
            if (stage == 0) {
                const int tx = (a.w + kBlockX - 1) / kBlockX;
                full_temporal_block<ST>(a, local, (local % tx) * kBlockX + threadIdx.x,
                                        (local / tx) * kBlockY + threadIdx.y);
            } else {
                const int L = stage - 2;
                LevelArgs lv;
                lv.col_src = (L & 1) ? e.colB : e.colA;
                lv.col_dst = (L & 1) ? e.colA : e.colB;
                lv.var_off = a.var_off;
                lv.ghalf = a.ghalf;
                lv.level = L;
                lv.last = L == hd.levels - 1;
                lv.lin = res_layout(a.w, a.h, L);
                lv.lout = res_layout(a.w, a.h, L + 1);
                const LevelGeom g = level_geom(a.w, a.h, 1 << L, R);
                // level 0 stages from the planes; the last level writes only colour
                if (L == 0)
                    full_level_tile<ST, R, true, true>(a, lv, g, local, sm);
                else if (lv.last)
                    full_level_tile<ST, R, false, false>(a, lv, g, local, sm);
                else
                    full_level_tile<ST, R, true, false>(a, lv, g, local, sm);
                __syncthreads();
            }
        }
        if (stage + 1 < hd.n_stages && !grid_barrier(bar, expect_blocks, spin_cycles)) return;
    }
}

// ------------------------------------------------------------------------
// Stage kernels over the same work table: one launch per stage for all the
// active streams (the work-list of one stage is the blocks of one grid).  The
// hardware schedules the blocks; each kernel keeps its own occupancy.


// STAGE 0 (K1): one CTA per pixel block.  STAGE 1 (K2): one chunk of
// kVarPerCta blocks per CTA (gridDim.x = variance_grid(items, SMs)).
template <int ST, int STAGE>
__global__ void __launch_bounds__(kBlockX* kBlockY) k_ms_pixel(const char* __restrict__ table, int cap)
{
    pdl_begin();
    const BatchHeader* hd = reinterpret_cast<const BatchHeader*>(table);
    const int* pf = reinterpret_cast<const int*>(table + table_prefix_offset()) + STAGE * (cap + 1);
    const BatchEntry* ent = reinterpret_cast<const BatchEntry*>(table + table_entries_offset(cap));
    const int n_str = hd->n, items = pf[n_str];
    if constexpr (STAGE == 0) {
        const int item = blockIdx.x;
        if (item >= items) return;
        const int j = find_stream(pf, n_str, item);
        const int local = item - pf[j];
        const FullArgs& a = ent[j].fa;
        const int tx = (a.w + kBlockX - 1) / kBlockX;
        full_temporal_block<ST>(a, local, (local % tx) * kBlockX + threadIdx.x, (local / tx) * kBlockY + threadIdx.y);
    } else {
        __shared__ VarTile vt;
        __shared__ VarList vl;
        variance_compact(
            int(blockIdx.x), int(gridDim.x), items,
            [&](int it) {
                const int j = find_stream(pf, n_str, it);
                return __ldcg(ent[j].fa.fb_flags + (it - pf[j])) != 0;
            },
            vl);
        const int n = vl.n;
        for (int e = 0; e < n; ++e) {
            const int it = vl.item[e];
            const int j = find_stream(pf, n_str, it), local = it - pf[j];
            const FullArgs& a = ent[j].fa;
            const int tx = (a.w + kBlockX - 1) / kBlockX;
            full_variance_tile<ST>(a, (local % tx) * kBlockX + threadIdx.x, (local / tx) * kBlockY + threadIdx.y, vt);
        }
    }
}

// VAR = false at the last level (colour only); PL at level 0 (staged from the planes).
template <int ST, int R, bool VAR, bool PL>
__global__ void __launch_bounds__(kLvTX* kLvRows, LevelOcc<R>::kCtas) k_ms_level(const char* __restrict__ table, int cap, int L)
{
    __shared__ LevelSmem<R> sm;
    pdl_begin();
    const BatchHeader* hd = reinterpret_cast<const BatchHeader*>(table);
    const int* pf = reinterpret_cast<const int*>(table + table_prefix_offset()) + (2 + L) * (cap + 1);
    const int item = blockIdx.x;
    if (item >= pf[hd->n]) return;
    const int j = find_stream(pf, hd->n, item);
    const BatchEntry& e = reinterpret_cast<const BatchEntry*>(table + table_entries_offset(cap))[j];
    const FullArgs& a = e.fa;
    LevelArgs lv;
    lv.col_src = (L & 1) ? e.colB : e.colA;
    lv.col_dst = (L & 1) ? e.colA : e.colB;
    lv.var_off = a.var_off;
    lv.ghalf = a.ghalf;
    lv.level = L;
    lv.last = L == hd->levels - 1;
    lv.lin = res_layout(a.w, a.h, L);
    lv.lout = res_layout(a.w, a.h, L + 1);
    full_level_tile<ST, R, VAR, PL>(a, lv, level_geom(a.w, a.h, 1 << L, R), item - pf[j], sm);
}

// The same stage with each stream's tiles staged by TMA through `maps` where
// its maps exist (tma_slot >= 0 and bit L of tma_mask), with plain loads
// otherwise.
template <int ST, int R, bool VAR, bool PL>
__global__ void __launch_bounds__(kLvTX* kLvRows, LevelOcc<R>::kCtas)
    k_ms_level_tma(const char* __restrict__ table, int cap, int L, const __grid_constant__ StageMaps maps)
{
    __shared__ LevelSmem<R> sm;
    __shared__ __align__(8) uint64_t bar;
    pdl_begin();
    const BatchHeader* hd = reinterpret_cast<const BatchHeader*>(table);
    const int* pf = reinterpret_cast<const int*>(table + table_prefix_offset()) + (2 + L) * (cap + 1);
    const int item = blockIdx.x;
    if (item >= pf[hd->n]) return;
    const int j = find_stream(pf, hd->n, item);
    const BatchEntry& e = reinterpret_cast<const BatchEntry*>(table + table_entries_offset(cap))[j];
    const FullArgs& a = e.fa;
    LevelArgs lv;
    lv.col_src = (L & 1) ? e.colB : e.colA;
    lv.col_dst = (L & 1) ? e.colA : e.colB;
    lv.var_off = a.var_off;
    lv.ghalf = a.ghalf;
    lv.level = L;
    lv.last = L == hd->levels - 1;
    lv.lin = res_layout(a.w, a.h, L);
    lv.lout = res_layout(a.w, a.h, L + 1);
    const LevelGeom g = level_geom(a.w, a.h, 1 << L, R);
    if (e.tma_slot >= 0 && ((e.tma_mask >> L) & 1u)) {
        // level 0 stages from the tc plane and this step's guide plane, the others from their records
        const CUtensorMap* tm = PL ? &maps.m[3 * e.tma_slot] : &maps.m[e.tma_slot];
        const CUtensorMap* tm2 = PL ? &maps.m[3 * e.tma_slot + 1 + e.guide_k] : tm;
        full_level_tile_tma<ST, R, VAR, PL>(a, lv, g, item - pf[j], sm, bar, tm, tm2);
    } else {
        full_level_tile<ST, R, VAR, PL>(a, lv, g, item - pf[j], sm);
    }
}

} // namespace tg
