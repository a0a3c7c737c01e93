// Batched SVGF: many streams of uneven resolution in one persistent launch per
// frame step (include/tg_svgf.h, "batches"); the kernel and its work table are
// in svgf_batch_kernel.cuh.
//
// Per step the host fills a pinned work table (double buffered) that a CUDA
// graph copies to the device before the kernel: the graph is captured once per
// (tile shape, grid) and replayed for any subset of streams.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <new>
#include <vector>

#include "svgf_batch_kernel.cuh"
#include "svgf_internal.h"

namespace tg {

Img to_img(const tg_image& im, uint32_t w);

} // namespace tg

using namespace tg;

struct tg_svgf_batch {
    int device = 0;
    tg_svgf_params p{};
    int n = 0;
    std::vector<uint32_t> w, h;
    char* arena = nullptr;
    size_t state_bytes = 0, scratch_bytes = 0;
    struct Stream {
        void* guide[2];
        void* hist[2];
        void* mom[2];
        void* tc;
        float2* grad;
        int* fb_flags;
        void* colA;
        void* colB;
        char* state;
        size_t state_len;
        uint64_t frames;
    };
    std::vector<Stream> st;
    int cap = 0;
    size_t tbytes = 0;
    char* d_table[2] = {nullptr, nullptr};
    char* h_table[2] = {nullptr, nullptr};
    int* h_err = nullptr;  // 2 pinned flags
    cudaEvent_t table_free[2] = {nullptr, nullptr};
    bool table_used[2] = {false, false};
    int tbuf = 0;
    BarrierState* d_bar = nullptr;
    int R = 2, ctas = 0, grid = 0;
    bool use_graph = true, graphs_ok = true;
    cudaGraphExec_t exec[2] = {nullptr, nullptr};
    cudaStream_t cap_stream = nullptr;
    uint64_t steps = 0, timeouts = 0;
    double tuned_ms = 0.0;
    int sm_count = 0;
    long long spin_cycles = kBarrierSpinCycles;
    int barrier_extra = 0;
    int strategy = TG_SVGF_BATCH_STAGES;
    std::vector<int> grids[2];  // per-stage grid of the step in table buffer k
    std::vector<int> sig[2];    // grids the graph of buffer k was captured with
    // TMA staging of the stage kernels, for tiles of 1 and of 2 rows per thread: each stage's maps of the
    // first kTmaStreams streams (built once: the streams' buffers never move) and which levels of each stream
    // have them; empty when no map could be encoded (plain loads)
    std::vector<StageMaps> stage_maps[2];
    std::vector<unsigned> tma_mask[2];
};

namespace {

size_t al256(size_t v) { return (v + 255) / 256 * 256; }

struct DevGuard {
    int prev = -1;
    bool sw = false;
    explicit DevGuard(int d)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != d) sw = cudaSetDevice(d) == cudaSuccess;
    }
    ~DevGuard()
    {
        if (sw) cudaSetDevice(prev);
    }
};

using KernelFn = void (*)(const char*, int, BarrierState*, unsigned, long long);

KernelFn kernel_of(bool f16, int R)
{
    if (f16) return R == 1 ? k_batch_step<ST_FP16, 1> : k_batch_step<ST_FP16, 2>;
    return R == 1 ? k_batch_step<ST_FP32, 1> : k_batch_step<ST_FP32, 2>;
}

int max_ctas_per_sm(bool f16, int R)
{
    int nb = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel_of(f16, R), kLvTX * kLvRows, 0) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return nb;
}

void drop_graphs(tg_svgf_batch* b)
{
    for (auto& e : b->exec)
        if (e) {
            cudaGraphExecDestroy(e);
            e = nullptr;
        }
}

int set_config(tg_svgf_batch* b, int strategy, int R, int ctas)
{
    b->strategy = strategy;
    const bool f16 = b->p.storage == TG_SVGF_STORAGE_FP16;
    const int lim = max_ctas_per_sm(f16, R);
    if (lim < 1) return fail(TG_ERR_CUDA, "persistent kernel cannot be resident (occupancy query failed)");
    if (ctas <= 0 || ctas > lim) ctas = lim;
    b->R = R;
    b->ctas = ctas;
    b->grid = ctas * b->sm_count;
    drop_graphs(b);
    return TG_OK;
}

using PixFn = void (*)(const char*, int);
using LevFn = void (*)(const char*, int, int);
using LevTmaFn = void (*)(const char*, int, int, const StageMaps);

PixFn pixel_kernel(bool f16, int stage)
{
    if (f16) return stage == 0 ? k_ms_pixel<ST_FP16, 0> : k_ms_pixel<ST_FP16, 1>;
    return stage == 0 ? k_ms_pixel<ST_FP32, 0> : k_ms_pixel<ST_FP32, 1>;
}

template <int ST, int R> LevFn level_kernel_r(int L, int levels)
{
    if (L == 0) return k_ms_level<ST, R, true, true>;
    return L == levels - 1 ? k_ms_level<ST, R, false, false> : k_ms_level<ST, R, true, false>;
}

// The stage kernel of level L: level 0 stages from the planes, the last level writes only colour.
LevFn level_kernel(bool f16, int R, int L, int levels)
{
    if (f16) return R == 1 ? level_kernel_r<ST_FP16, 1>(L, levels) : level_kernel_r<ST_FP16, 2>(L, levels);
    return R == 1 ? level_kernel_r<ST_FP32, 1>(L, levels) : level_kernel_r<ST_FP32, 2>(L, levels);
}

template <int ST, int R> LevTmaFn level_tma_kernel_r(int L, int levels)
{
    if (L == 0) return k_ms_level_tma<ST, R, true, true>;
    return L == levels - 1 ? k_ms_level_tma<ST, R, false, false> : k_ms_level_tma<ST, R, true, false>;
}

LevTmaFn level_tma_kernel(bool f16, int R, int L, int levels)
{
    if (f16) return R == 1 ? level_tma_kernel_r<ST_FP16, 1>(L, levels) : level_tma_kernel_r<ST_FP16, 2>(L, levels);
    return R == 1 ? level_tma_kernel_r<ST_FP32, 1>(L, levels) : level_tma_kernel_r<ST_FP32, 2>(L, levels);
}

// One launch per stage over the work table of buffer k.
cudaError_t launch_stages(tg_svgf_batch* b, int k, cudaStream_t s)
{
    cudaError_t e;
    if ((e = cudaMemcpyAsync(b->d_table[k], b->h_table[k], b->tbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    const bool f16 = b->p.storage == TG_SVGF_STORAGE_FP16;
    const std::vector<int>& g = b->grids[k];
    for (size_t st = 0; st < g.size(); ++st) {
        if (g[st] <= 0) continue;
        const char* tab = b->d_table[k];
        const int L = int(st) - 2;
        if (st < 2)
            e = launch_chain(pixel_kernel(f16, int(st)), dim3(g[st]), dim3(kBlockX, kBlockY), s, tab, b->cap);
        else if (!b->stage_maps[b->R == 1 ? 0 : 1].empty())
            e = launch_chain(level_tma_kernel(f16, b->R, L, b->p.levels), dim3(g[st]), dim3(kLvTX, kLvRows), s, tab, b->cap,
                             L, b->stage_maps[b->R == 1 ? 0 : 1][st - 2]);
        else
            e = launch_chain(level_kernel(f16, b->R, L, b->p.levels), dim3(g[st]), dim3(kLvTX, kLvRows), s, tab, b->cap, L);
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_step(tg_svgf_batch* b, int k, cudaStream_t s)
{
    if (b->strategy == TG_SVGF_BATCH_STAGES) return launch_stages(b, k, s);
    cudaError_t e;
    if ((e = cudaMemsetAsync(b->d_bar, 0, sizeof(BarrierState), s)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(b->d_table[k], b->h_table[k], b->tbytes, cudaMemcpyHostToDevice, s)) != cudaSuccess)
        return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(b->grid);
    cfg.blockDim = dim3(kLvTX, kLvRows);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const char* tab = b->d_table[k];
    const int cap = b->cap;
    BarrierState* bar = b->d_bar;
    const unsigned expect = unsigned(b->grid + b->barrier_extra);
    const long long spin = b->spin_cycles;
    if ((e = cudaLaunchKernelEx(&cfg, kernel_of(b->p.storage == TG_SVGF_STORAGE_FP16, b->R), tab, cap, bar, expect,
                                spin)) != cudaSuccess)
        return e;
    return cudaMemcpyAsync(b->h_err + k, &b->d_bar->err, sizeof(int), cudaMemcpyDeviceToHost, s);
}

// Captures the step of table buffer k into a graph; on any failure the batch
// falls back to direct launches.
void capture(tg_svgf_batch* b, int k)
{
    if (!b->use_graph || !b->graphs_ok) return;
    if (b->exec[k] && b->sig[k] == b->grids[k]) return;
    if (b->exec[k]) {
        cudaGraphExecDestroy(b->exec[k]);
        b->exec[k] = nullptr;
    }
    b->sig[k] = b->grids[k];
    cudaGraph_t g = nullptr;
    if (cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        cudaGetLastError();
        b->graphs_ok = false;
        return;
    }
    const cudaError_t le = launch_step(b, k, b->cap_stream);
    const cudaError_t ee = cudaStreamEndCapture(b->cap_stream, &g);
    if (le != cudaSuccess || ee != cudaSuccess || !g || cudaGraphInstantiate(&b->exec[k], g, 0) != cudaSuccess) {
        cudaGetLastError();
        b->exec[k] = nullptr;
        b->graphs_ok = false;
    }
    if (g) cudaGraphDestroy(g);
}

int check_stream_inputs(const tg_svgf_batch* b, uint32_t id, const tg_svgf_inputs& in, const tg_svgf_outputs& out)
{
    static const int rad[] = {TG_FMT_RGBA32F, TG_FMT_RGBA16F};
    static const int dep[] = {TG_FMT_R32F};
    static const int nrm[] = {TG_FMT_RGB32F, TG_FMT_RGBA32F, TG_FMT_OCT16};
    static const int mot[] = {TG_FMT_RG32F, TG_FMT_RG16F};
    const uint32_t W = b->w[id], H = b->h[id];
    int st;
    if ((st = check_image("radiance", in.radiance, W, H, rad, 2))) return st;
    if ((st = check_image("depth", in.depth, W, H, dep, 1))) return st;
    if ((st = check_image("normal", in.normal, W, H, nrm, 3))) return st;
    if ((st = check_image("motion", in.motion, W, H, mot, 2))) return st;
    if ((st = check_image("denoised", out.denoised, W, H, rad, 2))) return st;
    return TG_OK;
}

// Fills host table k for this step and advances the streams' frame counters.
void fill_table(tg_svgf_batch* b, int k, uint32_t n, const uint32_t* ids, const tg_svgf_inputs* in,
                const tg_svgf_outputs* out)
{
    char* t = b->h_table[k];
    std::memset(t, 0, b->tbytes);
    BatchHeader* hd = reinterpret_cast<BatchHeader*>(t);
    hd->n = int(n);
    hd->levels = b->p.levels;
    hd->n_stages = 2 + b->p.levels;
    int* prefix = reinterpret_cast<int*>(t + table_prefix_offset());
    BatchEntry* ent = reinterpret_cast<BatchEntry*>(t + table_entries_offset(b->cap));
    b->grids[k].assign(hd->n_stages, 0);
    for (int stage = 0; stage < hd->n_stages; ++stage) {
        int* pf = prefix + stage * (b->cap + 1);
        int acc = 0;
        for (uint32_t j = 0; j < n; ++j) {
            pf[j] = acc;
            const int W = int(b->w[ids[j]]), H = int(b->h[ids[j]]);
            if (stage < 2)
                acc += ((W + kBlockX - 1) / kBlockX) * ((H + kBlockY - 1) / kBlockY);
            else
                acc += int(level_blocks(level_geom(W, H, 1 << (stage - 2), b->R)));
        }
        pf[n] = acc;
        b->grids[k][stage] = stage == 1 ? variance_grid(acc, b->sm_count) : acc;
    }
    for (uint32_t j = 0; j < n; ++j) {
        tg_svgf_batch::Stream& s = b->st[ids[j]];
        const int cur = int(s.frames & 1u), prev = cur ^ 1;
        const uint32_t W = b->w[ids[j]];
        FullArgs& a = ent[j].fa;
        a.w = int(W);
        a.h = int(b->h[ids[j]]);
        a.radiance = to_img(in[j].radiance, W);
        a.depth = to_img(in[j].depth, W);
        a.normal = to_img(in[j].normal, W);
        a.motion = to_img(in[j].motion, W);
        a.out = to_img(out[j].denoised, W);
        a.guide_prev = s.guide[prev];
        a.hist_prev = s.hist[prev];
        a.mom_prev = s.mom[prev];
        a.guide_cur = s.guide[cur];
        a.hist_cur = s.hist[cur];
        a.mom_cur = s.mom[cur];
        a.tc = s.tc;
        a.grad = s.grad;
        a.fb_flags = s.fb_flags;
        a.col_dst = s.colA;
        a.var_off = col_var_offset_of(b->p, W, b->h[ids[j]]);
        a.ghalf = col_guide_half_of(b->p, W, b->h[ids[j]]);
        a.alpha = b->p.alpha;
        a.alpha_m = b->p.moments_alpha;
        a.sigma_l = b->p.sigma_l;
        a.sigma_n = b->p.sigma_n;
        a.sigma_z = b->p.sigma_z;
        a.sq_n = sigma_n_squarings(b->p.sigma_n);
        a.max_history = b->p.max_history;
        a.fallback_frames = b->p.fallback_frames;
        ent[j].colA = s.colA;
        ent[j].colB = s.colB;
        const int r = b->R == 1 ? 0 : 1;
        ent[j].tma_slot = (!b->stage_maps[r].empty() && ids[j] < uint32_t(kTmaStreams)) ? int(ids[j]) : -1;
        ent[j].tma_mask = ent[j].tma_slot >= 0 ? b->tma_mask[r][ids[j]] : 0u;
        ent[j].guide_k = cur;
        s.frames++;
    }
}

// Waits until host table k may be rewritten and collects its step's barrier flag.
int reclaim(tg_svgf_batch* b, int k)
{
    if (!b->table_used[k]) return TG_OK;
    if (cudaEventSynchronize(b->table_free[k]) != cudaSuccess)
        return fail(TG_ERR_CUDA, "batch step failed: %s", cudaGetErrorString(cudaGetLastError()));
    b->table_used[k] = false;
    if (b->h_err[k]) {
        b->h_err[k] = 0;
        b->timeouts++;
        return fail(TG_ERR_TIMEOUT, "a batch step's grid barrier gave up; that step's outputs are invalid");
    }
    return TG_OK;
}

int run_step(tg_svgf_batch* b, uint32_t n, const uint32_t* ids, const tg_svgf_inputs* in, const tg_svgf_outputs* out,
             cudaStream_t stream)
{
    const int k = b->tbuf;
    int st = reclaim(b, k);
    if (st == TG_ERR_CUDA) return st;
    fill_table(b, k, n, ids, in, out);
    capture(b, k);
    cudaError_t e;
    if (b->exec[k])
        e = cudaGraphLaunch(b->exec[k], stream);
    else
        e = launch_step(b, k, stream);
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "batch step launch failed: %s", cudaGetErrorString(e));
    if (cudaEventRecord(b->table_free[k], stream) != cudaSuccess) return fail(TG_ERR_CUDA, "event record failed");
    b->table_used[k] = true;
    b->tbuf ^= 1;
    b->steps++;
    return st;
}

void free_batch(tg_svgf_batch* b)
{
    drop_graphs(b);
    for (int k = 0; k < 2; ++k) {
        if (b->d_table[k]) cudaFree(b->d_table[k]);
        if (b->h_table[k]) cudaFreeHost(b->h_table[k]);
        if (b->table_free[k]) cudaEventDestroy(b->table_free[k]);
    }
    if (b->h_err) cudaFreeHost(b->h_err);
    if (b->d_bar) cudaFree(b->d_bar);
    if (b->arena) cudaFree(b->arena);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
}

// Encodes the level maps of the first kTmaStreams streams for 1 and 2 rows per
// thread and arranges them per stage (StageMaps); a batch whose streams have no
// encodable map keeps plain loads.
void build_batch_maps(tg_svgf_batch* b)
{
    CUtensorMap m[kFullMaps];
    const int nt = b->n < kTmaStreams ? b->n : kTmaStreams;
    for (int r = 0; r < 2; ++r) {
        b->tma_mask[r].assign(b->n, 0u);
        b->stage_maps[r].assign(b->p.levels, StageMaps{});
        unsigned any = 0;
        for (int j = 0; j < nt; ++j) {
            const tg_svgf_batch::Stream& s = b->st[j];
            const unsigned mask = full_level_maps(b->p, b->w[j], b->h[j], r + 1, s.colA, s.colB, s.tc, s.guide[0],
                                                  s.guide[1], m);
            b->tma_mask[r][j] = mask;
            any |= mask;
            for (int L = 0; L < b->p.levels; ++L) {
                if (!((mask >> L) & 1u)) continue;
                if (L == 0) {
                    for (int q = 0; q < 3; ++q) b->stage_maps[r][0].m[3 * j + q] = m[q];
                } else {
                    b->stage_maps[r][L].m[j] = m[2 + L];
                }
            }
        }
        if (!any) b->stage_maps[r].clear();
    }
}

} // namespace

extern "C" {

int tg_svgf_batch_create(const tg_svgf_batch_desc* d, tg_svgf_batch** out)
{
    if (!d || !out) return fail(TG_ERR_INVALID, "null descriptor or output");
    *out = nullptr;
    if (d->n_streams < 1 || d->n_streams > TG_SVGF_BATCH_MAX_STREAMS || !d->widths || !d->heights)
        return fail(TG_ERR_INVALID, "n_streams must be 1..%d with widths and heights", TG_SVGF_BATCH_MAX_STREAMS);
    if (d->params.mode != TG_SVGF_MODE_FULL) return fail(TG_ERR_INVALID, "batches run the FULL mode");
    int st = validate_params(d->params);
    if (st) return st;
    if (d->rows_per_thread < 0 || d->rows_per_thread > 2) return fail(TG_ERR_INVALID, "rows_per_thread must be 0..2");
    for (uint32_t j = 0; j < d->n_streams; ++j)
        if (d->widths[j] == 0 || d->heights[j] == 0 || d->widths[j] > 32768 || d->heights[j] > 32768)
            return fail(TG_ERR_INVALID, "stream %u: size %ux%u outside 1..32768", j, d->widths[j], d->heights[j]);
    int dev = d->device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(TG_ERR_CUDA, "no current CUDA device");
    DevGuard g(dev);
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev) != cudaSuccess || !coop) {
        cudaGetLastError();
        return fail(TG_ERR_UNSUPPORTED, "device %d cannot launch cooperative kernels", dev);
    }
    tg_svgf_batch* b = new (std::nothrow) tg_svgf_batch();
    if (!b) return fail(TG_ERR_OOM, "host allocation failed");
    b->device = dev;
    b->p = d->params;
    b->n = int(d->n_streams);
    b->w.assign(d->widths, d->widths + d->n_streams);
    b->h.assign(d->heights, d->heights + d->n_streams);
    b->use_graph = d->use_graph != 0;
    cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, dev);
    if (d->barrier_timeout_us > 0) {
        int khz = 0;
        cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, dev);
        b->spin_cycles = (long long)d->barrier_timeout_us * (khz > 0 ? khz : 2000000) / 1000;
    }
    b->barrier_extra = d->debug_barrier_extra > 0 ? d->debug_barrier_extra : 0;
    const bool f16 = b->p.storage == TG_SVGF_STORAGE_FP16;
    const size_t gb = f16 ? 8 : 16, c4 = f16 ? 8 : 16, mm = f16 ? 4 : 8;
    // arena: per stream [state | scratch]
    std::vector<size_t> off(b->n + 1, 0);
    for (int j = 0; j < b->n; ++j) {
        const size_t np = size_t(b->w[j]) * b->h[j];
        const size_t sb = state_bytes_of(b->p, b->w[j], b->h[j]);
        const size_t cb = al256(np * c4) + al256(np * sizeof(float2)) + al256(fb_flags_bytes_of(b->w[j], b->h[j])) +
                          2 * col_bytes_of(b->p, b->w[j], b->h[j]);
        b->state_bytes += sb;
        b->scratch_bytes += cb;
        off[j + 1] = off[j] + sb + cb;
    }
    auto cleanup = [&](int status) {
        free_batch(b);
        delete b;
        return status;
    };
    if (cudaMalloc(&b->arena, off[b->n]) != cudaSuccess) {
        cudaGetLastError();
        b->arena = nullptr;
        return cleanup(fail(TG_ERR_OOM, "cudaMalloc of %zu batch bytes failed", off[b->n]));
    }
    b->st.resize(b->n);
    for (int j = 0; j < b->n; ++j) {
        const size_t np = size_t(b->w[j]) * b->h[j];
        char* p = b->arena + off[j];
        tg_svgf_batch::Stream& s = b->st[j];
        s.state = p;
        s.state_len = state_bytes_of(b->p, b->w[j], b->h[j]);
        for (int k = 0; k < 2; ++k) {
            s.guide[k] = p;
            p += al256(np * gb);
            s.hist[k] = p;
            p += al256(np * c4);
            s.mom[k] = p;
            p += al256(np * mm);
        }
        s.tc = p;
        p += al256(np * c4);
        s.grad = reinterpret_cast<float2*>(p);
        p += al256(np * sizeof(float2));
        s.fb_flags = reinterpret_cast<int*>(p);
        p += al256(fb_flags_bytes_of(b->w[j], b->h[j]));
        const size_t colb = col_bytes_of(b->p, b->w[j], b->h[j]);
        s.colA = p;
        p += colb;
        s.colB = p;
        s.frames = 0;
    }
    if (cudaMemset(b->arena, 0, off[b->n]) != cudaSuccess) return cleanup(fail(TG_ERR_CUDA, "arena clear failed"));
    build_batch_maps(b);
    b->cap = b->n;
    b->tbytes = table_bytes(b->cap);
    for (int k = 0; k < 2; ++k) {
        if (cudaMalloc(&b->d_table[k], b->tbytes) != cudaSuccess ||
            cudaHostAlloc(reinterpret_cast<void**>(&b->h_table[k]), b->tbytes, cudaHostAllocDefault) != cudaSuccess ||
            cudaEventCreateWithFlags(&b->table_free[k], cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return cleanup(fail(TG_ERR_OOM, "work table allocation failed"));
        }
    }
    if (cudaHostAlloc(reinterpret_cast<void**>(&b->h_err), 2 * sizeof(int), cudaHostAllocDefault) != cudaSuccess ||
        cudaMalloc(&b->d_bar, sizeof(BarrierState)) != cudaSuccess ||
        cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking) != cudaSuccess) {
        cudaGetLastError();
        return cleanup(fail(TG_ERR_OOM, "barrier allocation failed"));
    }
    b->h_err[0] = b->h_err[1] = 0;
    if (cudaMemset(b->d_bar, 0, sizeof(BarrierState)) != cudaSuccess || cudaDeviceSynchronize() != cudaSuccess)
        return cleanup(fail(TG_ERR_CUDA, "batch initialisation failed"));
    if (d->strategy != TG_SVGF_BATCH_STAGES && d->strategy != TG_SVGF_BATCH_PERSISTENT)
        return cleanup(fail(TG_ERR_INVALID, "strategy %d unknown", d->strategy));
    st = set_config(b, d->strategy, d->rows_per_thread ? d->rows_per_thread : 2, d->ctas_per_sm);
    if (st) return cleanup(st);
    *out = b;
    return TG_OK;
}

static int check_step(tg_svgf_batch* b, uint32_t n, const uint32_t* ids, const tg_svgf_inputs* in,
                      const tg_svgf_outputs* out)
{
    if (!b) return fail(TG_ERR_INVALID, "null batch");
    if (n == 0) return TG_OK;
    if (!ids || !in || !out) return fail(TG_ERR_INVALID, "null stream ids, inputs or outputs");
    if (n > uint32_t(b->n)) return fail(TG_ERR_INVALID, "more streams than the batch holds");
    std::vector<char> seen(b->n, 0);
    for (uint32_t j = 0; j < n; ++j) {
        if (ids[j] >= uint32_t(b->n)) return fail(TG_ERR_INVALID, "stream id %u out of range", ids[j]);
        if (seen[ids[j]]) return fail(TG_ERR_INVALID, "stream %u listed twice in one step", ids[j]);
        seen[ids[j]] = 1;
        int st = check_stream_inputs(b, ids[j], in[j], out[j]);
        if (st) return st;
    }
    return TG_OK;
}

int tg_svgf_batch_denoise(tg_svgf_batch* b, uint32_t n, const uint32_t* ids, const tg_svgf_inputs* in,
                          const tg_svgf_outputs* out, void* stream)
{
    int st = check_step(b, n, ids, in, out);
    if (st || n == 0) return st;
    DevGuard g(b->device);
    return run_step(b, n, ids, in, out, static_cast<cudaStream_t>(stream));
}

int tg_svgf_batch_autotune(tg_svgf_batch* b, uint32_t n, const uint32_t* ids, const tg_svgf_inputs* in,
                           const tg_svgf_outputs* out, uint32_t steps, void* stream_v)
{
    int st = check_step(b, n, ids, in, out);
    if (st) return st;
    if (n == 0 || steps == 0) return fail(TG_ERR_INVALID, "autotune needs streams and steps");
    DevGuard g(b->device);
    cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
    const bool f16 = b->p.storage == TG_SVGF_STORAGE_FP16;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
        return fail(TG_ERR_CUDA, "event creation failed");
    double best = 1e30;
    int bestR = b->R, bestC = b->ctas, bestS = b->strategy;
    for (int cand = 0; cand < 2 * (1 + 3) && st == TG_OK; ++cand) {
        // candidates: (stages, R) for R = 1, 2, then (persistent, R, ctas) with 2, 4 or 6 CTAs of 128 threads
        // per SM, up to the occupancy limit
        const int strat = cand < 2 ? TG_SVGF_BATCH_STAGES : TG_SVGF_BATCH_PERSISTENT;
        const int R = cand < 2 ? cand + 1 : 1 + (cand - 2) / 3;
        const int c = cand < 2 ? 0 : 2 * (1 + (cand - 2) % 3);
        if (strat == TG_SVGF_BATCH_PERSISTENT && c > max_ctas_per_sm(f16, R)) continue;
        if ((st = set_config(b, strat, R, c))) break;
        if ((st = run_step(b, n, ids, in, out, stream)) != TG_OK) break;  // warm-up, also captures
        if ((st = run_step(b, n, ids, in, out, stream)) != TG_OK) break;
        cudaEventRecord(e0, stream);
        for (uint32_t k = 0; k < steps && st == TG_OK; ++k) st = run_step(b, n, ids, in, out, stream);
        cudaEventRecord(e1, stream);
        if (st) break;
        if (cudaEventSynchronize(e1) != cudaSuccess) {
            st = fail(TG_ERR_CUDA, "autotune step failed");
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms / steps < best) {
            best = ms / steps;
            bestR = R;
            bestC = c;
            bestS = strat;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int k = 0; k < 2; ++k) {
        const int r = reclaim(b, k);
        if (!st) st = r;
    }
    if (st) return st;
    if ((st = set_config(b, bestS, bestR, bestC))) return st;
    b->tuned_ms = best;
    // tuning advanced every stream: zero all state
    for (auto& s : b->st) {
        if (cudaMemsetAsync(s.state, 0, s.state_len, stream) != cudaSuccess)
            return fail(TG_ERR_CUDA, "state clear failed");
        s.frames = 0;
    }
    return TG_OK;
}

int tg_svgf_batch_reset_stream(tg_svgf_batch* b, uint32_t id, void* stream)
{
    if (!b) return fail(TG_ERR_INVALID, "null batch");
    if (id >= uint32_t(b->n)) return fail(TG_ERR_INVALID, "stream id %u out of range", id);
    DevGuard g(b->device);
    tg_svgf_batch::Stream& s = b->st[id];
    if (cudaMemsetAsync(s.state, 0, s.state_len, static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return fail(TG_ERR_CUDA, "state clear failed");
    s.frames = 0;
    return TG_OK;
}

int tg_svgf_batch_synchronize(tg_svgf_batch* b)
{
    if (!b) return fail(TG_ERR_INVALID, "null batch");
    DevGuard g(b->device);
    int st = TG_OK;
    for (int k = 0; k < 2; ++k) {
        const int r = reclaim(b, k);
        if (!st) st = r;
    }
    return st;
}

int tg_svgf_batch_get_info(const tg_svgf_batch* b, tg_svgf_batch_info* info)
{
    if (!b || !info) return fail(TG_ERR_INVALID, "null batch or info");
    std::memset(info, 0, sizeof *info);
    info->n_streams = uint32_t(b->n);
    info->rows_per_thread = b->R;
    info->ctas_per_sm = b->ctas;
    info->grid_ctas = b->grid;
    info->graphs = (b->use_graph && b->graphs_ok) ? 1 : 0;
    info->strategy = b->strategy;
    info->state_bytes = b->state_bytes;
    info->scratch_bytes = b->scratch_bytes;
    info->steps = b->steps;
    info->barrier_timeouts = b->timeouts;
    info->tuned_ms = b->tuned_ms;
    return TG_OK;
}

void tg_svgf_batch_destroy(tg_svgf_batch* b)
{
    if (!b) return;
    DevGuard g(b->device);
    cudaDeviceSynchronize();
    free_batch(b);
    delete b;
}

} // extern "C"
