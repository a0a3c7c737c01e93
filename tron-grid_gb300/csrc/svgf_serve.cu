// Serving loop: continuous batching of frames from many sessions under an HBM
// budget (include/tg_svgf.h, "serving").
//
// Threads.  Producers call tg_svgf_server_submit from any thread; a scheduler
// thread forms launches; a completion thread waits for each launch's result
// copy and completes its tickets.  Up to kMaxInflight launches are in flight:
// while launch k computes, the inputs of the launches after it are already
// being copied in (on a separate copy stream), and the outputs of k-1 copied
// out.  A session has at most two frames in flight, because its staging slots
// alternate by frame parity.  Completion events come from a pool and are
// reused.
//
// Memory.  One device allocation of the budget holds every resident session;
// a first-fit allocator hands out one block per session: state (guide,
// history, moments, ping-pong), scratch (temporal colour, depth gradient,
// a-trous images) and two input and two output staging slots (alternating by
// the session's frame parity, so that a session's next frame can be copied in
// while its current one runs).  A session that does not fit evicts the least
// recently used idle session; an evicted session is re-admitted with zeroed
// state, i.e. its next frame is a full disocclusion.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "svgf_batch_kernel.cuh"
#include "svgf_internal.h"

namespace tg {
Img to_img(const tg_image& im, uint32_t w);
}

using namespace tg;

namespace {

using Clock = std::chrono::steady_clock;

size_t al256(size_t v) { return (v + 255) / 256 * 256; }

// First-fit allocator over [0, cap) with coalescing of free neighbours.
class Arena {
public:
    explicit Arena(size_t cap = 0) { reset(cap); }
    void reset(size_t cap)
    {
        free_.clear();
        if (cap) free_[0] = cap;
        used_ = 0;
    }
    bool alloc(size_t bytes, size_t& off)
    {
        bytes = al256(bytes);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                off = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[off + bytes] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = al256(bytes);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }

private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0;
};

struct Req {
    uint64_t ticket = 0, session = 0;
    uint32_t w = 0, h = 0;
    tg_svgf_inputs in{};
    tg_svgf_outputs out{};
    Clock::time_point t_submit, t_launch, t_done;
    int status = -1;  // -1 = pending
    uint32_t batch_size = 0;
};

struct Sess {
    uint64_t id = 0;
    uint32_t w = 0, h = 0;
    int fmt[5] = {0, 0, 0, 0, 0};  // radiance, depth, normal, motion, output
    bool resident = false, ended = false, fresh = false;
    size_t off = 0, bytes = 0;
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
    char* in_slot[2][4];
    tg_image in_view[4];  // the current frame's inputs as the kernels read them (a slot, or mapped host memory)
    char* out_slot[2];
    uint64_t frames = 0, lru = 0;
    // TMA maps of the session's a-trous levels (full_level_maps layout), encoded at admission, and which levels
    // have them
    CUtensorMap maps[kFullMaps];
    unsigned tma_mask = 0;
    int pending = 0;  // queued + running frames
    int running = 0;  // frames in launches not yet complete (at most 2)
};

// Launches in flight at once (each with its own work table and graph).
#ifndef TG_SERVE_MAX_INFLIGHT
#define TG_SERVE_MAX_INFLIGHT 3
#endif
constexpr int kMaxInflight = TG_SERVE_MAX_INFLIGHT;

struct Flight {
    std::vector<Req*> reqs;
    std::vector<Sess*> sess;
    cudaEvent_t ev_comp = nullptr, ev_d2h = nullptr;
    int table_k = -1;
    bool launch_failed = false;  // a kernel of this launch was rejected at launch time
};

} // namespace

struct tg_svgf_server {
    tg_svgf_server_desc d{};
    int device = 0, sm_count = 0;
    bool f16 = false;
    char* base = nullptr;
    Arena arena;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_flight;
    std::deque<Req*> queue;
    std::unordered_map<uint64_t, Req*> reqs;
    std::unordered_map<uint64_t, Sess> sess;
    std::deque<Flight*> inflight;
    uint64_t next_ticket = 1, lru_tick = 0;
    bool stop = false, sched_done = false;
    std::thread sched, compl_thread;
    cudaStream_t s_h2d = nullptr, s_comp = nullptr, s_d2h = nullptr, cap_stream = nullptr;
    cudaEvent_t ev_h2d = nullptr;
    // persistent-launch machinery (batching)
    int cap = 0, grid = 0, launches = 0;
    size_t tbytes = 0;
    char* d_table[kMaxInflight] = {};
    char* h_table[kMaxInflight] = {};
    int* h_err = nullptr;
    BarrierState* d_bar = nullptr;
    cudaGraphExec_t exec[kMaxInflight] = {};
    std::vector<cudaEvent_t> ev_pool;  // completion events, reused
    StageMaps stage_maps[10];          // the stage kernels' maps of the launch being formed (one per level)
    bool graphs_ok = true;
    // stats
    uint64_t submitted = 0, completed = 0, failed = 0, admissions = 0, evictions = 0, n_launches = 0;
    uint64_t peak_resident = 0;
    uint32_t max_batch_seen = 0;
    std::vector<float> lat;
    double px_done = 0.0;
    Clock::time_point t_first, t_last;
    bool have_first = false;
};

namespace {

constexpr int kR = 2;

using StepFn = void (*)(const char*, int, BarrierState*, unsigned, long long);
StepFn step_kernel(bool f16) { return f16 ? k_batch_step<ST_FP16, kR> : k_batch_step<ST_FP32, kR>; }

size_t in_bytes(const Sess& s, int k) { return size_t(fmt_bytes(s.fmt[k])) * s.w * s.h; }

size_t slot_bytes(const tg_svgf_params& p, const Sess& s)
{
    const size_t np = size_t(s.w) * s.h;
    const bool f16 = p.storage == TG_SVGF_STORAGE_FP16;
    const size_t c4 = f16 ? 8 : 16;
    size_t b = al256(state_bytes_of(p, s.w, s.h));
    b += al256(np * c4) + al256(np * sizeof(float2)) + al256(fb_flags_bytes_of(s.w, s.h)) + 2 * col_bytes_of(p, s.w, s.h);
    for (int k = 0; k < 4; ++k) b += 2 * al256(in_bytes(s, k));
    b += 2 * al256(size_t(fmt_bytes(s.fmt[4])) * np);
    return b;
}

void carve(tg_svgf_server* sv, Sess& s)
{
    const size_t np = size_t(s.w) * s.h;
    const size_t gb = sv->f16 ? 8 : 16, c4 = sv->f16 ? 8 : 16, mm = sv->f16 ? 4 : 8;
    char* p = sv->base + s.off;
    s.state = p;
    for (int k = 0; k < 2; ++k) {
        s.guide[k] = p;
        p += al256(np * gb);
        s.hist[k] = p;
        p += al256(np * c4);
        s.mom[k] = p;
        p += al256(np * mm);
    }
    s.state_len = size_t(p - s.state);
    s.tc = p;
    p += al256(np * c4);
    s.grad = reinterpret_cast<float2*>(p);
    p += al256(np * sizeof(float2));
    s.fb_flags = reinterpret_cast<int*>(p);
    p += al256(fb_flags_bytes_of(s.w, s.h));
    const size_t colb = col_bytes_of(sv->d.params, s.w, s.h);
    s.colA = p;
    p += colb;
    s.colB = p;
    p += colb;
    for (int f = 0; f < 2; ++f)
        for (int k = 0; k < 4; ++k) {
            s.in_slot[f][k] = p;
            p += al256(in_bytes(s, k));
        }
    for (int f = 0; f < 2; ++f) {
        s.out_slot[f] = p;
        p += al256(size_t(fmt_bytes(s.fmt[4])) * np);
    }
    s.tma_mask = full_level_maps(sv->d.params, s.w, s.h, kR, s.colA, s.colB, s.tc, s.guide[0], s.guide[1], s.maps);
}

void release(tg_svgf_server* sv, Sess& s)
{
    if (!s.resident) return;
    sv->arena.release(s.off, s.bytes);
    s.resident = false;
}

// Makes `s` resident, evicting idle sessions not in `busy`; false if it must wait.
bool admit(tg_svgf_server* sv, Sess& s, const std::vector<uint64_t>& busy)
{
    if (s.resident) return true;
    s.bytes = slot_bytes(sv->d.params, s);
    size_t off = 0;
    while (!sv->arena.alloc(s.bytes, off)) {
        Sess* victim = nullptr;
        for (auto& kv : sv->sess) {
            Sess& c = kv.second;
            if (!c.resident || c.pending > 0 || &c == &s) continue;
            if (std::find(busy.begin(), busy.end(), c.id) != busy.end()) continue;
            if (!victim || c.lru < victim->lru) victim = &c;
        }
        if (!victim) return false;
        release(sv, *victim);
        sv->evictions++;
    }
    s.off = off;
    s.resident = true;
    s.fresh = true;
    s.frames = 0;
    carve(sv, s);
    sv->admissions++;
    sv->peak_resident = std::max<uint64_t>(sv->peak_resident, sv->arena.used());
    return true;
}

FullArgs args_for(tg_svgf_server* sv, Sess& s)
{
    const int cur = int(s.frames & 1u), prev = cur ^ 1;
    FullArgs a{};
    a.w = int(s.w);
    a.h = int(s.h);
    const int slot = cur;
    tg_image im[5];
    for (int k = 0; k < 4; ++k) im[k] = s.in_view[k];
    im[4] = tg_image{s.out_slot[slot], 0, s.fmt[4], 0};
    a.radiance = to_img(im[0], s.w);
    a.depth = to_img(im[1], s.w);
    a.normal = to_img(im[2], s.w);
    a.motion = to_img(im[3], s.w);
    a.out = to_img(im[4], s.w);
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
    a.var_off = col_var_offset_of(sv->d.params, s.w, s.h);
    a.ghalf = col_guide_half_of(sv->d.params, s.w, s.h);
    const tg_svgf_params& p = sv->d.params;
    a.alpha = p.alpha;
    a.alpha_m = p.moments_alpha;
    a.sigma_l = p.sigma_l;
    a.sigma_n = p.sigma_n;
    a.sigma_z = p.sigma_z;
    a.sq_n = sigma_n_squarings(p.sigma_n);
    a.max_history = p.max_history;
    a.fallback_frames = p.fallback_frames;
    return a;
}

cudaError_t enqueue_persistent(tg_svgf_server* sv, int k, cudaStream_t st)
{
    cudaError_t e;
    if ((e = cudaMemsetAsync(sv->d_bar, 0, sizeof(BarrierState), st)) != cudaSuccess) return e;
    if ((e = cudaMemcpyAsync(sv->d_table[k], sv->h_table[k], sv->tbytes, cudaMemcpyHostToDevice, st)) != cudaSuccess)
        return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(sv->grid);
    cfg.blockDim = dim3(kLvTX, kLvRows);
    cfg.stream = st;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const char* tab = sv->d_table[k];
    const int cap = sv->cap;
    BarrierState* bar = sv->d_bar;
    const unsigned expect = unsigned(sv->grid);
    const long long spin = kBarrierSpinCycles;
    if ((e = cudaLaunchKernelEx(&cfg, step_kernel(sv->f16), tab, cap, bar, expect, spin)) != cudaSuccess) return e;
    return cudaMemcpyAsync(sv->h_err + k, &sv->d_bar->err, sizeof(int), cudaMemcpyDeviceToHost, st);
}

void launch_stage_kernels(tg_svgf_server* sv, int k, const std::vector<int>& grids)
{
    cudaStream_t st = sv->s_comp;
    cudaMemcpyAsync(sv->d_table[k], sv->h_table[k], sv->tbytes, cudaMemcpyHostToDevice, st);
    for (size_t g = 0; g < grids.size(); ++g) {
        if (grids[g] <= 0) continue;
        const char* tab = sv->d_table[k];
        if (g < 2) {
            auto p16 = g == 0 ? k_ms_pixel<ST_FP16, 0> : k_ms_pixel<ST_FP16, 1>;
            auto p32 = g == 0 ? k_ms_pixel<ST_FP32, 0> : k_ms_pixel<ST_FP32, 1>;
            launch_chain(sv->f16 ? p16 : p32, dim3(grids[g]), dim3(kBlockX, kBlockY), st, tab, sv->cap);
        } else {
            // level 0 stages from the planes, the last level writes only colour
            const int L = int(g) - 2;
            const bool pl = L == 0, var = pl || L != sv->d.params.levels - 1;
            auto k16 = pl ? k_ms_level_tma<ST_FP16, kR, true, true>
                          : (var ? k_ms_level_tma<ST_FP16, kR, true, false> : k_ms_level_tma<ST_FP16, kR, false, false>);
            auto k32 = pl ? k_ms_level_tma<ST_FP32, kR, true, true>
                          : (var ? k_ms_level_tma<ST_FP32, kR, true, false> : k_ms_level_tma<ST_FP32, kR, false, false>);
            launch_chain(sv->f16 ? k16 : k32, dim3(grids[g]), dim3(kLvTX, kLvRows), st, tab, sv->cap, L, sv->stage_maps[L]);
        }
    }
}

void launch_batch(tg_svgf_server* sv, std::vector<Sess*>& ss, int k)
{
    char* t = sv->h_table[k];
    std::memset(t, 0, sv->tbytes);
    BatchHeader* hd = reinterpret_cast<BatchHeader*>(t);
    const int n = int(ss.size());
    hd->n = n;
    hd->levels = sv->d.params.levels;
    hd->n_stages = 2 + hd->levels;
    int* prefix = reinterpret_cast<int*>(t + table_prefix_offset());
    BatchEntry* ent = reinterpret_cast<BatchEntry*>(t + table_entries_offset(sv->cap));
    std::vector<int> grids(hd->n_stages, 0);
    for (int stage = 0; stage < hd->n_stages; ++stage) {
        int* pf = prefix + stage * (sv->cap + 1);
        int acc = 0;
        for (int j = 0; j < n; ++j) {
            pf[j] = acc;
            const int W = int(ss[j]->w), H = int(ss[j]->h);
            if (stage < 2)
                acc += ((W + kBlockX - 1) / kBlockX) * ((H + kBlockY - 1) / kBlockY);
            else
                acc += int(level_blocks(level_geom(W, H, 1 << (stage - 2), kR)));
        }
        pf[n] = acc;
        grids[stage] = stage == 1 ? variance_grid(acc, sv->sm_count) : acc;
    }
    // the stage kernels' maps: slot j of each stage's StageMaps holds the j-th frame's session's maps
    const bool stages = sv->d.strategy == TG_SVGF_BATCH_STAGES;
    for (int j = 0; j < n; ++j) {
        Sess& sj = *ss[j];
        ent[j].fa = args_for(sv, sj);
        ent[j].colA = sj.colA;
        ent[j].colB = sj.colB;
        ent[j].tma_slot = -1;
        if (stages && j < kTmaStreams && sj.tma_mask) {
            ent[j].tma_slot = j;
            ent[j].tma_mask = sj.tma_mask;
            ent[j].guide_k = int(sj.frames & 1u);
            for (int L = 0; L < hd->levels; ++L) {
                if (!((sj.tma_mask >> L) & 1u)) continue;
                if (L == 0)
                    for (int q = 0; q < 3; ++q) sv->stage_maps[0].m[3 * j + q] = sj.maps[q];
                else
                    sv->stage_maps[L].m[j] = sj.maps[2 + L];
            }
        }
    }
    if (sv->d.strategy == TG_SVGF_BATCH_STAGES) {
        launch_stage_kernels(sv, k, grids);
        return;
    }
    if (sv->d.use_graph && sv->graphs_ok && !sv->exec[k]) {
        cudaGraph_t g = nullptr;
        bool ok = cudaStreamBeginCapture(sv->cap_stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
        if (ok) {
            const cudaError_t le = enqueue_persistent(sv, k, sv->cap_stream);
            const cudaError_t ee = cudaStreamEndCapture(sv->cap_stream, &g);
            ok = le == cudaSuccess && ee == cudaSuccess && g && cudaGraphInstantiate(&sv->exec[k], g, 0) == cudaSuccess;
        }
        if (g) cudaGraphDestroy(g);
        if (!ok) {
            cudaGetLastError();
            sv->exec[k] = nullptr;
            sv->graphs_ok = false;
        }
    }
    if (sv->exec[k])
        cudaGraphLaunch(sv->exec[k], sv->s_comp);
    else
        enqueue_persistent(sv, k, sv->s_comp);
}

// The plain per-request path: the single-stream kernels, one launch each.
void launch_plain(tg_svgf_server* sv, Sess& s)
{
    FullArgs a = args_for(sv, s);
    const dim3 blk(kBlockX, kBlockY);
    const dim3 grd((s.w + kBlockX - 1) / kBlockX, (s.h + kBlockY - 1) / kBlockY);
    cudaStream_t st = sv->s_comp;
    const int vg = variance_grid(int(grd.x * grd.y), sv->sm_count);
    launch_chain(sv->f16 ? k_full_temporal<ST_FP16> : k_full_temporal<ST_FP32>, grd, blk, st, a);
    launch_chain(sv->f16 ? k_full_variance<ST_FP16> : k_full_variance<ST_FP32>, dim3(vg), blk, st, a);
    void* src = s.colA;
    void* oth = s.colB;
    for (int lv = 0; lv < sv->d.params.levels; ++lv) {
        a.col_src = src;
        a.col_dst = oth;
        a.level = lv;
        a.stride = 1 << lv;
        a.last = lv == sv->d.params.levels - 1;
        a.lin = res_layout(a.w, a.h, lv);
        a.lout = res_layout(a.w, a.h, lv + 1);
        const LevelGeom g = level_geom(a.w, a.h, a.stride, kR);
        const dim3 lgrid(level_blocks(g)), lblk(kLvTX, kLvRows);
        // level 0 stages from the planes, the last level writes only colour; tiles are staged by TMA where the
        // session's maps were encoded, as the single-stream path does
        if ((s.tma_mask >> lv) & 1u) {
            const LevelArgs la = level_args_of(a);
            const CUtensorMap& tm = lv == 0 ? s.maps[0] : s.maps[2 + lv];
            const CUtensorMap& tm2 = lv == 0 ? s.maps[1 + int(s.frames & 1u)] : tm;
            auto t16 = lv == 0 ? k_full_level_tma<ST_FP16, kR, true, true>
                               : (a.last ? k_full_level_tma<ST_FP16, kR, false, false>
                                         : k_full_level_tma<ST_FP16, kR, true, false>);
            auto t32 = lv == 0 ? k_full_level_tma<ST_FP32, kR, true, true>
                               : (a.last ? k_full_level_tma<ST_FP32, kR, false, false>
                                         : k_full_level_tma<ST_FP32, kR, true, false>);
            launch_chain(sv->f16 ? t16 : t32, lgrid, lblk, st, a, la, g, tm, tm2);
        } else {
            auto k16 = lv == 0 ? k_full_level_tiled<ST_FP16, kR, true, true>
                               : (a.last ? k_full_level_tiled<ST_FP16, kR, false> : k_full_level_tiled<ST_FP16, kR, true>);
            auto k32 = lv == 0 ? k_full_level_tiled<ST_FP32, kR, true, true>
                               : (a.last ? k_full_level_tiled<ST_FP32, kR, false> : k_full_level_tiled<ST_FP32, kR, true>);
            launch_chain(sv->f16 ? k16 : k32, lgrid, lblk, st, a, g);
        }
        std::swap(src, oth);
    }
}

// Device address at which the GPU reads host memory `p` in place: page-locked
// memory mapped into the device's address space (cudaHostAlloc,
// cudaHostRegister) on this server's device; null for anything else (pageable
// memory, device memory), which is copied in instead.
void* mapped_view(const tg_svgf_server* sv, const void* p)
{
    cudaPointerAttributes at;
    if (!p || cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (at.type != cudaMemoryTypeHost || !at.devicePointer || at.device != sv->device) return nullptr;
    return at.devicePointer;
}

// A completion event from the pool (created when the pool is empty); the
// caller holds sv->mu.
cudaEvent_t pool_event(tg_svgf_server* sv)
{
    if (!sv->ev_pool.empty()) {
        cudaEvent_t e = sv->ev_pool.back();
        sv->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
    return e;
}

void finish(tg_svgf_server* sv, Req* r, int status, Clock::time_point now)
{
    r->status = status;
    r->t_done = now;
    if (status == TG_OK) {
        sv->completed++;
        if (sv->lat.size() < (size_t(1) << 22))
            sv->lat.push_back(float(std::chrono::duration<double, std::milli>(now - r->t_submit).count()));
        sv->px_done += double(r->w) * r->h;
        sv->t_last = now;
    } else {
        sv->failed++;
    }
}

void scheduler(tg_svgf_server* sv)
{
    cudaSetDevice(sv->device);
    int batch_no = 0;
    for (;;) {
        std::vector<Req*> batch;
        std::vector<Sess*> ss;
        std::vector<Sess*> fresh;
        bool failed_any = false;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv_work.wait(lk, [&] {
                return (sv->stop && sv->queue.empty()) || (!sv->queue.empty() && int(sv->inflight.size()) < kMaxInflight);
            });
            if (sv->stop && sv->queue.empty()) break;
            std::vector<uint64_t> busy;
            const uint32_t maxb = sv->d.batching ? sv->d.max_batch : 1u;
            const uint64_t max_px = sv->d.max_batch_pixels ? sv->d.max_batch_pixels : (uint64_t(4) << 20);
            uint64_t batch_px = 0;
            const Clock::time_point now = Clock::now();
            for (auto it = sv->queue.begin(); it != sv->queue.end() && batch.size() < maxb;) {
                Req* r = *it;
                Sess& s = sv->sess[r->session];
                if (s.ended) {
                    finish(sv, r, TG_ERR_STATE, now);
                    failed_any = true;
                    it = sv->queue.erase(it);
                    if (--s.pending == 0) {
                        release(sv, s);
                        sv->sess.erase(r->session);
                    }
                    continue;
                }
                if (s.running >= 2 || std::find(busy.begin(), busy.end(), s.id) != busy.end()) {
                    ++it;
                    continue;
                }
                if (!batch.empty() && batch_px + uint64_t(r->w) * r->h > max_px) break;
                // a frame of another size or format restarts the session
                const int f[5] = {r->in.radiance.format, r->in.depth.format, r->in.normal.format, r->in.motion.format,
                                  r->out.denoised.format};
                const bool same = s.w == r->w && s.h == r->h && std::equal(f, f + 5, s.fmt);
                if (!same) {
                    if (s.resident && s.pending > 1) {  // its earlier frames are still running
                        busy.push_back(s.id);
                        ++it;
                        continue;
                    }
                    release(sv, s);
                    s.w = r->w;
                    s.h = r->h;
                    std::copy(f, f + 5, s.fmt);
                }
                if (!s.resident) {
                    if (slot_bytes(sv->d.params, s) > sv->d.hbm_budget_bytes) {
                        finish(sv, r, TG_ERR_BUDGET, now);
                        failed_any = true;
                        s.pending--;
                        it = sv->queue.erase(it);
                        continue;
                    }
                    if (!admit(sv, s, busy)) {  // waits for running frames to free memory
                        busy.push_back(s.id);
                        ++it;
                        continue;
                    }
                }
                if (s.fresh) fresh.push_back(&s);
                s.fresh = false;
                busy.push_back(s.id);
                s.running++;
                batch_px += uint64_t(r->w) * r->h;
                batch.push_back(r);
                ss.push_back(&s);
                it = sv->queue.erase(it);
            }
            if (batch.empty()) {
                if (failed_any) {
                    lk.unlock();
                    sv->cv_done.notify_all();
                    continue;
                }
                // nothing launchable now (memory held by running frames): wait for a completion
                sv->cv_work.wait_for(lk, std::chrono::milliseconds(1));
                continue;
            }
        }
        if (failed_any) sv->cv_done.notify_all();
        const int k = batch_no % kMaxInflight;
        // Inputs: page-locked, mapped host images are read by the temporal kernel in place over the host link
        // (no copy, no API call per image); others are copied into the session's slot on the copy stream
        // (slots alternate by frame parity).
        bool copied = false;
        for (size_t j = 0; j < batch.size(); ++j) {
            Req* r = batch[j];
            Sess& s = *ss[j];
            const int slot = int(s.frames & 1u);
            const tg_image* src[4] = {&r->in.radiance, &r->in.depth, &r->in.normal, &r->in.motion};
            for (int q = 0; q < 4; ++q) {
                const size_t row = size_t(fmt_bytes(s.fmt[q])) * s.w;
                const size_t hp = src[q]->pitch_bytes ? size_t(src[q]->pitch_bytes) : row;
                if (void* dv = mapped_view(sv, src[q]->ptr)) {
                    s.in_view[q] = tg_image{dv, int64_t(hp), s.fmt[q], 0};
                    continue;
                }
                copy_image_async(s.in_slot[slot][q], row, src[q]->ptr, hp, row, s.h, cudaMemcpyHostToDevice, sv->s_h2d);
                s.in_view[q] = tg_image{s.in_slot[slot][q], 0, s.fmt[q], 0};
                copied = true;
            }
        }
        if (copied) {
            cudaEventRecord(sv->ev_h2d, sv->s_h2d);
            cudaStreamWaitEvent(sv->s_comp, sv->ev_h2d, 0);
        }
        for (Sess* s : fresh) cudaMemsetAsync(s->state, 0, s->state_len, sv->s_comp);
        Flight* fl = new Flight();
        fl->reqs = batch;
        fl->sess = ss;
        // a launch of one frame runs the single-stream kernels (no work table to copy or search); two or more run
        // the batched kernels, whose results are bit-identical
        const bool batched = sv->d.batching && batch.size() > 1;
        fl->table_k = (batched && sv->d.strategy == TG_SVGF_BATCH_PERSISTENT) ? k : -1;
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            fl->ev_comp = pool_event(sv);
            fl->ev_d2h = pool_event(sv);
        }
        const Clock::time_point tl = Clock::now();
        if (batched)
            launch_batch(sv, ss, k);
        else
            launch_plain(sv, *ss[0]);
        fl->launch_failed = cudaGetLastError() != cudaSuccess;
        cudaEventRecord(fl->ev_comp, sv->s_comp);
        cudaStreamWaitEvent(sv->s_d2h, fl->ev_comp, 0);
        for (size_t j = 0; j < batch.size(); ++j) {
            Req* r = batch[j];
            Sess& s = *ss[j];
            const int slot = int(s.frames & 1u);
            const size_t row = size_t(fmt_bytes(s.fmt[4])) * s.w;
            const size_t op = r->out.denoised.pitch_bytes ? size_t(r->out.denoised.pitch_bytes) : row;
            copy_image_async(r->out.denoised.ptr, op, s.out_slot[slot], row, row, s.h, cudaMemcpyDeviceToHost, sv->s_d2h);
            s.frames++;
            r->t_launch = tl;
            r->batch_size = uint32_t(batch.size());
        }
        cudaEventRecord(fl->ev_d2h, sv->s_d2h);
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            sv->n_launches++;
            sv->max_batch_seen = std::max<uint32_t>(sv->max_batch_seen, uint32_t(batch.size()));
            sv->inflight.push_back(fl);
        }
        sv->cv_flight.notify_one();
        batch_no++;
    }
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->sched_done = true;
    }
    sv->cv_flight.notify_all();
}

void completer(tg_svgf_server* sv)
{
    cudaSetDevice(sv->device);
    for (;;) {
        Flight* fl = nullptr;
        {
            std::unique_lock<std::mutex> lk(sv->mu);
            sv->cv_flight.wait(lk, [&] { return !sv->inflight.empty() || sv->sched_done; });
            if (sv->inflight.empty()) break;
            fl = sv->inflight.front();
        }
        const cudaError_t e = cudaEventSynchronize(fl->ev_d2h);
        int status = (e == cudaSuccess && !fl->launch_failed) ? TG_OK : TG_ERR_CUDA;
        if (status == TG_OK && fl->table_k >= 0 && sv->h_err[fl->table_k]) {
            sv->h_err[fl->table_k] = 0;
            status = TG_ERR_TIMEOUT;
        }
        const Clock::time_point now = Clock::now();
        {
            std::lock_guard<std::mutex> lk(sv->mu);
            for (Sess* s : fl->sess) s->running--;
            for (Req* r : fl->reqs) {
                finish(sv, r, status, now);
                Sess& s = sv->sess[r->session];
                s.pending--;
                s.lru = ++sv->lru_tick;
                if (s.ended && s.pending == 0) {
                    release(sv, s);
                    sv->sess.erase(r->session);
                }
            }
            sv->inflight.pop_front();
            sv->ev_pool.push_back(fl->ev_comp);
            sv->ev_pool.push_back(fl->ev_d2h);
        }
        delete fl;
        sv->cv_done.notify_all();
        sv->cv_work.notify_all();
    }
}

void teardown(tg_svgf_server* sv)
{
    for (auto& e : sv->exec)
        if (e) cudaGraphExecDestroy(e);
    for (int k = 0; k < kMaxInflight; ++k) {
        if (sv->d_table[k]) cudaFree(sv->d_table[k]);
        if (sv->h_table[k]) cudaFreeHost(sv->h_table[k]);
    }
    for (cudaEvent_t e : sv->ev_pool) cudaEventDestroy(e);
    if (sv->h_err) cudaFreeHost(sv->h_err);
    if (sv->d_bar) cudaFree(sv->d_bar);
    if (sv->base) cudaFree(sv->base);
    cudaStream_t streams[4] = {sv->s_h2d, sv->s_comp, sv->s_d2h, sv->cap_stream};
    for (auto s : streams)
        if (s) cudaStreamDestroy(s);
    if (sv->ev_h2d) cudaEventDestroy(sv->ev_h2d);
    for (auto& kv : sv->reqs) delete kv.second;
}

} // namespace

extern "C" {

int tg_svgf_server_create(const tg_svgf_server_desc* d, tg_svgf_server** out)
{
    if (!d || !out) return fail(TG_ERR_INVALID, "null descriptor or output");
    *out = nullptr;
    if (d->params.mode != TG_SVGF_MODE_FULL) return fail(TG_ERR_INVALID, "the server runs the FULL mode");
    int st = validate_params(d->params);
    if (st) return st;
    if (d->max_batch < 1 || d->max_batch > TG_SVGF_BATCH_MAX_STREAMS)
        return fail(TG_ERR_INVALID, "max_batch must be 1..%d", TG_SVGF_BATCH_MAX_STREAMS);
    if (d->max_sessions < 1) return fail(TG_ERR_INVALID, "max_sessions must be positive");
    if (d->hbm_budget_bytes < (64u << 10)) return fail(TG_ERR_INVALID, "hbm_budget_bytes below 64 KiB");
    int dev = d->device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(TG_ERR_CUDA, "no current CUDA device");
    if (cudaSetDevice(dev) != cudaSuccess) return fail(TG_ERR_CUDA, "CUDA device %d unavailable", dev);
    tg_svgf_server* sv = new (std::nothrow) tg_svgf_server();
    if (!sv) return fail(TG_ERR_OOM, "host allocation failed");
    sv->d = *d;
    sv->device = dev;
    sv->f16 = d->params.storage == TG_SVGF_STORAGE_FP16;
    cudaDeviceGetAttribute(&sv->sm_count, cudaDevAttrMultiProcessorCount, dev);
    auto bail = [&](int status) {
        teardown(sv);
        delete sv;
        return status;
    };
    if (cudaMalloc(&sv->base, d->hbm_budget_bytes) != cudaSuccess) {
        cudaGetLastError();
        sv->base = nullptr;
        return bail(fail(TG_ERR_OOM, "cudaMalloc of the %llu-byte session budget failed",
                         (unsigned long long)d->hbm_budget_bytes));
    }
    sv->arena.reset(d->hbm_budget_bytes);
    if (cudaStreamCreateWithFlags(&sv->s_h2d, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&sv->s_comp, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&sv->s_d2h, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&sv->cap_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&sv->ev_h2d, cudaEventDisableTiming) != cudaSuccess)
        return bail(fail(TG_ERR_CUDA, "stream creation failed"));
    if (d->strategy != TG_SVGF_BATCH_STAGES && d->strategy != TG_SVGF_BATCH_PERSISTENT)
        return bail(fail(TG_ERR_INVALID, "strategy %d unknown", d->strategy));
    if (d->batching) {
        int coop = 0;
        cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
        if (!coop) return bail(fail(TG_ERR_UNSUPPORTED, "device cannot launch cooperative kernels"));
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, step_kernel(sv->f16), kLvTX * kLvRows, 0) !=
                cudaSuccess ||
            nb < 1)
            return bail(fail(TG_ERR_CUDA, "persistent kernel cannot be resident"));
        sv->grid = nb * sv->sm_count;
        sv->cap = int(d->max_batch);
        sv->tbytes = table_bytes(sv->cap);
        for (int k = 0; k < kMaxInflight; ++k)
            if (cudaMalloc(&sv->d_table[k], sv->tbytes) != cudaSuccess ||
                cudaHostAlloc(reinterpret_cast<void**>(&sv->h_table[k]), sv->tbytes, cudaHostAllocDefault) !=
                    cudaSuccess)
                return bail(fail(TG_ERR_OOM, "work table allocation failed"));
        if (cudaHostAlloc(reinterpret_cast<void**>(&sv->h_err), kMaxInflight * sizeof(int), cudaHostAllocDefault) !=
                cudaSuccess ||
            cudaMalloc(&sv->d_bar, sizeof(BarrierState)) != cudaSuccess)
            return bail(fail(TG_ERR_OOM, "barrier allocation failed"));
        for (int k = 0; k < kMaxInflight; ++k) sv->h_err[k] = 0;
    }
    if (cudaDeviceSynchronize() != cudaSuccess) return bail(fail(TG_ERR_CUDA, "server initialisation failed"));
    try {
        sv->sched = std::thread(scheduler, sv);
        sv->compl_thread = std::thread(completer, sv);
    } catch (...) {
        return bail(fail(TG_ERR_OOM, "thread creation failed"));
    }
    *out = sv;
    return TG_OK;
}

int tg_svgf_server_submit(tg_svgf_server* sv, uint64_t session, uint32_t width, uint32_t height,
                          const tg_svgf_inputs* in, const tg_svgf_outputs* out, uint64_t* ticket)
{
    if (!sv || !in || !out || !ticket) return fail(TG_ERR_INVALID, "null argument");
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(TG_ERR_INVALID, "size %ux%u outside 1..32768", width, height);
    static const int rad[] = {TG_FMT_RGBA32F, TG_FMT_RGBA16F};
    static const int dep[] = {TG_FMT_R32F};
    static const int nrm[] = {TG_FMT_RGB32F, TG_FMT_RGBA32F, TG_FMT_OCT16};
    static const int mot[] = {TG_FMT_RG32F, TG_FMT_RG16F};
    int st;
    if ((st = check_image("radiance", in->radiance, width, height, rad, 2))) return st;
    if ((st = check_image("depth", in->depth, width, height, dep, 1))) return st;
    if ((st = check_image("normal", in->normal, width, height, nrm, 3))) return st;
    if ((st = check_image("motion", in->motion, width, height, mot, 2))) return st;
    if ((st = check_image("denoised", out->denoised, width, height, rad, 2))) return st;
    Req* r = new (std::nothrow) Req();
    if (!r) return fail(TG_ERR_OOM, "host allocation failed");
    r->session = session;
    r->w = width;
    r->h = height;
    r->in = *in;
    r->out = *out;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        if (sv->stop) {
            delete r;
            return fail(TG_ERR_STATE, "server is shutting down");
        }
        auto it = sv->sess.find(session);
        if (it == sv->sess.end()) {
            if (sv->sess.size() >= sv->d.max_sessions) {
                // forget the least recently used idle, non-resident or evictable session record
                Sess* victim = nullptr;
                for (auto& kv : sv->sess)
                    if (kv.second.pending == 0 && (!victim || kv.second.lru < victim->lru)) victim = &kv.second;
                if (!victim) {
                    delete r;
                    return fail(TG_ERR_BUDGET, "max_sessions sessions are all busy");
                }
                if (victim->resident) sv->evictions++;
                release(sv, *victim);
                sv->sess.erase(victim->id);
            }
            Sess s;
            s.id = session;
            it = sv->sess.emplace(session, s).first;
        }
        it->second.pending++;
        r->ticket = sv->next_ticket++;
        sv->reqs[r->ticket] = r;
        sv->queue.push_back(r);
        sv->submitted++;
        if (!sv->have_first) {
            sv->t_first = r->t_submit;
            sv->have_first = true;
        }
        *ticket = r->ticket;
    }
    sv->cv_work.notify_one();
    return TG_OK;
}

int tg_svgf_server_wait(tg_svgf_server* sv, uint64_t ticket, int64_t timeout_us, tg_svgf_request_info* info)
{
    if (!sv) return fail(TG_ERR_INVALID, "null server");
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return fail(TG_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    Req* r = it->second;
    auto done = [&] { return r->status != -1; };
    if (timeout_us < 0)
        sv->cv_done.wait(lk, done);
    else if (!sv->cv_done.wait_for(lk, std::chrono::microseconds(timeout_us), done))
        return fail(TG_ERR_TIMEOUT, "ticket %llu not complete", (unsigned long long)ticket);
    if (info) {
        info->status = r->status;
        info->batch_size = r->batch_size;
        info->latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
        info->queue_ms = r->status == TG_OK ? std::chrono::duration<double, std::milli>(r->t_launch - r->t_submit).count()
                                            : 0.0;
    }
    sv->reqs.erase(it);
    delete r;
    return TG_OK;
}

int tg_svgf_server_end_session(tg_svgf_server* sv, uint64_t session)
{
    if (!sv) return fail(TG_ERR_INVALID, "null server");
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        auto it = sv->sess.find(session);
        if (it == sv->sess.end()) return fail(TG_ERR_INVALID, "unknown session %llu", (unsigned long long)session);
        it->second.ended = true;
        if (it->second.pending == 0) {
            release(sv, it->second);
            sv->sess.erase(it);
        }
    }
    sv->cv_work.notify_one();
    return TG_OK;
}

int tg_svgf_server_get_stats(tg_svgf_server* sv, tg_svgf_server_stats* o, int reset)
{
    if (!sv || !o) return fail(TG_ERR_INVALID, "null argument");
    std::lock_guard<std::mutex> lk(sv->mu);
    std::memset(o, 0, sizeof *o);
    o->submitted = sv->submitted;
    o->completed = sv->completed;
    o->failed = sv->failed;
    o->admissions = sv->admissions;
    o->evictions = sv->evictions;
    o->launches = sv->n_launches;
    o->resident_bytes = sv->arena.used();
    o->peak_resident_bytes = sv->peak_resident;
    o->max_batch_seen = sv->max_batch_seen;
    for (auto& kv : sv->sess) o->resident_sessions += kv.second.resident ? 1 : 0;
    if (!sv->lat.empty()) {
        std::vector<float> v = sv->lat;
        std::sort(v.begin(), v.end());
        o->p50_ms = v[v.size() / 2];
        o->p99_ms = v[std::min(v.size() - 1, size_t(0.99 * v.size()))];
        double sum = 0;
        for (float x : v) sum += x;
        o->mean_ms = sum / v.size();
    }
    if (sv->have_first && sv->completed) {
        o->wall_s = std::chrono::duration<double>(sv->t_last - sv->t_first).count();
        o->mpx_per_s = o->wall_s > 0 ? sv->px_done / o->wall_s / 1e6 : 0.0;
    }
    if (reset) {
        sv->lat.clear();
        sv->px_done = 0;
        sv->have_first = false;
        sv->submitted = sv->completed = sv->failed = sv->admissions = sv->evictions = sv->n_launches = 0;
        sv->max_batch_seen = 0;
        sv->peak_resident = sv->arena.used();
    }
    return TG_OK;
}

void tg_svgf_server_destroy(tg_svgf_server* sv)
{
    if (!sv) return;
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
    }
    sv->cv_work.notify_all();
    if (sv->sched.joinable()) sv->sched.join();
    sv->cv_flight.notify_all();
    if (sv->compl_thread.joinable()) sv->compl_thread.join();
    cudaSetDevice(sv->device);
    cudaDeviceSynchronize();
    teardown(sv);
    delete sv;
}

} // extern "C"
