// C ABI of the single-stream SVGF denoiser (include/tg_svgf.h).
//
// The handle replaces the reference's seven engine-owned images and their
// frame-parity descriptor sets (src/main.cpp:1326-1397, :2401-2446): it owns
// the ping-pong state (REF_EXACT: moments; FULL: guide, colour history,
// moments) and the per-frame scratch, all in one device allocation each, and
// alternates the ping-pong halves by frame parity exactly as the reference
// alternates descriptor sets.
#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "svgf_internal.h"
#include "svgf_kernels.cuh"
#include "svgf_level.cuh"

using namespace tg;

namespace tg {

thread_local std::string g_last_error;

int fail(int status, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_last_error = buf;
    return status;
}

int fmt_bytes(int fmt)
{
    switch (fmt) {
    case TG_FMT_RGBA32F: return 16;
    case TG_FMT_RGBA16F: return 8;
    case TG_FMT_R32F: return 4;
    case TG_FMT_RGB32F: return 12;
    case TG_FMT_OCT16: return 4;
    case TG_FMT_RG32F: return 8;
    case TG_FMT_RG16F: return 4;
    case TG_FMT_RGBA8: return 4;
    case TG_FMT_BGRA8: return 4;
    default: return 0;
    }
}

static int fmt_align(int fmt)
{
    switch (fmt) {
    case TG_FMT_RGBA32F: return 16;
    case TG_FMT_RGBA16F: return 8;
    case TG_FMT_RG32F: return 8;
    default: return 4;
    }
}

int check_image(const char* what, const tg_image& im, uint32_t w, uint32_t h, const int* allowed, int n_allowed)
{
    bool ok = false;
    for (int k = 0; k < n_allowed; ++k) ok |= im.format == allowed[k];
    if (!ok) return fail(TG_ERR_INVALID, "%s: unsupported format %d", what, im.format);
    if (!im.ptr) return fail(TG_ERR_INVALID, "%s: null pointer", what);
    const int64_t bpp = fmt_bytes(im.format);
    const int64_t pitch = im.pitch_bytes ? im.pitch_bytes : bpp * int64_t(w);
    const int al = fmt_align(im.format);
    if (pitch < bpp * int64_t(w)) return fail(TG_ERR_INVALID, "%s: pitch %lld below row size", what, (long long)pitch);
    if ((reinterpret_cast<uintptr_t>(im.ptr) % al) != 0 || (pitch % al) != 0)
        return fail(TG_ERR_INVALID, "%s: address and pitch must be multiples of %d bytes", what, al);
    (void)h;
    return TG_OK;
}

Img to_img(const tg_image& im, uint32_t w)
{
    Img r;
    r.ptr = static_cast<char*>(im.ptr);
    r.pitch = im.pitch_bytes ? im.pitch_bytes : int64_t(fmt_bytes(im.format)) * w;
    r.fmt = im.format;
    r.pad = 0;
    return r;
}

int sigma_n_squarings(float sigma_n)
{
    for (int k = 0; k <= 10; ++k)
        if (sigma_n == float(1 << k)) return k;
    return -1;
}

static size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Bytes per pixel of each handle-owned buffer.
struct Layout {
    size_t guide, c4, mom, rec;
};

static Layout layout_of(const tg_svgf_params& p)
{
    const bool f16 = p.storage == TG_SVGF_STORAGE_FP16;
    Layout l;
    l.guide = f16 ? 8 : 16;
    l.c4 = f16 ? 8 : 16;
    l.mom = f16 ? 4 : 8;
    // a-trous scratch: FULL records carry the guide and stay float32 in both storage forms (32 B), REF_EXACT
    // images are the reference's own formats
    l.rec = p.mode == TG_SVGF_MODE_FULL ? 32 : l.c4;
    return l;
}

size_t rec_bytes_of(const tg_svgf_params& p) { return layout_of(p).rec; }

size_t state_bytes_of(const tg_svgf_params& p, uint32_t w, uint32_t h)
{
    const size_t n = size_t(w) * h;
    const Layout l = layout_of(p);
    if (p.mode == TG_SVGF_MODE_REF_EXACT) return 2 * align_up(n * l.mom, 256);
    return 2 * (align_up(n * l.guide, 256) + align_up(n * l.c4, 256) + align_up(n * l.mom, 256));
}

// Pixels of one a-trous scratch buffer: the largest residue-major layout any
// level reads or writes (strides 1 .. 2^(levels-1)).
size_t col_pixels_of(const tg_svgf_params& p, uint32_t w, uint32_t h)
{
    size_t n = 0;
    for (int lg = 0; lg < p.levels; ++lg) {
        const size_t s = size_t(1) << lg;
        const size_t m = s * s * ((w + s - 1) / s) * ((h + s - 1) / s);
        n = m > n ? m : n;
    }
    return n;
}

size_t col_guide_half_of(const tg_svgf_params& p, uint32_t w, uint32_t h) { return col_pixels_of(p, w, h); }

size_t col_var_offset_of(const tg_svgf_params& p, uint32_t w, uint32_t h)
{
    return align_up(col_pixels_of(p, w, h) * layout_of(p).rec, 256);
}

size_t col_bytes_of(const tg_svgf_params& p, uint32_t w, uint32_t h)
{
    const size_t recs = col_var_offset_of(p, w, h);
    if (p.mode == TG_SVGF_MODE_REF_EXACT) return recs;
    return recs + align_up(col_pixels_of(p, w, h) * sizeof(float), 256);
}

size_t fb_flags_bytes_of(uint32_t w, uint32_t h)
{
    return size_t((w + kBlockX - 1) / kBlockX) * ((h + kBlockY - 1) / kBlockY) * sizeof(int);
}

size_t scratch_bytes_of(const tg_svgf_params& p, uint32_t w, uint32_t h)
{
    const size_t n = size_t(w) * h;
    const Layout l = layout_of(p);
    const size_t col = col_bytes_of(p, w, h);
    if (p.mode == TG_SVGF_MODE_REF_EXACT) return 2 * col + 256;  // + the device error word
    return align_up(n * l.c4, 256) + 2 * col + align_up(n * sizeof(float) * 2, 256) + align_up(fb_flags_bytes_of(w, h), 256) +
           256;
}

int validate_params(const tg_svgf_params& p)
{
    if (p.mode != TG_SVGF_MODE_REF_EXACT && p.mode != TG_SVGF_MODE_FULL)
        return fail(TG_ERR_INVALID, "params.mode %d unknown", p.mode);
    if (p.storage != TG_SVGF_STORAGE_FP32 && p.storage != TG_SVGF_STORAGE_FP16)
        return fail(TG_ERR_INVALID, "params.storage %d unknown", p.storage);
    if (p.levels < 1 || p.levels > 10) return fail(TG_ERR_INVALID, "params.levels %d outside 1..10", p.levels);
    if (p.mode == TG_SVGF_MODE_FULL) {
        if (p.max_history < 1) return fail(TG_ERR_INVALID, "params.max_history must be >= 1");
        if (!(p.alpha > 0.0f && p.alpha <= 1.0f)) return fail(TG_ERR_INVALID, "params.alpha outside (0, 1]");
        if (!(p.moments_alpha > 0.0f && p.moments_alpha <= 1.0f))
            return fail(TG_ERR_INVALID, "params.moments_alpha outside (0, 1]");
        if (!(p.sigma_l > 0.0f) || !(p.sigma_n > 0.0f) || !(p.sigma_z > 0.0f))
            return fail(TG_ERR_INVALID, "params.sigma_* must be positive");
    } else {
        if (!(p.moments_alpha >= 0.0f && p.moments_alpha <= 1.0f))
            return fail(TG_ERR_INVALID, "params.moments_alpha outside [0, 1]");
        if (!(p.variance_epsilon > 0.0f)) return fail(TG_ERR_INVALID, "params.variance_epsilon must be positive");
    }
    return TG_OK;
}

} // namespace tg

namespace tg {
// Output rows per thread of the tiled a-trous kernels: FULL (kLevelR) and
// REF_EXACT (kRefR).
constexpr int kLevelR = 2;
#ifndef TG_REF_R
#define TG_REF_R 2
#endif
constexpr int kRefR = TG_REF_R;

typedef void (*LevelTmaFn)(FullArgs, LevelArgs, LevelGeom, const CUtensorMap, const CUtensorMap);
typedef void (*LevelTiledFn)(FullArgs, LevelGeom);

// The FULL a-trous kernel for a level: FP16 or FP32 storage, VAR = false at the
// last level (it writes only colour), PL at level 0 (staged from the planes).
template <bool PL> LevelTmaFn level_tma_kernel(bool f16, bool last)
{
    if (f16) return last ? k_full_level_tma<ST_FP16, kLevelR, false, PL> : k_full_level_tma<ST_FP16, kLevelR, true, PL>;
    return last ? k_full_level_tma<ST_FP32, kLevelR, false, PL> : k_full_level_tma<ST_FP32, kLevelR, true, PL>;
}
template <bool PL> LevelTiledFn level_tiled_kernel(bool f16, bool last)
{
    if (f16) return last ? k_full_level_tiled<ST_FP16, kLevelR, false, PL> : k_full_level_tiled<ST_FP16, kLevelR, true, PL>;
    return last ? k_full_level_tiled<ST_FP32, kLevelR, false, PL> : k_full_level_tiled<ST_FP32, kLevelR, true, PL>;
}
enum Family { F_REF_FIRST = 0, F_REF_LEVEL, F_FULL_TEMPORAL, F_FULL_VARIANCE, F_FULL_LEVEL, kFamilies };
static const char* kFamilyName[kFamilies] = {"ref_first", "ref_level", "full_temporal", "full_variance", "full_level"};
} // namespace tg

struct tg_svgf {
    int device = 0;
    int sms = 1;  // multiprocessors of the device
    uint32_t w = 0, h = 0;
    tg_svgf_params p{};
    uint64_t frame = 0;
    char* state = nullptr;
    char* scratch = nullptr;
    size_t state_bytes = 0, scratch_bytes = 0;
    // carved views
    void* guide[2] = {nullptr, nullptr};
    void* hist[2] = {nullptr, nullptr};
    void* mom[2] = {nullptr, nullptr};
    void* tc = nullptr;
    void* colA = nullptr;
    void* colB = nullptr;
    float2* grad = nullptr;
    int* fb_flags = nullptr;
    int* d_err = nullptr;  // device error word of bounded waits
    int flags = 0;
    bool tma = false;                // a-trous tiles staged by TMA
    CUtensorMap tmaps[10];           // per level: the level's input records
    bool tma0 = false;               // level 0 staged by TMA from the tc and guide planes
    CUtensorMap tm_tc, tm_guide[2];  // row-major tc and guide[parity] (level 0 reads these, not records)
    // REF_EXACT: maps over each later pass's input planes, and over the caller's radiance (re-encoded when the
    // caller's buffer, pitch or format changes)
    bool ref_lv_ok[10] = {};
    CUtensorMap ref_lv[10];
    bool ref_in_ok = false;
    const void* ref_in_ptr = nullptr;
    int64_t ref_in_pitch = 0;
    int32_t ref_in_fmt = -1;
    CUtensorMap ref_in;
    // host-call staging: a ring of three sets, so that a frame's upload never
    // waits for the download of the frame two before it
    static constexpr int kStaging = 3;
    struct Staging {
        char* buf = nullptr;
        size_t bytes = 0;
        cudaEvent_t ev_in = nullptr, ev_comp = nullptr, ev_done = nullptr;
        bool used = false;
    } stg[kStaging];
    int stg_next = 0;
    cudaStream_t copy_stream = nullptr;  // host -> device
    cudaStream_t d2h_stream = nullptr;   // device -> host (its own stream, so uploads never queue behind it)
    // per-kernel CUDA-event profiling
    struct Prof {
        bool on = false;
        struct Rec {
            int fam;
            double bytes;
            cudaEvent_t a, b;
        };
        std::vector<Rec> pending;
        std::vector<cudaEvent_t> pool;
        uint32_t launches[kFamilies] = {};
        double ms[kFamilies] = {};
        double bytes[kFamilies] = {};
    } prof;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    bool switched = false;
    explicit DeviceGuard(int dev)
    {
        if (cudaGetDevice(&prev) == cudaSuccess && prev != dev) switched = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard()
    {
        if (switched) cudaSetDevice(prev);
    }
};

void carve(tg_svgf* s)
{
    const size_t n = size_t(s->w) * s->h;
    const Layout l = layout_of(s->p);
    char* p = s->state;
    auto take = [&](size_t bytes) {
        void* r = p;
        p += align_up(bytes, 256);
        return r;
    };
    if (s->p.mode == TG_SVGF_MODE_REF_EXACT) {
        s->mom[0] = take(n * l.mom);
        s->mom[1] = take(n * l.mom);
        p = s->scratch;
        s->colA = take(col_pixels_of(s->p, s->w, s->h) * l.c4);
        s->colB = take(col_pixels_of(s->p, s->w, s->h) * l.c4);
        s->guide[0] = s->guide[1] = s->hist[0] = s->hist[1] = s->tc = nullptr;
        s->grad = nullptr;
        s->fb_flags = nullptr;
        s->d_err = static_cast<int*>(take(sizeof(int)));
    } else {
        for (int k = 0; k < 2; ++k) {
            s->guide[k] = take(n * l.guide);
            s->hist[k] = take(n * l.c4);
            s->mom[k] = take(n * l.mom);
        }
        p = s->scratch;
        s->tc = take(n * l.c4);
        s->colA = take(col_bytes_of(s->p, s->w, s->h));
        s->colB = take(col_bytes_of(s->p, s->w, s->h));
        s->grad = static_cast<float2*>(take(n * sizeof(float2)));
        s->fb_flags = static_cast<int*>(take(fb_flags_bytes_of(s->w, s->h)));
        s->d_err = static_cast<int*>(take(sizeof(int)));
    }
}

typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_tiled()
{
    static EncodeTiledFn fn = nullptr;
    static bool tried = false;
    if (!tried) {
        tried = true;
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
        cudaGetLastError();
    }
    return fn;
}

// One tensor map per a-trous level L >= 1 over that level's input records in
// the residue-major layout of stride 2^L: {float, row, plane, half-plane};
// box = one 36 x (4R + 4) halo tile, whose rows are contiguous lines.
// Level 0 has no records: its maps cover the tc and guide planes.
// REF_EXACT: a 3-D map {texel, row, plane} over pass L's input (residue-major
// planes of stride 2^L; 8-byte texels of fp16 images as UINT64, 16-byte ones as
// 4 floats), box = one 36 x (4R + 4) halo tile of one plane.  A level whose plane
// rows are not a multiple of 16 bytes stages with plain loads.
void build_ref_maps(tg_svgf* s, EncodeTiledFn enc)
{
    const bool f16 = s->p.storage == TG_SVGF_STORAGE_FP16;
    const uint64_t tb = f16 ? 8 : 16;
    for (int lv = 1; lv < s->p.levels && lv < 10; ++lv) {
        s->ref_lv_ok[lv] = false;
        const ResLayout L = res_layout(int(s->w), int(s->h), lv);
        if ((tb * L.pw) % 16 || (tb * L.pw * L.ph) % 16) continue;
        void* base = (lv & 1) ? s->colB : s->colA;  // pass 1 reads col B, pass 2 col A, ...
        const cuuint64_t planes = cuuint64_t(1) << (2 * lv);
        const cuuint64_t dim[3] = {f16 ? cuuint64_t(L.pw) : 4ull * L.pw, cuuint64_t(L.ph), planes};
        const cuuint64_t str[2] = {tb * L.pw, tb * L.pw * L.ph};
        const cuuint32_t box[3] = {f16 ? cuuint32_t(LevelTile<kRefR>::SW) : 4u * LevelTile<kRefR>::SW,
                                   LevelTile<kRefR>::SH, 1};
        const cuuint32_t es[3] = {1, 1, 1};
        const CUresult r = enc(&s->ref_lv[lv], f16 ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3,
                               base, dim, str, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        s->ref_lv_ok[lv] = r == CUDA_SUCCESS;
    }
}

// REF_EXACT: the 2-D map over the caller's radiance {texel, row} (RGBA16F as
// UINT64 texels, RGBA32F as 4 floats), re-encoded when the buffer, its pitch or
// its format changes; false (plain loads) when TMA cannot address it.
bool ref_input_map(tg_svgf* s, const tg_image& im)
{
    if (s->flags & TG_SVGF_FLAG_NO_TMA) return false;
    const int64_t tb = im.format == TG_FMT_RGBA16F ? 8 : 16;
    const int64_t pitch = im.pitch_bytes ? im.pitch_bytes : tb * int64_t(s->w);
    if (s->ref_in_ok && s->ref_in_ptr == im.ptr && s->ref_in_pitch == pitch && s->ref_in_fmt == im.format) return true;
    s->ref_in_ok = false;
    EncodeTiledFn enc = encode_tiled();
    if (!enc || (reinterpret_cast<uintptr_t>(im.ptr) % 16) || pitch % 16) return false;
    const bool h = tb == 8;
    const cuuint64_t dim[2] = {h ? cuuint64_t(s->w) : 4ull * s->w, s->h};
    const cuuint64_t str[1] = {cuuint64_t(pitch)};
    const cuuint32_t box[2] = {h ? cuuint32_t(LevelTile<kRefR>::SW) : 4u * LevelTile<kRefR>::SW,
                               LevelTile<kRefR>::SH};
    const cuuint32_t es[2] = {1, 1};
    if (enc(&s->ref_in, h ? CU_TENSOR_MAP_DATA_TYPE_UINT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, im.ptr, dim, str, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    s->ref_in_ok = true;
    s->ref_in_ptr = im.ptr;
    s->ref_in_pitch = pitch;
    s->ref_in_fmt = im.format;
    return true;
}

void build_tensor_maps(tg_svgf* s)
{
    s->tma = false;
    for (bool& ok : s->ref_lv_ok) ok = false;
    s->ref_in_ok = false;
    if (s->flags & TG_SVGF_FLAG_NO_TMA) return;
    EncodeTiledFn enc = encode_tiled();
    if (!enc) return;
    if (s->p.mode == TG_SVGF_MODE_REF_EXACT) {
        build_ref_maps(s, enc);
        s->tma = true;  // interior tiles of the later passes (where their planes allow) and of the first pass
        return;
    }
    CUtensorMap maps[kFullMaps];
    const unsigned m = full_level_maps(s->p, s->w, s->h, kLevelR, s->colA, s->colB, s->tc, s->guide[0], s->guide[1], maps);
    for (int lv = 1; lv < s->p.levels; ++lv) {
        if (!((m >> lv) & 1u)) return;
        s->tmaps[lv] = maps[2 + lv];
    }
    s->tma = true;
    s->tma0 = m & 1u;
    if (s->tma0) {
        s->tm_tc = maps[0];
        s->tm_guide[0] = maps[1];
        s->tm_guide[1] = maps[2];
    }
}

void free_buffers(tg_svgf* s)
{
    if (s->state) cudaFree(s->state);
    if (s->scratch) cudaFree(s->scratch);
    s->state = s->scratch = nullptr;
    s->state_bytes = s->scratch_bytes = 0;
}

void free_staging(tg_svgf* s)
{
    for (auto& g : s->stg) {
        if (g.buf) cudaFree(g.buf);
        if (g.ev_in) cudaEventDestroy(g.ev_in);
        if (g.ev_comp) cudaEventDestroy(g.ev_comp);
        if (g.ev_done) cudaEventDestroy(g.ev_done);
        g = tg_svgf::Staging{};
    }
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    if (s->d2h_stream) cudaStreamDestroy(s->d2h_stream);
    s->copy_stream = nullptr;
    s->d2h_stream = nullptr;
}

int alloc_buffers(tg_svgf* s)
{
    s->state_bytes = state_bytes_of(s->p, s->w, s->h);
    s->scratch_bytes = scratch_bytes_of(s->p, s->w, s->h);
    if (cudaMalloc(&s->state, s->state_bytes) != cudaSuccess) {
        cudaGetLastError();
        s->state = nullptr;
        return fail(TG_ERR_OOM, "cudaMalloc of %zu state bytes failed", s->state_bytes);
    }
    if (cudaMalloc(&s->scratch, s->scratch_bytes) != cudaSuccess) {
        cudaGetLastError();
        s->scratch = nullptr;
        free_buffers(s);
        return fail(TG_ERR_OOM, "cudaMalloc of %zu scratch bytes failed", s->scratch_bytes);
    }
    carve(s);
    build_tensor_maps(s);
    if (cudaMemset(s->state, 0, s->state_bytes) != cudaSuccess || cudaMemset(s->scratch, 0, s->scratch_bytes) != cudaSuccess ||
        cudaDeviceSynchronize() != cudaSuccess) {
        free_buffers(s);
        return fail(TG_ERR_CUDA, "zeroing the SVGF state failed: %s", cudaGetErrorString(cudaGetLastError()));
    }
    return TG_OK;
}

int check_inputs(const tg_svgf* s, const tg_svgf_inputs* in, const tg_svgf_outputs* out)
{
    if (!in || !out) return fail(TG_ERR_INVALID, "null inputs or outputs");
    static const int rad[] = {TG_FMT_RGBA32F, TG_FMT_RGBA16F};
    static const int dep[] = {TG_FMT_R32F};
    static const int nrm[] = {TG_FMT_RGB32F, TG_FMT_RGBA32F, TG_FMT_OCT16};
    static const int mot[] = {TG_FMT_RG32F, TG_FMT_RG16F};
    int st;
    if ((st = check_image("radiance", in->radiance, s->w, s->h, rad, 2))) return st;
    if ((st = check_image("denoised", out->denoised, s->w, s->h, rad, 2))) return st;
    if (s->p.mode == TG_SVGF_MODE_FULL) {
        if ((st = check_image("depth", in->depth, s->w, s->h, dep, 1))) return st;
        if ((st = check_image("normal", in->normal, s->w, s->h, nrm, 3))) return st;
        if ((st = check_image("motion", in->motion, s->w, s->h, mot, 2))) return st;
    }
    return TG_OK;
}

} // namespace

namespace tg {

// TMA maps of a FULL stream's a-trous levels for tiles of R output rows per
// thread (box = 36 x (4R + 4) cells); see svgf_internal.h for the layout and
// the mask.  Each map's preconditions (16-byte strides and base) are those of
// cuTensorMapEncodeTiled; a level whose map cannot be encoded stages with plain
// loads.
unsigned full_level_maps(const tg_svgf_params& p, uint32_t w, uint32_t h, int R, void* colA, void* colB, void* tc,
                         void* guide0, void* guide1, CUtensorMap* maps)
{
    EncodeTiledFn enc = encode_tiled();
    if (!enc || p.mode != TG_SVGF_MODE_FULL) return 0;
    const cuuint32_t SW = kLvTX + 4, SH = kLvRows * R + 4;
    const bool f16 = p.storage == TG_SVGF_STORAGE_FP16;
    unsigned mask = 0;
    for (int lv = 1; lv < p.levels && 2 + lv < kFullMaps; ++lv) {
        const ResLayout L = res_layout(int(w), int(h), lv);
        void* base = (lv & 1) ? colB : colA;  // level L reads the records level L-1 wrote
        const cuuint64_t planes = cuuint64_t(1) << (2 * lv);
        // a row of either half-plane as 4 pw floats: one contiguous line per tile row and half
        const cuuint64_t dim[4] = {4ull * L.pw, cuuint64_t(L.ph), planes, 2};
        const cuuint64_t str[3] = {16ull * L.pw, 16ull * L.pw * L.ph, 16ull * col_guide_half_of(p, w, h)};
        const cuuint32_t box[4] = {4 * SW, SH, 1, 1};
        const cuuint32_t es[4] = {1, 1, 1, 1};
        if (enc(&maps[2 + lv], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base, dim, str, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
            mask |= 1u << lv;
    }
    // Level 0's planes: FP32 {float, row}, FP16 {8-byte texel, row} (its row pitch must be a multiple of 16 bytes,
    // so an odd width stages level 0 with plain loads); each tile row is one contiguous line.
    if (f16 && (8ull * w) % 16) return mask;
    void* planes[3] = {tc, guide0, guide1};
    for (int k = 0; k < 3; ++k) {
        CUresult r;
        if (f16) {
            const cuuint64_t dim[2] = {w, h};
            const cuuint64_t str[1] = {8ull * w};
            const cuuint32_t box[2] = {SW, SH};
            const cuuint32_t es[2] = {1, 1};
            r = enc(&maps[k], CU_TENSOR_MAP_DATA_TYPE_UINT64, 2, planes[k], dim, str, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        } else {
            const cuuint64_t dim[2] = {4ull * w, h};
            const cuuint64_t str[1] = {16ull * w};
            const cuuint32_t box[2] = {4 * SW, SH};
            const cuuint32_t es[2] = {1, 1};
            r = enc(&maps[k], CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, planes[k], dim, str, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        }
        if (r != CUDA_SUCCESS) return mask;
    }
    return mask | 1u;
}


static cudaEvent_t prof_event(tg_svgf* s)
{
    cudaEvent_t e = nullptr;
    if (!s->prof.pool.empty()) {
        e = s->prof.pool.back();
        s->prof.pool.pop_back();
    } else if (cudaEventCreate(&e) != cudaSuccess) {
        e = nullptr;
    }
    return e;
}

// Launches `body` on `stream`, bracketed by an event pair when profiling.
template <class F> static void launch(tg_svgf* s, cudaStream_t stream, int fam, double bytes, F body)
{
    if (!s->prof.on) {
        body();
        return;
    }
    cudaEvent_t a = prof_event(s), b = prof_event(s);
    if (a) cudaEventRecord(a, stream);
    body();
    if (b) cudaEventRecord(b, stream);
    if (a && b) {
        s->prof.pending.push_back({fam, bytes, a, b});
    } else {
        if (a) s->prof.pool.push_back(a);
        if (b) s->prof.pool.push_back(b);
    }
}

// Enqueues one frame of the chain on `stream`.  Shared by the device and host
// entry points.
int launch_frame(tg_svgf* s, const tg_svgf_inputs* in, const tg_svgf_outputs* out, cudaStream_t stream)
{
    const dim3 blk(kBlockX, kBlockY);
    const dim3 grd((s->w + kBlockX - 1) / kBlockX, (s->h + kBlockY - 1) / kBlockY);
    const int cur = int(s->frame & 1u), prev = cur ^ 1;
    const bool f16 = s->p.storage == TG_SVGF_STORAGE_FP16;
    if (s->p.mode == TG_SVGF_MODE_REF_EXACT) {
        RefArgs a{};
        a.w = int(s->w);
        a.h = int(s->h);
        a.raw = to_img(in->radiance, s->w);
        a.out = to_img(out->denoised, s->w);
        a.mom_prev = s->mom[prev];
        a.mom_curr = s->mom[cur];
        a.phi = s->p.sigma_l;
        a.alpha_m = s->p.moments_alpha;
        a.var_eps = s->p.variance_epsilon;
        const double npx = double(s->w) * s->h;
        const double c4 = f16 ? 8 : 16, mm = f16 ? 4 : 8;
        const double rb = fmt_bytes(in->radiance.format), ob = fmt_bytes(out->denoised.format);
        const int levels = s->p.levels;
        int lv = 0;
        a.err = s->d_err;
        RefMaps maps;
        if (ref_input_map(s, in->radiance)) maps.first = &s->ref_in;
        for (int L = 1; L < levels && L < 10; ++L)
            if (s->ref_lv_ok[L]) maps.level[L] = &s->ref_lv[L];
        enqueue_ref_chain<kRefR>(a, s->colA, s->colB, levels, f16, stream, maps, [&](bool first, auto body) {
            const bool last = lv == levels - 1;
            // compulsory bytes: the fused pass reads radiance and moments_prev and writes moments_curr; every
            // pass reads its input image and writes its output (the caller's image at the last pass)
            const double bytes = npx * ((first ? rb + 2 * mm : c4) + (last ? ob : c4));
            launch(s, stream, first ? F_REF_FIRST : F_REF_LEVEL, bytes, body);
            ++lv;
        });
    } else {
        FullArgs a{};
        a.w = int(s->w);
        a.h = int(s->h);
        a.radiance = to_img(in->radiance, s->w);
        a.depth = to_img(in->depth, s->w);
        a.normal = to_img(in->normal, s->w);
        a.motion = to_img(in->motion, s->w);
        a.out = to_img(out->denoised, s->w);
        a.guide_prev = s->guide[prev];
        a.hist_prev = s->hist[prev];
        a.mom_prev = s->mom[prev];
        a.guide_cur = s->guide[cur];
        a.hist_cur = s->hist[cur];
        a.mom_cur = s->mom[cur];
        a.tc = s->tc;
        a.grad = s->grad;
        a.fb_flags = s->fb_flags;
        a.err = s->d_err;
        a.alpha = s->p.alpha;
        a.alpha_m = s->p.moments_alpha;
        a.sigma_l = s->p.sigma_l;
        a.sigma_n = s->p.sigma_n;
        a.sigma_z = s->p.sigma_z;
        a.sq_n = sigma_n_squarings(s->p.sigma_n);
        a.max_history = s->p.max_history;
        a.fallback_frames = s->p.fallback_frames;
        a.col_dst = s->colA;
        a.var_off = col_var_offset_of(s->p, s->w, s->h);
        a.ghalf = col_guide_half_of(s->p, s->w, s->h);
        const double npx = double(s->w) * s->h;
        const double gb = f16 ? 8 : 16, c4 = f16 ? 8 : 16, mm = f16 ? 4 : 8;
        const double inb = fmt_bytes(in->radiance.format) + fmt_bytes(in->depth.format) +
                           fmt_bytes(in->normal.format) + fmt_bytes(in->motion.format);
        const double ob = fmt_bytes(out->denoised.format);
        const double vb = 4;   // variance plane entry
        const double rb = 32;  // a-trous record
        // temporal: inputs + previous guide/history/moments, writes guide, tc, moments, depth gradient and
        // the variance plane entry (every pixel with a history of fallback_frames or more)
        launch(s, stream, F_FULL_TEMPORAL, npx * (inb + 2 * (gb + c4 + mm) + 8 + vb), [&] {
            launch_chain(f16 ? k_full_temporal<ST_FP16> : k_full_temporal<ST_FP32>, grd, blk, stream, a);
        });
        // variance: the block flags; the flagged blocks' short-history pixels (data-dependent, not counted)
        launch(s, stream, F_FULL_VARIANCE, double(fb_flags_bytes_of(s->w, s->h)), [&] {
            const int vg = variance_grid(int(grd.x * grd.y), s->sms);
            launch_chain(f16 ? k_full_variance<ST_FP16> : k_full_variance<ST_FP32>, dim3(vg), blk, stream, a);
        });
        void* src = s->colA;
        void* oth = s->colB;
        for (int lv = 0; lv < s->p.levels; ++lv) {
            a.col_src = src;
            a.col_dst = oth;
            a.level = lv;
            a.stride = 1 << lv;
            a.last = lv == s->p.levels - 1;
            a.lin = res_layout(a.w, a.h, lv);
            a.lout = res_layout(a.w, a.h, lv + 1);
            // level: records (colour, variance, guide), variance plane and depth gradient in, records and
            // variance plane (or the output) out; level 0 reads tc (colour and length), guide and variance
            // plane instead of records and also writes the history
            const double lb = (lv == 0 ? c4 + gb : rb) + vb + 8 + (a.last ? ob : rb + vb) + (lv == 0 ? c4 : 0);
            const LevelGeom lg = level_geom(a.w, a.h, a.stride, kLevelR);
            const dim3 lgrid(level_blocks(lg)), lblk(kLvTX, kLvRows);
            // the last level writes only colour: its kernels leave out the variance propagation
            launch(s, stream, F_FULL_LEVEL, npx * lb, [&] {
                const bool pl = lv == 0;
                if (s->tma && (!pl || s->tma0)) {
                    const LevelArgs la = level_args_of(a);
                    if (pl)
                        launch_chain(level_tma_kernel<true>(f16, a.last), lgrid, lblk, stream, a, la, lg, s->tm_tc,
                                     s->tm_guide[cur]);
                    else
                        launch_chain(level_tma_kernel<false>(f16, a.last), lgrid, lblk, stream, a, la, lg, s->tmaps[lv],
                                     s->tmaps[lv]);
                } else {
                    launch_chain(pl ? level_tiled_kernel<true>(f16, a.last) : level_tiled_kernel<false>(f16, a.last), lgrid,
                                 lblk, stream, a, lg);
                }
            });
            void* t = src;
            src = oth;
            oth = t;
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    s->frame++;
    return TG_OK;
}

} // namespace tg

extern "C" {

const char* tg_status_string(int status)
{
    switch (status) {
    case TG_OK: return "ok";
    case TG_ERR_INVALID: return "invalid argument";
    case TG_ERR_OOM: return "out of memory";
    case TG_ERR_CUDA: return "CUDA error";
    case TG_ERR_TIMEOUT: return "timeout";
    case TG_ERR_BUDGET: return "over HBM budget";
    case TG_ERR_UNSUPPORTED: return "unsupported";
    case TG_ERR_STATE: return "invalid state";
    default: return "unknown status";
    }
}

const char* tg_last_error(void) { return g_last_error.c_str(); }

int tg_svgf_params_default(int32_t mode, int32_t storage, tg_svgf_params* out)
{
    if (!out) return fail(TG_ERR_INVALID, "null params");
    if (mode != TG_SVGF_MODE_REF_EXACT && mode != TG_SVGF_MODE_FULL) return fail(TG_ERR_INVALID, "mode %d unknown", mode);
    if (storage != TG_SVGF_STORAGE_FP32 && storage != TG_SVGF_STORAGE_FP16)
        return fail(TG_ERR_INVALID, "storage %d unknown", storage);
    std::memset(out, 0, sizeof *out);
    out->mode = mode;
    out->storage = storage;
    if (mode == TG_SVGF_MODE_REF_EXACT) {
        // src/svgf_denoise.slang:137 (SIGMA_COLOR_BASE), :144 (ALPHA_MOMENTS),
        // :150 (VARIANCE_EPSILON); src/main.cpp:929 (three wavelet passes).
        out->levels = 3;
        out->sigma_l = 2.0f;
        out->moments_alpha = 0.2f;
        out->variance_epsilon = 1e-4f;
        out->alpha = 1.0f;
        out->max_history = 1;
        out->fallback_frames = 0;
        out->sigma_n = 1.0f;
        out->sigma_z = 1.0f;
    } else {
        out->levels = 5;
        out->alpha = 0.2f;
        out->moments_alpha = 0.2f;
        out->sigma_l = 4.0f;
        out->sigma_n = 128.0f;
        out->sigma_z = 1.0f;
        out->max_history = 32;
        out->fallback_frames = 4;
        out->variance_epsilon = 1e-4f;
    }
    return TG_OK;
}

uint64_t tg_svgf_state_bytes(const tg_svgf_params* params, uint32_t width, uint32_t height)
{
    if (!params) return 0;
    return state_bytes_of(*params, width, height);
}

int tg_svgf_create(const tg_svgf_desc* desc, tg_svgf** out)
{
    if (!desc || !out) return fail(TG_ERR_INVALID, "null descriptor or output handle");
    *out = nullptr;
    if (desc->width == 0 || desc->height == 0 || desc->width > 32768 || desc->height > 32768)
        return fail(TG_ERR_INVALID, "size %ux%u outside 1..32768", desc->width, desc->height);
    int st = validate_params(desc->params);
    if (st) return st;
    int dev = desc->device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(TG_ERR_CUDA, "no current CUDA device");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || dev >= ndev) {
        cudaGetLastError();
        return fail(TG_ERR_CUDA, "CUDA device %d unavailable", dev);
    }
    DeviceGuard g(dev);
    tg_svgf* s = new (std::nothrow) tg_svgf();
    if (!s) return fail(TG_ERR_OOM, "host allocation failed");
    s->device = dev;
    cudaDeviceGetAttribute(&s->sms, cudaDevAttrMultiProcessorCount, dev);
    if (s->sms < 1) s->sms = 1;
    s->w = desc->width;
    s->h = desc->height;
    s->p = desc->params;
    s->flags = desc->flags;
    st = alloc_buffers(s);
    if (st) {
        delete s;
        return st;
    }
    *out = s;
    return TG_OK;
}

int tg_svgf_denoise(tg_svgf* s, const tg_svgf_inputs* in, const tg_svgf_outputs* out, void* stream)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    int st = check_inputs(s, in, out);
    if (st) return st;
    DeviceGuard g(s->device);
    return launch_frame(s, in, out, static_cast<cudaStream_t>(stream));
}

int tg_svgf_denoise_host(tg_svgf* s, const tg_svgf_inputs* in, const tg_svgf_outputs* out, void* stream_v)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    int st = check_inputs(s, in, out);
    if (st) return st;
    DeviceGuard g(s->device);
    cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
    const bool full = s->p.mode == TG_SVGF_MODE_FULL;
    const tg_image* src_imgs[4] = {&in->radiance, &in->depth, &in->normal, &in->motion};
    const int n_in = full ? 4 : 1;
    size_t off[5], need = 0;
    for (int k = 0; k < n_in; ++k) {
        off[k] = need;
        need += align_up(size_t(fmt_bytes(src_imgs[k]->format)) * s->w * s->h, 256);
    }
    off[4] = need;
    need += align_up(size_t(fmt_bytes(out->denoised.format)) * s->w * s->h, 256);
    if (!s->copy_stream && cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(TG_ERR_CUDA, "copy stream creation failed");
    if (!s->d2h_stream && cudaStreamCreateWithFlags(&s->d2h_stream, cudaStreamNonBlocking) != cudaSuccess)
        return fail(TG_ERR_CUDA, "copy stream creation failed");
    tg_svgf::Staging& sg = s->stg[s->stg_next];
    if (sg.bytes < need) {
        if (sg.buf) {
            // The previous use of this buffer must be finished before it is freed.
            if (sg.used && cudaEventSynchronize(sg.ev_done) != cudaSuccess)
                return fail(TG_ERR_CUDA, "staging wait failed");
            cudaFree(sg.buf);
            sg.buf = nullptr;
            sg.bytes = 0;
        }
        if (cudaMalloc(&sg.buf, need) != cudaSuccess) {
            cudaGetLastError();
            sg.buf = nullptr;
            return fail(TG_ERR_OOM, "cudaMalloc of %zu staging bytes failed", need);
        }
        sg.bytes = need;
        sg.used = false;
    }
    if (!sg.ev_in) {
        if (cudaEventCreateWithFlags(&sg.ev_in, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&sg.ev_comp, cudaEventDisableTiming) != cudaSuccess ||
            cudaEventCreateWithFlags(&sg.ev_done, cudaEventDisableTiming) != cudaSuccess)
            return fail(TG_ERR_CUDA, "event creation failed");
    }
    // H2D on the copy stream, after the previous user of this staging set has
    // finished copying its result out.
    if (sg.used && cudaStreamWaitEvent(s->copy_stream, sg.ev_done, 0) != cudaSuccess)
        return fail(TG_ERR_CUDA, "stream wait failed");
    tg_svgf_inputs din{};
    tg_image* dst_imgs[4] = {&din.radiance, &din.depth, &din.normal, &din.motion};
    for (int k = 0; k < n_in; ++k) {
        const tg_image& hi = *src_imgs[k];
        const size_t row = size_t(fmt_bytes(hi.format)) * s->w;
        const size_t hp = hi.pitch_bytes ? size_t(hi.pitch_bytes) : row;
        *dst_imgs[k] = tg_image{sg.buf + off[k], int64_t(row), hi.format, 0};
        const cudaError_t ce =
            copy_image_async(sg.buf + off[k], row, hi.ptr, hp, row, s->h, cudaMemcpyHostToDevice, s->copy_stream);
        if (ce != cudaSuccess) return fail(TG_ERR_CUDA, "input copy failed: %s", cudaGetErrorString(cudaGetLastError()));
    }
    if (cudaEventRecord(sg.ev_in, s->copy_stream) != cudaSuccess || cudaStreamWaitEvent(stream, sg.ev_in, 0) != cudaSuccess)
        return fail(TG_ERR_CUDA, "event record failed");
    const size_t orow = size_t(fmt_bytes(out->denoised.format)) * s->w;
    tg_svgf_outputs dout{};
    dout.denoised = tg_image{sg.buf + off[4], int64_t(orow), out->denoised.format, 0};
    st = launch_frame(s, &din, &dout, stream);
    if (st) return st;
    if (cudaEventRecord(sg.ev_comp, stream) != cudaSuccess || cudaStreamWaitEvent(s->d2h_stream, sg.ev_comp, 0) != cudaSuccess)
        return fail(TG_ERR_CUDA, "event record failed");
    const size_t op = out->denoised.pitch_bytes ? size_t(out->denoised.pitch_bytes) : orow;
    const cudaError_t oe =
        copy_image_async(out->denoised.ptr, op, sg.buf + off[4], orow, orow, s->h, cudaMemcpyDeviceToHost, s->d2h_stream);
    if (oe != cudaSuccess) return fail(TG_ERR_CUDA, "output copy failed: %s", cudaGetErrorString(cudaGetLastError()));
    if (cudaEventRecord(sg.ev_done, s->d2h_stream) != cudaSuccess) return fail(TG_ERR_CUDA, "event record failed");
    sg.used = true;
    s->stg_next = (s->stg_next + 1) % tg_svgf::kStaging;
    return TG_OK;
}

static int read_err(const tg_svgf* s, int* v)
{
    *v = 0;
    if (!s->d_err) return TG_OK;
    if (cudaMemcpy(v, s->d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
        return fail(TG_ERR_CUDA, "error word read failed: %s", cudaGetErrorString(cudaGetLastError()));
    return TG_OK;
}

int tg_svgf_synchronize(tg_svgf* s)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    DeviceGuard g(s->device);
    for (auto& sg : s->stg)
        if (sg.used && cudaEventSynchronize(sg.ev_done) != cudaSuccess)
            return fail(TG_ERR_CUDA, "synchronize failed: %s", cudaGetErrorString(cudaGetLastError()));
    int e = 0;
    int st = read_err(s, &e);
    if (st) return st;
    if (e) return fail(TG_ERR_TIMEOUT, "a bounded device-side wait gave up; results since are invalid");
    return TG_OK;
}

int tg_svgf_reset(tg_svgf* s, void* stream)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    DeviceGuard g(s->device);
    if (cudaMemsetAsync(s->state, 0, s->state_bytes, static_cast<cudaStream_t>(stream)) != cudaSuccess)
        return fail(TG_ERR_CUDA, "reset failed: %s", cudaGetErrorString(cudaGetLastError()));
    s->frame = 0;
    return TG_OK;
}

int tg_svgf_resize(tg_svgf* s, uint32_t width, uint32_t height)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(TG_ERR_INVALID, "size %ux%u outside 1..32768", width, height);
    DeviceGuard g(s->device);
    if (cudaDeviceSynchronize() != cudaSuccess) return fail(TG_ERR_CUDA, "synchronize failed");
    free_buffers(s);
    free_staging(s);
    s->w = width;
    s->h = height;
    s->frame = 0;
    return alloc_buffers(s);
}

int tg_svgf_get_info(const tg_svgf* s, tg_svgf_info* info)
{
    if (!s || !info) return fail(TG_ERR_INVALID, "null handle or info");
    std::memset(info, 0, sizeof *info);
    info->width = s->w;
    info->height = s->h;
    info->frame_index = s->frame;
    info->state_bytes = s->state_bytes;
    info->scratch_bytes = s->scratch_bytes;
    info->staging_bytes = 0;
    for (const auto& sg : s->stg) info->staging_bytes += sg.bytes;
    info->kernels_per_frame = uint32_t(s->p.levels + (s->p.mode == TG_SVGF_MODE_FULL ? 2 : 1));
    info->tma = s->tma ? 1u : 0u;
    int e = 0;
    DeviceGuard g(s->device);
    const int st = read_err(s, &e);
    info->device_errors = uint32_t(e);
    return st;
}

int tg_svgf_profile_enable(tg_svgf* s, int enable)
{
    if (!s) return fail(TG_ERR_INVALID, "null handle");
    s->prof.on = enable != 0;
    return TG_OK;
}

int tg_svgf_profile_read(tg_svgf* s, tg_svgf_kernel_stat* stats, int capacity, int* count, int reset)
{
    if (!s || !count || (capacity > 0 && !stats)) return fail(TG_ERR_INVALID, "null argument");
    DeviceGuard g(s->device);
    for (auto& r : s->prof.pending) {
        float ms = 0.0f;
        if (cudaEventSynchronize(r.b) != cudaSuccess || cudaEventElapsedTime(&ms, r.a, r.b) != cudaSuccess)
            return fail(TG_ERR_CUDA, "profile event failed: %s", cudaGetErrorString(cudaGetLastError()));
        s->prof.launches[r.fam] += 1;
        s->prof.ms[r.fam] += ms;
        s->prof.bytes[r.fam] += r.bytes;
        s->prof.pool.push_back(r.a);
        s->prof.pool.push_back(r.b);
    }
    s->prof.pending.clear();
    int n = 0;
    for (int f = 0; f < kFamilies; ++f) {
        if (!s->prof.launches[f]) continue;
        if (n < capacity) {
            tg_svgf_kernel_stat& o = stats[n];
            std::memset(&o, 0, sizeof o);
            std::snprintf(o.name, sizeof o.name, "%s", kFamilyName[f]);
            o.launches = s->prof.launches[f];
            o.total_ms = s->prof.ms[f];
            o.algo_bytes = s->prof.bytes[f];
        }
        ++n;
    }
    *count = n;
    if (reset) {
        for (int f = 0; f < kFamilies; ++f) {
            s->prof.launches[f] = 0;
            s->prof.ms[f] = 0.0;
            s->prof.bytes[f] = 0.0;
        }
    }
    return TG_OK;
}

void tg_svgf_destroy(tg_svgf* s)
{
    if (!s) return;
    DeviceGuard g(s->device);
    cudaDeviceSynchronize();
    for (auto& r : s->prof.pending) {
        cudaEventDestroy(r.a);
        cudaEventDestroy(r.b);
    }
    for (auto e : s->prof.pool) cudaEventDestroy(e);
    free_staging(s);
    free_buffers(s);
    delete s;
}

} // extern "C"
