// Reference-exact SVGF frame that allocates no memory.
//
// Who needs this: callers that cannot call cudaMalloc when they denoise.  A
// real-time render thread must not stall on the allocator mid-frame (a device
// allocation can block for milliseconds and may synchronise the device), and
// plug-in hosts that hand out a fixed memory budget, or that only give their
// plug-ins streams and buffers they already own, forbid allocation outright.
// Such callers cannot create a tg_svgf handle (tg_svgf_create allocates its
// state).  This entry point takes every per-frame image from the caller -
// including the moments the reference keeps in its own ping-pong images - and
// keeps its only scratch, the two wavelet ping-pong images of the reference
// chain (src/svgf_denoise.slang:84-90), in the fixed device array below.
//
// The array lives in this library's device code: every GPU that loads the
// library holds its 16 MiB until the process exits.  Each CUDA context on a
// device has its own copy, so calls on different devices (or in different
// contexts) never share it.  Calls in one context share it, so calls whose work
// overlaps on the GPU (different streams, or different host threads) race on
// it; callers order them, e.g. on one stream or with events.
#include <cuda_runtime.h>

#include <mutex>

#include "noalloc_ctx_cache.h"
#include "svgf_internal.h"
#include "svgf_kernels.cuh"
#include "svgf_level.cuh"

namespace {

constexpr size_t kScratchBytes = size_t(16) << 20;  // TG_SVGF_NOALLOC_SCRATCH_BYTES
static_assert(kScratchBytes == TG_SVGF_NOALLOC_SCRATCH_BYTES, "header and library disagree on the scratch size");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// The array's device address belongs to a CUDA context, not to a device
// number: a driver-API caller may run in a context other than the device's
// primary one, and cudaDeviceReset replaces the primary context.  The address
// is therefore cached per context (noalloc_ctx_cache.h), keyed by the
// context's unique id, and looked up again for a context not seen before.
// Without the driver entry points it is looked up on every call.
typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

std::mutex g_setup_mu;
tg::CtxAddrCache g_ctx_cache;

void* driver_entry(const char* name)
{
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion(name, &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
        p = nullptr;
    cudaGetLastError();
    return p;
}

// Unique id of the calling thread's current context (0 if it has none or it cannot be read).
unsigned long long current_context_id()
{
    static CtxGetCurrentFn get_current = reinterpret_cast<CtxGetCurrentFn>(driver_entry("cuCtxGetCurrent"));
    static CtxGetIdFn get_id = reinterpret_cast<CtxGetIdFn>(driver_entry("cuCtxGetId"));
    if (!get_current || !get_id) return 0;
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (get_current(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// Device address of the scratch in the current context (the host-side name
// of the array is not a device address).  The lookup makes the device's
// primary context current on a thread that had none.
int scratch_address(void** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return tg::fail(TG_ERR_CUDA, "no usable current CUDA device");
    std::lock_guard<std::mutex> lock(g_setup_mu);
    cudaError_t err = cudaSuccess;
    const int st = tg::ctx_cached_address(
        g_ctx_cache, current_context_id,
        [&err](void** p) {
            err = cudaGetSymbolAddress(p, g_noalloc_scratch);
            return (err == cudaSuccess && *p) ? 0 : 1;
        },
        out);
    if (st)
        return tg::fail(TG_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed: %s", cudaGetErrorString(err));
    return TG_OK;
}

// Pixels of one wavelet image in the residue-major layouts of strides
// 2 .. 2^(levels-1), the layouts the passes hand on (the first pass reads the
// caller's radiance and the last writes the caller's image).
size_t wavelet_pixels(int levels, uint32_t w, uint32_t h)
{
    size_t n = 0;
    for (int lg = 1; lg < levels; ++lg) {
        const size_t s = size_t(1) << lg;
        const size_t m = s * s * ((w + s - 1) / s) * ((h + s - 1) / s);
        n = m > n ? m : n;
    }
    return n;
}

} // namespace

using namespace tg;

extern "C" int tg_svgf_denoise_ref_noalloc(const tg_svgf_params* params, uint32_t width, uint32_t height,
                                           const tg_image* radiance, const tg_image* moments_prev,
                                           const tg_image* moments_curr, const tg_image* denoised, void* stream_v)
{
    if (!params || !radiance || !moments_prev || !moments_curr || !denoised)
        return fail(TG_ERR_INVALID, "null argument");
    if (params->mode != TG_SVGF_MODE_REF_EXACT) return fail(TG_ERR_INVALID, "no-alloc path supports REF_EXACT only");
    int st = validate_params(*params);
    if (st) return st;
    if (width == 0 || height == 0 || width > 32768 || height > 32768)
        return fail(TG_ERR_INVALID, "size %ux%u outside 1..32768", width, height);
    const bool f16 = params->storage == TG_SVGF_STORAGE_FP16;
    const size_t c4 = f16 ? 8 : 16;
    const size_t wav = wavelet_pixels(params->levels, width, height);
    const size_t img_bytes = (wav * c4 + 255) / 256 * 256;  // each wavelet image starts 256-byte aligned
    if (2 * img_bytes > kScratchBytes)
        return fail(TG_ERR_INVALID,
                    "%ux%u needs %zu bytes of wavelet scratch (2 images of %zu padded pixels); the no-alloc scratch "
                    "holds %zu bytes",
                    width, height, 2 * img_bytes, wav, kScratchBytes);
    static const int rad[] = {TG_FMT_RGBA32F, TG_FMT_RGBA16F};
    const int mom_fmt[] = {f16 ? TG_FMT_RG16F : TG_FMT_RG32F};
    if ((st = check_image("radiance", *radiance, width, height, rad, 2))) return st;
    if ((st = check_image("denoised", *denoised, width, height, rad, 2))) return st;
    if ((st = check_image("moments_prev", *moments_prev, width, height, mom_fmt, 1))) return st;
    if ((st = check_image("moments_curr", *moments_curr, width, height, mom_fmt, 1))) return st;
    const int64_t mrow = int64_t(fmt_bytes(mom_fmt[0])) * width;
    if ((moments_prev->pitch_bytes && moments_prev->pitch_bytes != mrow) ||
        (moments_curr->pitch_bytes && moments_curr->pitch_bytes != mrow))
        return fail(TG_ERR_INVALID, "moments images must be tightly packed (pitch %lld)", (long long)mrow);

    void* scratch = nullptr;
    if ((st = scratch_address(&scratch))) return st;
    // Nothing in the scratch has to start at zero: each pass writes every pixel
    // it hands to the next (the first pass reads only the caller's images), and
    // layout padding is never read.
    char* wa = static_cast<char*>(scratch);
    char* wb = wa + img_bytes;

    cudaStream_t stream = static_cast<cudaStream_t>(stream_v);
    RefArgs a{};
    a.w = int(width);
    a.h = int(height);
    a.raw = Img{static_cast<char*>(radiance->ptr),
                radiance->pitch_bytes ? radiance->pitch_bytes : int64_t(fmt_bytes(radiance->format)) * width,
                radiance->format, 0};
    a.out = Img{static_cast<char*>(denoised->ptr),
                denoised->pitch_bytes ? denoised->pitch_bytes : int64_t(fmt_bytes(denoised->format)) * width,
                denoised->format, 0};
    a.mom_prev = moments_prev->ptr;
    a.mom_curr = moments_curr->ptr;
    a.phi = params->sigma_l;
    a.alpha_m = params->moments_alpha;
    a.var_eps = params->variance_epsilon;
    // plain staging (no tensor maps): TMA's bounded waits report through a device error word this entry point
    // does not have
    enqueue_ref_chain<2>(a, wa, wb, params->levels, f16, stream, RefMaps{}, [](bool, auto body) { body(); });
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "kernel launch failed: %s", cudaGetErrorString(e));
    return TG_OK;
}
