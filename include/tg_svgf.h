/*
 * tg_svgf.h - C ABI of the GB300-native SVGF denoiser.
 *
 * This is the drop-in boundary for TronGrid's SVGF combined-lighting pass.  In
 * the reference the pass is a Vulkan compute pipeline: one shader entry point
 * `svgfMain` (src/svgf_denoise.slang:152-275) dispatched four times per frame
 * with a 16-byte push block {width, height, pass_id, stride}
 * (src/main.cpp:262-269, :906-947) over seven engine-owned images
 * (src/main.cpp:1326-1397) that are zeroed at start-up and on resize
 * (src/main.cpp:1399-1496, :1547-1603) and bound in frame-parity descriptor
 * sets (src/main.cpp:2401-2446).  Here the same pass is one call per frame on
 * a CUDA stream; the handle owns the history / moments / scratch images and
 * the caller owns the per-frame inputs and outputs.
 *
 * Conventions
 *  - Every call returns a tg_status; no call throws across the ABI.  After a
 *    failure tg_last_error() returns a message for the calling thread.
 *  - A handle is not thread-safe: calls on one handle must be serialised by the
 *    caller.  Distinct handles may be used concurrently.  Work is ordered on
 *    the stream passed in (NULL = the CUDA legacy default stream).
 *  - Images are linear, row-major, pitched device buffers (tg_image).
 *    pitch_bytes == 0 means tightly packed.  The base address and pitch of a
 *    4 x float32 image must be multiples of 16 bytes, of a 4 x binary16 image
 *    multiples of 8, of every other format multiples of 4.
 */
#ifndef TG_SVGF_H
#define TG_SVGF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TG_SVGF_ABI_VERSION 1

#if defined(__GNUC__)
#define TG_API __attribute__((visibility("default")))
#else
#define TG_API
#endif

typedef enum tg_status {
    TG_OK = 0,
    TG_ERR_INVALID = 1,     /* bad argument, descriptor, format, pitch or alignment */
    TG_ERR_OOM = 2,         /* a device or host allocation failed */
    TG_ERR_CUDA = 3,        /* a CUDA runtime call failed */
    TG_ERR_TIMEOUT = 4,     /* a bounded wait (device or host side) gave up */
    TG_ERR_BUDGET = 5,      /* serving: the request does not fit the HBM budget */
    TG_ERR_UNSUPPORTED = 6, /* valid but unimplemented combination */
    TG_ERR_STATE = 7        /* the object is not in a state that allows the call */
} tg_status;

typedef enum tg_format {
    TG_FMT_NONE = 0,
    TG_FMT_RGBA32F = 1, /* 4 x float32 (16 B/px) */
    TG_FMT_RGBA16F = 2, /* 4 x binary16 (8 B/px): the reference's rgba16f */
    TG_FMT_R32F = 3,    /* 1 x float32: linear view-space depth */
    TG_FMT_RGB32F = 4,  /* 3 x float32 (12 B/px): unit normal */
    TG_FMT_OCT16 = 5,   /* 2 x snorm16 octahedral unit normal (4 B/px) */
    TG_FMT_RG32F = 6,   /* 2 x float32: motion vector */
    TG_FMT_RG16F = 7,   /* 2 x binary16: motion vector */
    TG_FMT_RGBA8 = 8,   /* 4 x 8-bit UNORM, R first (4 B/px) */
    TG_FMT_BGRA8 = 9    /* 4 x 8-bit UNORM, B first: the reference's B8G8R8A8_UNORM swapchain */
} tg_format;

typedef struct tg_image {
    void* ptr;           /* address of row 0, pixel 0 */
    int64_t pitch_bytes; /* bytes between rows; 0 = width * pixel size */
    int32_t format;      /* tg_format */
    int32_t reserved;
} tg_image;

typedef enum tg_svgf_mode {
    /* The reference shader exactly: moments EMA + sqrt-variance init pass, then
     * `levels` (3) a-trous passes at strides 1, 2, 4 with the luminance-only
     * edge stop, clamp-to-edge taps and unchanged variance propagation
     * (src/svgf_denoise.slang:176-274).  Uses only inputs.radiance. */
    TG_SVGF_MODE_REF_EXACT = 0,
    /* Schied et al. 2017 SVGF: motion-vector reprojection with a bilinear 2x2
     * history fetch and depth/normal consistency test, history length, colour
     * and moment EMA, 7x7 spatial variance for short histories, `levels` (5)
     * a-trous levels with luminance/normal/depth edge stops and squared-weight
     * variance propagation; level 0 writes the colour history. */
    TG_SVGF_MODE_FULL = 1
} tg_svgf_mode;

typedef enum tg_svgf_storage {
    TG_SVGF_STORAGE_FP32 = 0, /* history, moments and scratch in float32 */
    TG_SVGF_STORAGE_FP16 = 1  /* binary16 colour/moments, octahedral 2x16-bit normals;
                                 REF_EXACT: the reference's rgba16f/rg16f images */
} tg_svgf_storage;

/* The reference's compile-time constants (src/svgf_denoise.slang:118, :137,
 * :144, :150 and the pass count of src/main.cpp:929) as a runtime block. */
typedef struct tg_svgf_params {
    int32_t mode;             /* tg_svgf_mode */
    int32_t storage;          /* tg_svgf_storage */
    int32_t levels;           /* a-trous levels, 1..10; reference: 3 */
    int32_t max_history;      /* FULL: history length cap (>= 1) */
    int32_t fallback_frames;  /* FULL: 7x7 spatial variance while history < this */
    int32_t reserved0;
    float alpha;              /* FULL: colour EMA weight */
    float moments_alpha;      /* moment EMA weight; reference ALPHA_MOMENTS = 0.2 */
    float sigma_l;            /* FULL: luminance edge stop; REF_EXACT: SIGMA_COLOR_BASE = 2 */
    float sigma_n;            /* FULL: normal edge-stop exponent */
    float sigma_z;            /* FULL: depth edge-stop scale */
    float variance_epsilon;   /* REF_EXACT: VARIANCE_EPSILON = 1e-4 */
    float reserved[4];
} tg_svgf_params;

/* tg_svgf_desc.flags */
#define TG_SVGF_FLAG_NO_TMA 1 /* stage a-trous tiles with plain loads instead of the tensor-memory accelerator */

typedef struct tg_svgf_desc {
    uint32_t width;
    uint32_t height;
    tg_svgf_params params;
    int32_t device; /* CUDA device ordinal; -1 = the calling thread's current device */
    int32_t flags;  /* TG_SVGF_FLAG_* */
} tg_svgf_desc;

/* Per-frame inputs.  REF_EXACT reads only `radiance` (the reference's
 * lighting_raw, src/svgf_denoise.slang:61-63).  FULL also reads depth (R32F),
 * normal (RGB32F / RGBA32F / OCT16, world space, unit length) and motion
 * (RG32F / RG16F: the offset in pixels from this pixel's centre to the same
 * surface point's position in the previous frame). */
typedef struct tg_svgf_inputs {
    tg_image radiance; /* RGBA32F or RGBA16F; alpha ignored */
    tg_image depth;
    tg_image normal;
    tg_image motion;
} tg_svgf_inputs;

/* Per-frame output: the reference's denoised_indirect image
 * (src/svgf_denoise.slang:92-94, written with alpha = 1 at :264-267). */
typedef struct tg_svgf_outputs {
    tg_image denoised; /* RGBA32F or RGBA16F */
} tg_svgf_outputs;

typedef struct tg_svgf_info {
    uint32_t width;
    uint32_t height;
    uint64_t frame_index;       /* frames denoised since create / reset / resize */
    uint64_t state_bytes;       /* device bytes of persistent state (history, moments, guide) */
    uint64_t scratch_bytes;     /* device bytes of per-frame scratch */
    uint64_t staging_bytes;     /* device bytes of host-call staging (0 until first host call) */
    uint32_t kernels_per_frame; /* kernel launches per tg_svgf_denoise */
    uint32_t device_errors;     /* nonzero: a bounded device-side wait gave up (results since are invalid) */
    uint32_t tma;               /* 1: a-trous tiles are staged by the tensor-memory accelerator */
    uint32_t reserved;
} tg_svgf_info;

typedef struct tg_svgf tg_svgf;

/* Fills `out` with the defaults of a mode: REF_EXACT reproduces the reference
 * constants; FULL uses sigma_l 4, sigma_n 128, sigma_z 1, alpha 0.2,
 * moments_alpha 0.2, 5 levels, history cap 32, fallback below 4 frames. */
TG_API int tg_svgf_params_default(int32_t mode, int32_t storage, tg_svgf_params* out);

/* Allocates and zeroes the handle's state (replaces image creation,
 * src/main.cpp:1326-1397, the zero clear, :1399-1496, and pipeline /
 * descriptor creation, :2288-2446).  Synchronises the device once. */
TG_API int tg_svgf_create(const tg_svgf_desc* desc, tg_svgf** out);

/* Denoises one frame on `stream` (a cudaStream_t): replaces the SVGF block of
 * recordFrame, src/main.cpp:906-947.  Reads the previous frame's state, writes
 * this frame's state, writes outputs->denoised.  Asynchronous. */
TG_API int tg_svgf_denoise(tg_svgf* h, const tg_svgf_inputs* inputs, const tg_svgf_outputs* outputs, void* stream);

/* As tg_svgf_denoise, with inputs and output in HOST memory.  Copies the inputs
 * to handle-owned device staging, denoises and copies the result back, all
 * ordered after prior work on `stream`; returns before the copies finish.
 * The copies run on the handle's own streams, so the caller keeps the host
 * buffers alive and unmodified until tg_svgf_synchronize returns.  Host
 * buffers should be page-locked for the copies to overlap with compute; the
 * staging is a ring of three sets, so up to three frames are in flight.  A
 * dense image (pitch_bytes 0 or equal to the row) moves by one linear copy,
 * which is markedly faster than the row-by-row copy a padded pitch needs. */
TG_API int tg_svgf_denoise_host(tg_svgf* h, const tg_svgf_inputs* host_inputs, const tg_svgf_outputs* host_outputs,
                         void* stream);

/* Waits until every host copy issued by tg_svgf_denoise_host on this handle
 * has landed in host memory (the compute is ordered on the caller's stream),
 * then reports TG_ERR_TIMEOUT if a bounded device-side wait of any earlier
 * frame gave up. */
TG_API int tg_svgf_synchronize(tg_svgf* h);

/* Zeroes all history: the next frame is a full disocclusion (replaces the
 * zero clear of src/main.cpp:1399-1496).  Ordered on `stream`. */
TG_API int tg_svgf_reset(tg_svgf* h, void* stream);

/* Reallocates the state for a new resolution and zeroes it (replaces
 * rebuildFrameBuffers, src/main.cpp:1547-1603).  Synchronises the device. */
TG_API int tg_svgf_resize(tg_svgf* h, uint32_t width, uint32_t height);

TG_API int tg_svgf_get_info(const tg_svgf* h, tg_svgf_info* info);

/* Frees everything the handle owns after waiting for its work.  NULL is a no-op. */
TG_API void tg_svgf_destroy(tg_svgf* h);

TG_API const char* tg_status_string(int status);
TG_API const char* tg_last_error(void);

/* Per-kernel timing.  While enabled, every kernel launch of tg_svgf_denoise /
 * tg_svgf_denoise_host is bracketed by a CUDA event pair on the launch stream;
 * tg_svgf_profile_read waits for those events and returns, per kernel family,
 * the launch count, the summed event time and the summed compulsory bytes
 * (each buffer the kernel must read or write, counted once per pixel). */
typedef struct tg_svgf_kernel_stat {
    char name[32];     /* "ref_first", "ref_level", "full_temporal", "full_variance", "full_level" */
    uint32_t launches;
    uint32_t reserved;
    double total_ms;
    double algo_bytes;
} tg_svgf_kernel_stat;

TG_API int tg_svgf_profile_enable(tg_svgf* h, int enable);
TG_API int tg_svgf_profile_read(tg_svgf* h, tg_svgf_kernel_stat* stats, int capacity, int* count, int reset);

/* ---------------------------------------------------------------- batches --
 * Many independent camera streams of uneven resolution (the bot-mode eye
 * frames of docs/AI_INTERFACE.md:340-380, which the reference only designs)
 * denoised together: every frame step of the listed streams runs as ONE
 * persistent cooperative launch that walks a tile work-list spanning all
 * streams, stage by stage (temporal, variance, a-trous levels) with a bounded
 * grid barrier between stages, optionally replayed from a CUDA graph.  FULL
 * mode only.  Each stream keeps its own history/moments/guide state on the
 * device; a stream's result is identical alone and in any mix of streams. */
#define TG_SVGF_BATCH_MAX_STREAMS 1024

/* How a step runs: one kernel launch per stage over the work-list of all the
 * step's streams (7 launches per step with 5 levels, whatever the number of
 * streams), or one persistent cooperative launch with a grid barrier between
 * stages.  tg_svgf_batch_autotune measures both. */
#define TG_SVGF_BATCH_STAGES 0
#define TG_SVGF_BATCH_PERSISTENT 1

typedef struct tg_svgf_batch tg_svgf_batch;

typedef struct tg_svgf_batch_desc {
    uint32_t n_streams;        /* 1 .. TG_SVGF_BATCH_MAX_STREAMS */
    const uint32_t* widths;    /* n_streams widths */
    const uint32_t* heights;   /* n_streams heights */
    tg_svgf_params params;     /* mode must be TG_SVGF_MODE_FULL */
    int32_t device;            /* -1 = current */
    int32_t rows_per_thread;   /* a-trous outputs per thread (tile 32 x 4r): 1 or 2; 0 = 2 until autotuned */
    int32_t ctas_per_sm;       /* persistent CTAs (of 128 threads) per SM, up to the occupancy limit; 0 = that limit */
    int32_t use_graph;         /* nonzero: replay each step from a captured CUDA graph */
    int32_t strategy;          /* TG_SVGF_BATCH_STAGES (default) or TG_SVGF_BATCH_PERSISTENT */
    uint32_t barrier_timeout_us; /* bound of each grid-barrier wait; 0 = about one second */
    int32_t debug_barrier_extra; /* test hook: the barrier also waits for this many CTAs that do not
                                    exist, so every step's wait runs out (TG_ERR_TIMEOUT); 0 otherwise */
} tg_svgf_batch_desc;

typedef struct tg_svgf_batch_info {
    uint32_t n_streams;
    int32_t rows_per_thread;   /* current tile shape: 32 x (4 * rows_per_thread) outputs */
    int32_t ctas_per_sm;
    int32_t grid_ctas;         /* persistent grid size */
    int32_t graphs;            /* 1 when steps replay CUDA graphs */
    int32_t strategy;          /* TG_SVGF_BATCH_STAGES or TG_SVGF_BATCH_PERSISTENT */
    uint64_t state_bytes;      /* device state of all streams */
    uint64_t scratch_bytes;    /* device scratch of all streams */
    uint64_t steps;            /* frame steps run */
    uint64_t barrier_timeouts; /* steps whose grid barrier gave up (TG_ERR_TIMEOUT) */
    double tuned_ms;           /* step time of the autotuned choice (0 before tuning) */
} tg_svgf_batch_info;

TG_API int tg_svgf_batch_create(const tg_svgf_batch_desc* desc, tg_svgf_batch** out);

/* One frame step: stream_ids[k] gets inputs[k] and writes outputs[k]
 * (device images, FULL-mode formats).  A stream may appear at most once.
 * Enqueued on `stream`; reports TG_ERR_TIMEOUT for an earlier step whose grid
 * barrier gave up (that step's outputs are invalid). */
TG_API int tg_svgf_batch_denoise(tg_svgf_batch* b, uint32_t n, const uint32_t* stream_ids,
                                 const tg_svgf_inputs* inputs, const tg_svgf_outputs* outputs, void* stream);

/* Times every candidate - strategy x rows_per_thread (x ctas_per_sm for the
 * persistent launch) - on `steps` steps of the given frames, keeps the
 * fastest, then zeroes every stream's state. */
TG_API int tg_svgf_batch_autotune(tg_svgf_batch* b, uint32_t n, const uint32_t* stream_ids,
                                  const tg_svgf_inputs* inputs, const tg_svgf_outputs* outputs, uint32_t steps,
                                  void* stream);

/* Zeroes one stream's history (its next frame is a full disocclusion). */
TG_API int tg_svgf_batch_reset_stream(tg_svgf_batch* b, uint32_t stream_id, void* stream);

/* Waits for the batch's work and reports a barrier timeout of any step. */
TG_API int tg_svgf_batch_synchronize(tg_svgf_batch* b);

TG_API int tg_svgf_batch_get_info(const tg_svgf_batch* b, tg_svgf_batch_info* info);

TG_API void tg_svgf_batch_destroy(tg_svgf_batch* b);

/* ---------------------------------------------------------------- serving --
 * A request loop over many sessions (camera streams that come and go): frames
 * are submitted from any host thread with host buffers and complete
 * asynchronously.  With batching on, a scheduler thread admits every queued
 * frame whose session has a free slot (one frame per session per batch, in
 * arrival order), copies the batch's inputs in while the previous batch runs,
 * and denoises the batch in one persistent launch (continuous batching); with
 * batching off every request is launched on its own (the plain per-request
 * path).  Each session's history stays resident on the device inside an HBM
 * budget: a session that does not fit evicts the least recently used idle
 * session (one with no queued or running frame); an evicted session's next
 * frame restarts as a full disocclusion.  FULL mode only. */
typedef struct tg_svgf_server tg_svgf_server;

typedef struct tg_svgf_server_desc {
    tg_svgf_params params;     /* mode must be TG_SVGF_MODE_FULL */
    uint64_t hbm_budget_bytes; /* device bytes for resident sessions (state, scratch, staging) */
    uint32_t max_sessions;     /* sessions known at once (resident or not) */
    uint32_t max_batch;        /* frames per launch, 1 .. TG_SVGF_BATCH_MAX_STREAMS */
    int32_t device;            /* -1 = current */
    int32_t batching;          /* 1: continuous batching; 0: plain per-request launches */
    int32_t use_graph;         /* batching with the persistent strategy: replay launches from CUDA graphs */
    int32_t strategy;          /* batching: TG_SVGF_BATCH_STAGES (default) or TG_SVGF_BATCH_PERSISTENT */
    uint64_t max_batch_pixels; /* batching: stop adding frames to a launch past this many pixels (the
                                  first frame is always taken); bounds a launch's duration and so the
                                  wait of the frames queued behind it.  0 = 4 Mpx */
} tg_svgf_server_desc;

typedef struct tg_svgf_request_info {
    int32_t status;      /* TG_OK, TG_ERR_BUDGET (session larger than the budget), TG_ERR_STATE (session ended) ... */
    uint32_t batch_size; /* frames in the launch that carried this request */
    double latency_ms;   /* submit -> result in host memory */
    double queue_ms;     /* submit -> launch */
} tg_svgf_request_info;

typedef struct tg_svgf_server_stats {
    uint64_t submitted, completed, failed;
    uint64_t admissions, evictions, launches;
    uint64_t resident_bytes, peak_resident_bytes;
    uint32_t resident_sessions, max_batch_seen;
    double p50_ms, p99_ms, mean_ms; /* latency of completed requests since the last reset */
    double mpx_per_s;               /* pixels completed / (last completion - first submit) */
    double wall_s;
} tg_svgf_server_stats;

TG_API int tg_svgf_server_create(const tg_svgf_server_desc* desc, tg_svgf_server** out);

/* Queues one frame of `session` (width x height; host inputs/outputs, kept
 * alive and unmodified until the ticket completes).  Inputs in page-locked
 * host memory mapped for the device (cudaHostAlloc, cudaHostRegister; e.g.
 * torch pin_memory) are read by the kernels in place over the host link, with
 * no copy; other host inputs are copied into device slots.  Outputs are copied
 * out (page-locked outputs overlap with the next launches). */
TG_API int tg_svgf_server_submit(tg_svgf_server* s, uint64_t session, uint32_t width, uint32_t height,
                                 const tg_svgf_inputs* host_inputs, const tg_svgf_outputs* host_outputs,
                                 uint64_t* ticket);

/* Waits for a ticket (timeout_us < 0: no limit); TG_ERR_TIMEOUT if it did not
 * complete in time, else TG_OK with the request's own status in info.  A
 * completed ticket is forgotten once waited for. */
TG_API int tg_svgf_server_wait(tg_svgf_server* s, uint64_t ticket, int64_t timeout_us, tg_svgf_request_info* info);

/* Ends a session: its queued frames fail with TG_ERR_STATE and its device
 * memory is released once no frame of it is running. */
TG_API int tg_svgf_server_end_session(tg_svgf_server* s, uint64_t session);

TG_API int tg_svgf_server_get_stats(tg_svgf_server* s, tg_svgf_server_stats* stats, int reset);

/* Stops the scheduler after the queued work and frees everything. */
TG_API void tg_svgf_server_destroy(tg_svgf_server* s);

/* Reference-exact frame for callers that cannot allocate device memory.
 * This entry point has no counterpart in the reference.  It exists for callers
 * that must not call cudaMalloc while they denoise: a real-time render thread
 * (a device allocation can stall for milliseconds and may synchronise the
 * device mid-frame) and plug-in hosts that give their plug-ins a fixed memory
 * budget or only buffers and streams they already own.  Such callers cannot
 * create a tg_svgf handle, which allocates its state.
 *
 * The caller passes every image: radiance in, moments_prev in, moments_curr
 * out (the reference's moments ping-pong, src/svgf_denoise.slang:76-82:
 * RG16F with TG_SVGF_STORAGE_FP16, RG32F with TG_SVGF_STORAGE_FP32, tightly
 * packed, zero for the first frame) and denoised out.  The only scratch, the
 * two wavelet ping-pong images, lives in a fixed 16 MiB device array inside
 * this library, which every GPU that loads the library holds until exit.
 * With the default 3 levels that bounds the frame to about 1 Mpx with fp16
 * images (e.g. 1280x720) and about 0.5 Mpx with fp32 images (e.g. 960x540);
 * more levels pad the wavelet images further and lower the bound (at 10
 * levels 960x540 fp32 no longer fits).  Frames that do not fit are rejected
 * with TG_ERR_INVALID before anything is launched.  params->mode must be
 * TG_SVGF_MODE_REF_EXACT.
 *
 * Each CUDA context (one per device for runtime-API callers) has its own copy
 * of the array.  The first call in a context looks up the array's device
 * address in that context (the calling thread's current one) and caches it by
 * the context's unique id; make that first call before any stream capture.
 * Calls on different devices or in different contexts never share the array.
 * Calls in the same context do, and the array keeps the last call's contents:
 * calls whose work overlaps on the GPU race, so order them (one stream, or
 * events between streams).  No call allocates. */
#define TG_SVGF_NOALLOC_SCRATCH_BYTES (16u << 20)
TG_API int tg_svgf_denoise_ref_noalloc(const tg_svgf_params* params, uint32_t width, uint32_t height,
                                       const tg_image* radiance, const tg_image* moments_prev,
                                       const tg_image* moments_curr, const tg_image* denoised, void* stream);

/* Bytes of device state a FULL or REF_EXACT stream of w x h keeps resident
 * (history, moments, guide), for admission control. */
TG_API uint64_t tg_svgf_state_bytes(const tg_svgf_params* params, uint32_t width, uint32_t height);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* TG_SVGF_H */
