/* C ABI of the GB300 bloom + post-process chain.
 *
 * Replaces the reference's per-frame bloom and post-process dispatches
 * (src/main.cpp:306-430 recordBloomDownsample / recordBloomUpsample and the
 * post-process dispatch; shaders src/bloom_downsample.slang and
 * src/postprocess.slang): thresholded Karis-weighted extraction of the HDR
 * frame into a half-resolution rgba16f bloom mip chain, 2x2 downsampling to
 * the smallest mip, additive 3x3 tent upsampling back to mip 0, then chromatic
 * aberration, bloom composite, ACES fitted tonemap, sRGB encode, cool colour
 * grade and vignette into the display image.
 *
 * The handle owns the bloom image (like the reference's bloom_image,
 * src/main.cpp:1298-1321, recreated on resize); the caller owns the HDR input
 * and the display output. */
#ifndef TG_POST_H
#define TG_POST_H

#include <stdint.h>

#include "tg_svgf.h" /* TG_API, tg_status, tg_image, TG_FMT_* */

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tg_post_params {
    float bloom_threshold; /* luminance below which HDR samples do not bloom (reference BLOOM_THRESHOLD 1.0) */
    float bloom_strength;  /* scale of the bloom added before tonemapping (reference BLOOM_STRENGTH 0.095) */
    uint32_t max_mips;     /* bloom mip chain cap (reference BLOOM_MAX_MIPS 6); at least 1 */
    uint32_t reserved;
} tg_post_params;

typedef struct tg_post tg_post;

typedef struct tg_post_info {
    uint32_t width, height;   /* frame size */
    uint32_t mip_count;       /* min(floor(log2(max(W/2, H/2))) + 1, max_mips) */
    uint32_t reserved0;
    uint64_t bloom_bytes;     /* device bytes of the bloom chain */
    uint32_t mip_width[16];   /* mip i is max((W/2) >> i, 1) x max((H/2) >> i, 1) */
    uint32_t mip_height[16];
    void* mip_ptr[16];        /* device pointers of the rgba16f mips (row-major, unpadded), valid until resize / destroy */
} tg_post_info;

/* The reference's constants (src/main.cpp:92-98). */
TG_API int tg_post_params_default(tg_post_params* params);

/* Allocates the bloom chain for frames of width x height on `device` (-1 = current). */
TG_API int tg_post_create(uint32_t width, uint32_t height, const tg_post_params* params, int device, tg_post** out);

/* One frame, enqueued on `stream`: `hdr` is TG_FMT_RGBA16F (the reference's HDR image) or TG_FMT_RGBA32F;
 * `out` is TG_FMT_BGRA8 (the reference's B8G8R8A8_UNORM swapchain), TG_FMT_RGBA8 (both rounded to nearest,
 * ties to even, after clamping to [0, 1]) or TG_FMT_RGBA32F (the unquantised colour).  Allocates nothing. */
TG_API int tg_post_process(tg_post* h, const tg_image* hdr, const tg_image* out, void* stream);

/* Reallocates the bloom chain for a new frame size (the reference recreates its bloom image on resize). */
TG_API int tg_post_resize(tg_post* h, uint32_t width, uint32_t height);

TG_API int tg_post_get_info(const tg_post* h, tg_post_info* info);

TG_API void tg_post_destroy(tg_post* h);

#ifdef __cplusplus
}
#endif

#endif /* TG_POST_H */
