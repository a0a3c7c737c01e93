/* C ABI of the GB300 eye-frame readback for AI entities.
 *
 * Builds the readback half of the reference's designed "vision" path
 * (docs/AI_INTERFACE.md:338-400; no code in the reference): each tick the
 * engine renders every entity's view at the resolution its brain asked for,
 * and the frames reach the brains as RGB888 (row-major, top to bottom) plus
 * float32 depth in [0, 1], through CPU-visible memory, triple-buffered, read
 * two frames behind rendering.  Here one kernel packs the eye images of all
 * entities into a device copy of the frame's slot, one copy-engine transfer
 * moves the slot into a ring of page-locked host slots, and `tg_eye_acquire`
 * returns the reference's TgVisionData view of a finished frame.  The offscreen render itself is not part of this
 * library: the caller passes each eye's colour and depth images. */
#ifndef TG_EYE_H
#define TG_EYE_H

#include <stdint.h>

#include "tg_svgf.h" /* TG_API, tg_status, tg_image, TG_FMT_* */

#ifdef __cplusplus
extern "C" {
#endif

#define TG_EYE_MAX_EYES 4096

/* The reference's TgVisionData (docs/AI_INTERFACE.md:368-381). */
typedef struct tg_vision_data {
    const uint8_t* rgb;    /* width * height * 3 bytes, row-major, top to bottom */
    const float* depth;    /* width * height floats, normalised [0, 1] */
    uint32_t width;
    uint32_t height;
    double fov_horizontal; /* radians */
} tg_vision_data;

typedef struct tg_eye_desc {
    uint32_t n_eyes;          /* 1 .. TG_EYE_MAX_EYES */
    const uint32_t* widths;   /* per eye, as requested by its brain */
    const uint32_t* heights;
    const double* fov_horizontal; /* per eye (may be NULL: 0) */
    uint32_t ring;            /* host slots; 0 = 3 (the reference's triple buffering) */
    int device;               /* -1 = current */
    void* host_buffer;        /* optional caller memory (e.g. a shared-memory region) of host_bytes, page-locked
                                 by the handle for the copies; NULL = allocated by the handle */
    uint64_t host_bytes;
} tg_eye_desc;

typedef struct tg_eye tg_eye;

/* Bytes of host memory a ring needs (16-byte aligned slots and eyes). */
TG_API uint64_t tg_eye_host_bytes(uint32_t n_eyes, const uint32_t* widths, const uint32_t* heights, uint32_t ring);

TG_API int tg_eye_create(const tg_eye_desc* desc, tg_eye** out);

/* Packs frame `frame`'s eye images into host slot frame % ring, enqueued on `stream`.  colour[i] is
 * TG_FMT_BGRA8 / TG_FMT_RGBA8 (bytes copied) or TG_FMT_RGBA16F / TG_FMT_RGBA32F (clamped to [0, 1] and rounded
 * to nearest, ties to even, to 8 bits); depth[i] is TG_FMT_R32F (copied).  Frames are submitted in order. */
TG_API int tg_eye_submit(tg_eye* h, uint64_t frame, const tg_image* colour, const tg_image* depth, void* stream);

/* Waits until frame `frame` has landed in host memory and fills out[0 .. n_eyes-1] with views into its slot.
 * The views stay valid until frame + ring is submitted.  TG_ERR_STATE if that frame was never submitted or
 * has been overwritten. */
TG_API int tg_eye_acquire(tg_eye* h, uint64_t frame, tg_vision_data* out);

TG_API void tg_eye_destroy(tg_eye* h);

#ifdef __cplusplus
}
#endif

#endif /* TG_EYE_H */
