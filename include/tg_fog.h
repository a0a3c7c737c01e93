/* C ABI of the GB300 volumetric-fog froxel filter.
 *
 * Replaces the reference's filter dispatch (src/main.cpp:993-1005: bind the
 * filter pipeline and the frame-parity descriptor set {inject, history,
 * output}, push VolumetricFilterPushConstants, dispatch ceil(W/8) x ceil(H/8)
 * x D groups of src/volumetric_filter.slang filterMain).  Per froxel: the 3x3
 * mean of the injected light over the in-grid neighbours of its slice; with
 * valid history, its centre reprojected into the previous frame and, when it
 * lands inside the previous grid and depth range, blended as
 * history + (mean - history) * alpha with a trilinear, clamp-to-edge history
 * fetch.
 *
 * Like the reference, the caller owns the three volumes and alternates the
 * (history, output) pair between two allocations each frame. */
#ifndef TG_FOG_H
#define TG_FOG_H

#include <stdint.h>

#include "tg_svgf.h" /* TG_API, tg_status, TG_FMT_* */

#ifdef __cplusplus
extern "C" {
#endif

/* Parameters of one filter pass, in the byte layout of the reference's
 * VolumetricFilterPushConstants (src/main.cpp:221-234; 176 bytes), so an
 * engine passes the block it already fills for the push constants. */
typedef struct tg_fog_filter_params {
    float inv_view_projection[16];  /* this frame; column-major: element (col, row) at [col * 4 + row] */
    float prev_view_projection[16]; /* previous frame; same layout */
    float camera_pos[3];            /* world-space camera position of this frame */
    float alpha;                    /* EMA weight of the current (spatial) estimate */
    uint32_t froxel_width;
    uint32_t froxel_height;
    uint32_t froxel_depth;
    uint32_t history_valid;         /* 0: the output is the spatial mean (first frame) */
    float near_plane;               /* logarithmic slice distribution near .. far (view depth) */
    float far_plane;
    float pad0;
    float pad1;
} tg_fog_filter_params;

/* A froxel volume in device memory: froxel_depth slices of froxel_height rows
 * of froxel_width rgba texels. */
typedef struct tg_volume {
    void* ptr;
    int64_t row_pitch_bytes;   /* 0: width x texel bytes */
    int64_t slice_pitch_bytes; /* 0: height x row pitch */
    int32_t format;            /* TG_FMT_RGBA16F (the reference's images) or TG_FMT_RGBA32F */
    int32_t reserved;
} tg_volume;

/* One filter pass, enqueued on `stream` (a cudaStream_t; NULL = legacy
 * default).  `history` and `output` share a format; `inject_raw` may use the
 * other one.  `output` must not overlap `inject_raw` or `history` (the pass
 * reads neighbours of both).  Allocates nothing; returns TG_ERR_INVALID for
 * bad dimensions, formats, alignment, pitches, depth range or overlapping
 * volumes, TG_ERR_CUDA when the launch fails. */
TG_API int tg_fog_filter(const tg_fog_filter_params* params, const tg_volume* inject_raw, const tg_volume* history,
                         const tg_volume* output, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TG_FOG_H */
