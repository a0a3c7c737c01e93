// Helpers shared by the translation units of the SVGF library (not part of
// the public ABI).
#pragma once

#include <cstddef>
#include <cstdint>
#include <string>

#include <cuda.h>
#include <cuda_runtime.h>

#include "tg_svgf.h"

struct tg_svgf;

namespace tg {

struct Img;

extern thread_local std::string g_last_error;

// Records a message for tg_last_error() and returns `status`.
int fail(int status, const char* fmt, ...);

int fmt_bytes(int fmt);
int check_image(const char* what, const tg_image& im, uint32_t w, uint32_t h, const int* allowed, int n_allowed);
int validate_params(const tg_svgf_params& p);
int sigma_n_squarings(float sigma_n);
size_t state_bytes_of(const tg_svgf_params& p, uint32_t w, uint32_t h);
size_t scratch_bytes_of(const tg_svgf_params& p, uint32_t w, uint32_t h);
// Pixels of one a-trous scratch image in the largest residue-major layout used.
size_t col_pixels_of(const tg_svgf_params& p, uint32_t w, uint32_t h);
// Bytes of one a-trous scratch record (FULL: colour, variance and guide).
size_t rec_bytes_of(const tg_svgf_params& p);
// Bytes of one a-trous scratch buffer: the records, then (FULL mode) a compact
// plane of the records' variances in the same residue-major layout, which the
// levels read for the 3x3 variance blur.
size_t col_bytes_of(const tg_svgf_params& p, uint32_t w, uint32_t h);
// Byte offset of that variance plane from the start of the buffer.
size_t col_var_offset_of(const tg_svgf_params& p, uint32_t w, uint32_t h);
// FP32 FULL records are stored as two half-planes (all colours, then all
// guides): the index of the guide half-plane in 16-byte units.
size_t col_guide_half_of(const tg_svgf_params& p, uint32_t w, uint32_t h);
// Bytes of the per-pixel-block fallback flags of a FULL frame.
size_t fb_flags_bytes_of(uint32_t w, uint32_t h);

// Copies an image of h rows of `row` bytes between pitched buffers: one
// linear copy when both pitches equal the row (a dense image), a 2-D copy
// otherwise.  (Dense 4K images moved by 2-D copies measured up to 3x slower
// between pinned host memory and the device than by linear copies.)
inline cudaError_t copy_image_async(void* dst, size_t dpitch, const void* src, size_t spitch, size_t row, size_t h,
                                    cudaMemcpyKind kind, cudaStream_t st)
{
    if (dpitch == row && spitch == row) return cudaMemcpyAsync(dst, src, row * h, kind, st);
    return cudaMemcpy2DAsync(dst, dpitch, src, spitch, row, h, kind, st);
}

// TMA maps of one FULL stream's a-trous levels for tiles of R output rows per
// thread: [0] the tc plane, [1] and [2] the guide planes of parity 0 and 1
// (level 0 stages from these), [2 + L] the input records of level L >= 1.
// Returns a mask: bit 0 = the three plane maps were encoded, bit L = level L's.
constexpr int kFullMaps = 12;
unsigned full_level_maps(const tg_svgf_params& p, uint32_t w, uint32_t h, int R, void* colA, void* colB, void* tc,
                         void* guide0, void* guide1, CUtensorMap* maps);

} // namespace tg
