// Host driver for the reference shader compiled as C++.  TEST INFRASTRUCTURE ONLY.
//
// Includes the shader source as translated by oracle/build.py and runs it the
// way the reference host does (`src/main.cpp:929-944`): pass 0 (init) and
// passes 1..3 at strides 1, 2, 4, one invocation of `svgfMain` per pixel of a
// ceil(W/8) x ceil(H/8) grid of 8x8 groups, with the moments ping-pong of
// `src/main.cpp:2401-2446` left to the caller (it passes prev and curr).
#include "slang_prelude.hpp"

bool g_slang_fp16_store = true;

#include "svgf_denoise_gen.cpp"

#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// One frame of the reference chain.  raw: h*w*4, mom_prev / mom_curr: h*w*2,
// out: h*w*4 (float32).  fp16_store selects rgba16f/rg16f store rounding.
int ref_svgf_frame(int w, int h, float* raw, float* mom_prev, float* mom_curr, float* out, int fp16_store,
                   int threads)
{
    if (w <= 0 || h <= 0) return 1;
#ifdef _OPENMP
    int prev_threads = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    g_slang_fp16_store = fp16_store != 0;
    size_t n = size_t(w) * h;
    std::vector<float4> a(n), b(n);
    lighting_raw.data = reinterpret_cast<float4*>(raw);
    lighting_raw.width = w;
    wavelet_a.data = a.data();
    wavelet_a.width = w;
    wavelet_b.data = b.data();
    wavelet_b.width = w;
    denoised_indirect.data = reinterpret_cast<float4*>(out);
    denoised_indirect.width = w;
    moments_prev.data = reinterpret_cast<float2*>(mom_prev);
    moments_prev.width = w;
    moments_curr.data = reinterpret_cast<float2*>(mom_curr);
    moments_curr.width = w;

    const uint strides[4] = {0u, 1u, 2u, 4u};
    const int gx = (w + 7) / 8 * 8, gy = (h + 7) / 8 * 8;
    for (uint pass = 0; pass < 4; ++pass) {
        push.screen_width = uint(w);
        push.screen_height = uint(h);
        push.pass_id = pass;
        push.stride = strides[pass];
#pragma omp parallel for schedule(static)
        for (int y = 0; y < gy; ++y) {
            for (int x = 0; x < gx; ++x) {
                uint3 id;
                id.x = uint(x);
                id.y = uint(y);
                id.z = 0u;
                svgfMain(id);
            }
        }
    }
#ifdef _OPENMP
    omp_set_num_threads(prev_threads);
#endif
    return 0;
}

} // extern "C"
