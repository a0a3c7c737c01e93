// Host driver for the reference froxel-filter shader compiled as C++.
// TEST INFRASTRUCTURE ONLY.
//
// Includes `src/volumetric_filter.slang` as translated by oracle/build.py and
// runs it the way the reference host does (`src/main.cpp:993-1005`): one
// invocation of `filterMain` per froxel of a ceil(W/8) x ceil(H/8) x D grid of
// 8x8x1 groups, the push-constant block copied in byte for byte, the
// (history, output) ping-pong left to the caller.
#include "slang_prelude_fog.hpp"

bool g_slang_fp16_store = true;

#include "volumetric_filter_gen.cpp"

#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

static_assert(sizeof(FilterPushConstants) == 176, "FilterPushConstants must keep the reference's 176-byte layout");

extern "C" {

// params: the 176-byte push block; raw / hist / out: D*H*W*4 float32 texels.
int ref_fog_filter(const void* params, float* raw, float* hist, float* out, int fp16_store, int threads)
{
    std::memcpy(&push, params, sizeof push);
    const int W = int(push.froxel_width), H = int(push.froxel_height), D = int(push.froxel_depth);
    if (W <= 0 || H <= 0 || D <= 0) return 1;
#ifdef _OPENMP
    const int prev = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    g_slang_fp16_store = fp16_store != 0;
    RWTexture3D<float4>* imgs[3] = {&froxel_inject_raw, &froxel_history, &froxel_output};
    float* ptrs[3] = {raw, hist, out};
    for (int k = 0; k < 3; ++k) {
        imgs[k]->data = reinterpret_cast<float4*>(ptrs[k]);
        imgs[k]->width = W;
        imgs[k]->height = H;
    }
    const int gx = (W + 7) / 8 * 8, gy = (H + 7) / 8 * 8;
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < D; ++z)
        for (int y = 0; y < gy; ++y)
            for (int x = 0; x < gx; ++x) filterMain(uint3(uint(x), uint(y), uint(z)));
#ifdef _OPENMP
    omp_set_num_threads(prev);
#endif
    return 0;
}

} // extern "C"
