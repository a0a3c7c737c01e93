// Host driver for the reference bloom and post-process shaders compiled as
// C++.  TEST INFRASTRUCTURE ONLY.
//
// Includes `src/bloom_downsample.slang` and `src/postprocess.slang` as
// translated by oracle/build.py (each in its own namespace: both declare
// `hdr_input`, `push` and `LUMINANCE_WEIGHTS`) and runs them the way the
// reference host does each frame (`src/main.cpp:306-430`, `:1298-1321`):
// a bloom image of half the frame's size (at least 1x1) with
// min(floor(log2(max side)) + 1, max_mips) rgba16f mips; bloomExtractMain into
// mip 0; bloomDownsampleMain into mips 1 .. N-1; bloomUpsampleMain from mip N-2
// down to mip 0, each adding the tent-filtered next mip into its own; then
// postprocessMain from the HDR image and bloom mip 0 into the 8-bit UNORM
// swapchain image.  Every dispatch covers ceil(w/8) x ceil(h/8) groups of 8x8.
#include "slang_prelude_post.hpp"

namespace bloom_ref {
#include "bloom_downsample_gen.cpp"
}
namespace post_ref {
#include "postprocess_gen.cpp"
}

#include <algorithm>
#include <cmath>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class F> void dispatch(int w, int h, F f)
{
    const int gx = (w + 7) / 8 * 8, gy = (h + 7) / 8 * 8;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < gy; ++y)
        for (int x = 0; x < gx; ++x) f(uint3(uint(x), uint(y), 0u));
}

} // namespace

extern "C" {

// hdr: h*w*4 float32 (fp16-representable values); out: h*w*4 float32 holding
// the UNORM8 values (k / 255); mips_out (optional): the final bloom mips,
// concatenated, each mw*mh*4.  Returns the mip count, or -1 on bad arguments.
int ref_post_frame(int w, int h, const float* hdr, float threshold, float strength, int max_mips, float* out,
                   float* mips_out, int threads)
{
    if (w <= 0 || h <= 0 || max_mips < 1) return -1;
#ifdef _OPENMP
    const int prev = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const uint32_t bw = std::max(uint32_t(w) / 2, 1u), bh = std::max(uint32_t(h) / 2, 1u);
    const uint32_t levels = uint32_t(std::floor(std::log2(float(std::max(bw, bh))))) + 1;
    const int n = int(std::min(levels, uint32_t(max_mips)));
    std::vector<std::vector<float4>> mip(n);
    std::vector<int> mw(n), mh(n);
    for (int i = 0; i < n; ++i) {
        mw[i] = int(std::max(bw >> i, 1u));
        mh[i] = int(std::max(bh >> i, 1u));
        mip[i].assign(size_t(mw[i]) * mh[i], float4(0.f, 0.f, 0.f, 0.f));
    }
    std::vector<float4> hdr_img(size_t(w) * h);
    for (size_t k = 0; k < hdr_img.size(); ++k)
        hdr_img[k] = float4(hdr[4 * k], hdr[4 * k + 1], hdr[4 * k + 2], hdr[4 * k + 3]);

    auto bind = [](RWTexture2D<float4>& t, std::vector<float4>& img, int iw, int ih, int store) {
        t.data = img.data();
        t.width = iw;
        t.height = ih;
        t.store = store;
    };
    using namespace bloom_ref;
    bind(bloom_ref::hdr_input, hdr_img, w, h, STORE_FP16);
    bloom_ref::push.threshold = threshold;
    bind(bloom_src, mip[0], mw[0], mh[0], STORE_FP16);
    bind(bloom_dst, mip[0], mw[0], mh[0], STORE_FP16);
    dispatch(mw[0], mh[0], [](uint3 id) { bloomExtractMain(id); });
    for (int i = 1; i < n; ++i) {
        bind(bloom_src, mip[i - 1], mw[i - 1], mh[i - 1], STORE_FP16);
        bind(bloom_dst, mip[i], mw[i], mh[i], STORE_FP16);
        dispatch(mw[i], mh[i], [](uint3 id) { bloomDownsampleMain(id); });
    }
    for (int i = n - 2; i >= 0; --i) {
        bind(bloom_src, mip[i + 1], mw[i + 1], mh[i + 1], STORE_FP16);
        bind(bloom_dst, mip[i], mw[i], mh[i], STORE_FP16);
        dispatch(mw[i], mh[i], [](uint3 id) { bloomUpsampleMain(id); });
    }

    std::vector<float4> sw(size_t(w) * h);
    bind(post_ref::hdr_input, hdr_img, w, h, STORE_FP16);
    bind(post_ref::swapchain_output, sw, w, h, STORE_UNORM8);
    bind(post_ref::bloom_texture, mip[0], mw[0], mh[0], STORE_FP16);
    post_ref::push.bloom_strength = strength;
    dispatch(w, h, [](uint3 id) { post_ref::postprocessMain(id); });

    for (size_t k = 0; k < sw.size(); ++k) {
        out[4 * k] = sw[k].x;
        out[4 * k + 1] = sw[k].y;
        out[4 * k + 2] = sw[k].z;
        out[4 * k + 3] = sw[k].w;
    }
    if (mips_out) {
        size_t o = 0;
        for (int i = 0; i < n; ++i)
            for (const float4& v : mip[i]) {
                mips_out[o++] = v.x;
                mips_out[o++] = v.y;
                mips_out[o++] = v.z;
                mips_out[o++] = v.w;
            }
    }
#ifdef _OPENMP
    omp_set_num_threads(prev);
#endif
    return n;
}

} // extern "C"
