// CPU oracle for the bloom + post-process chain.  TEST INFRASTRUCTURE ONLY:
// this file is the checker that the CUDA path is compared against (and the
// timed CPU baseline of its bench line); nothing in the product links, loads or
// calls it.
//
// A restatement of the reference shaders `src/bloom_downsample.slang`
// (bloomExtractMain :45-82, bloomDownsampleMain :84-110, bloomUpsampleMain
// :112-173) and `src/postprocess.slang` (postprocessMain :121-179 with its
// helpers :60-119), driven the way the reference host drives them each frame
// (`src/main.cpp:306-430`, bloom image `:1298-1321`), templated on the
// arithmetic type T (float for parity, double for accuracy):
//
//  * a bloom image of max(W/2, 1) x max(H/2, 1) with
//    N = min(floor(log2(max side)) + 1, max_mips) mips, mip i of size
//    max(side >> i, 1);
//  * extract: for each mip-0 texel the 2x2 HDR block (clamped), each sample
//    max(rgb, 0) zeroed below the luminance threshold and weighted by
//    1 / (1 + luminance) (Karis), normalised by max(sum of weights, 1e-7);
//  * downsample: mean of the clamped 2x2 block of the previous mip;
//  * upsample, mip N-2 down to 0: each texel adds the (1 2 1)x(1 2 1)/16 tent of
//    the next mip around (x/2, y/2), clamped, to its own value;
//  * post: per pixel, red and blue sampled at +/- a radial chromatic-aberration
//    offset (truncated to whole pixels, clamped), each sample the HDR colour
//    plus strength x bloom mip 0 at half its coordinates; ACES fitted tonemap
//    (input matrix, rational fit, output matrix, saturate); sRGB encode; a 15%
//    blend toward a cool tint of the luminance; radial vignette; alpha 1.
//
// Sums are evaluated left to right as the shaders write them.  Every bloom
// store is rounded to binary16 when fp16_store (the reference's rgba16f bloom
// image); the output is quantised to 8-bit UNORM with round-to-nearest-even
// when unorm8 (the B8G8R8A8_UNORM swapchain image, `src/swapchain.cpp:26-40`),
// and is returned as k / 255.  Compile with -ffp-contract=off.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T> struct V3 {
    T r, g, b;
};

template <class T> inline T lum(V3<T> c) { return c.r * T(0.2126f) + c.g * T(0.7152f) + c.b * T(0.0722f); }

inline float rnd16(float v) { return static_cast<float>(static_cast<_Float16>(v)); }

template <class T> struct Img {
    std::vector<T> px;  // rgba
    int w = 0, h = 0;
    V3<T> rgb(int x, int y) const
    {
        const T* p = &px[(size_t(y) * w + x) * 4];
        return {p[0], p[1], p[2]};
    }
    void put(int x, int y, V3<T> v, bool f16)
    {
        T* p = &px[(size_t(y) * w + x) * 4];
        const T c[4] = {v.r, v.g, v.b, T(1)};
        for (int k = 0; k < 4; ++k) p[k] = f16 ? T(rnd16(float(c[k]))) : c[k];
    }
};

template <class T> T sat(T v) { return v < T(0) ? T(0) : (v > T(1) ? T(1) : v); }

template <class T> T srgb(T c)
{
    c = c > T(0) ? c : T(0);
    if (c <= T(0.0031308f)) return c * T(12.92f);
    return T(1.055f) * T(std::pow(c, T(1.0f / 2.4f))) - T(0.055f);
}

template <class T> V3<T> aces(V3<T> c)
{
    static const float IN[3][3] = {{0.59719f, 0.35458f, 0.04823f}, {0.07600f, 0.90834f, 0.01566f},
                                   {0.02840f, 0.13383f, 0.83777f}};
    static const float OUT[3][3] = {{1.60475f, -0.53108f, -0.07367f}, {-0.10208f, 1.10813f, -0.00605f},
                                    {-0.00327f, -0.07276f, 1.07602f}};
    auto mv = [](const float M[3][3], V3<T> v) {
        return V3<T>{T(M[0][0]) * v.r + T(M[0][1]) * v.g + T(M[0][2]) * v.b,
                     T(M[1][0]) * v.r + T(M[1][1]) * v.g + T(M[1][2]) * v.b,
                     T(M[2][0]) * v.r + T(M[2][1]) * v.g + T(M[2][2]) * v.b};
    };
    auto fit = [](T v) {
        const T a = v * (v + T(0.0245786f)) - T(0.000090537f);
        const T b = v * (T(0.983729f) * v + T(0.4329510f)) + T(0.238081f);
        return a / b;
    };
    V3<T> x = mv(IN, c);
    x = {fit(x.r), fit(x.g), fit(x.b)};
    x = mv(OUT, x);
    return {sat(x.r), sat(x.g), sat(x.b)};
}

template <class T>
int post_frame(int W, int H, const float* hdr_in, float threshold, float strength, int max_mips, float* out,
               float* mips_out, bool f16, bool unorm8)
{
    if (W <= 0 || H <= 0 || max_mips < 1) return -1;
    Img<T> hdr;
    hdr.w = W;
    hdr.h = H;
    hdr.px.assign(hdr_in, hdr_in + size_t(W) * H * 4);
    const uint32_t bw = std::max(uint32_t(W) / 2, 1u), bh = std::max(uint32_t(H) / 2, 1u);
    const int n = int(std::min(uint32_t(std::floor(std::log2(float(std::max(bw, bh))))) + 1, uint32_t(max_mips)));
    std::vector<Img<T>> mip(n);
    for (int i = 0; i < n; ++i) {
        mip[i].w = int(std::max(bw >> i, 1u));
        mip[i].h = int(std::max(bh >> i, 1u));
        mip[i].px.assign(size_t(mip[i].w) * mip[i].h * 4, T(0));
    }
    const T thr = T(threshold);
    // extract
    {
        Img<T>& d = mip[0];
#pragma omp parallel for schedule(static)
        for (int y = 0; y < d.h; ++y)
            for (int x = 0; x < d.w; ++x) {
                V3<T> s[4];
                T wgt[4];
                for (int k = 0; k < 4; ++k) {
                    const int sx = std::min(2 * x + (k & 1), W - 1), sy = std::min(2 * y + (k >> 1), H - 1);
                    V3<T> c = hdr.rgb(sx, sy);
                    c = {c.r > T(0) ? c.r : T(0), c.g > T(0) ? c.g : T(0), c.b > T(0) ? c.b : T(0)};
                    const T keep = lum(c) >= thr ? T(1) : T(0);
                    c = {c.r * keep, c.g * keep, c.b * keep};
                    s[k] = c;
                    wgt[k] = T(1) / (T(1) + lum(c));
                }
                const T ws = wgt[0] + wgt[1] + wgt[2] + wgt[3];
                const T den = ws > T(1e-7f) ? ws : T(1e-7f);
                V3<T> r;
                r.r = (s[0].r * wgt[0] + s[1].r * wgt[1] + s[2].r * wgt[2] + s[3].r * wgt[3]) / den;
                r.g = (s[0].g * wgt[0] + s[1].g * wgt[1] + s[2].g * wgt[2] + s[3].g * wgt[3]) / den;
                r.b = (s[0].b * wgt[0] + s[1].b * wgt[1] + s[2].b * wgt[2] + s[3].b * wgt[3]) / den;
                d.put(x, y, r, f16);
            }
    }
    // downsample
    for (int i = 1; i < n; ++i) {
        const Img<T>& s = mip[i - 1];
        Img<T>& d = mip[i];
#pragma omp parallel for schedule(static)
        for (int y = 0; y < d.h; ++y)
            for (int x = 0; x < d.w; ++x) {
                V3<T> c[4];
                for (int k = 0; k < 4; ++k) c[k] = s.rgb(std::min(2 * x + (k & 1), s.w - 1), std::min(2 * y + (k >> 1), s.h - 1));
                d.put(x, y,
                      {(c[0].r + c[1].r + c[2].r + c[3].r) * T(0.25f), (c[0].g + c[1].g + c[2].g + c[3].g) * T(0.25f),
                       (c[0].b + c[1].b + c[2].b + c[3].b) * T(0.25f)},
                      f16);
            }
    }
    // upsample
    for (int i = n - 2; i >= 0; --i) {
        const Img<T>& s = mip[i + 1];
        Img<T>& d = mip[i];
#pragma omp parallel for schedule(static)
        for (int y = 0; y < d.h; ++y)
            for (int x = 0; x < d.w; ++x) {
                const int bx = x / 2, by = y / 2;
                V3<T> sum{T(0), T(0), T(0)};
                for (int dy = -1; dy <= 1; ++dy)
                    for (int dx = -1; dx <= 1; ++dx) {
                        const T wk = T(float((dx == 0 ? 2 : 1) * (dy == 0 ? 2 : 1)) / 16.0f);
                        const V3<T> c = s.rgb(std::clamp(bx + dx, 0, s.w - 1), std::clamp(by + dy, 0, s.h - 1));
                        sum = {sum.r + wk * c.r, sum.g + wk * c.g, sum.b + wk * c.b};
                    }
                const V3<T> e = d.rgb(x, y);
                d.put(x, y, {e.r + sum.r, e.g + sum.g, e.b + sum.b}, f16);
            }
    }
    // post
    const Img<T>& bl = mip[0];
    const T st = T(strength);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const T u = (T(x) + T(0.5f)) / T(W), v = (T(y) + T(0.5f)) / T(H);
            const T ox = u - T(0.5f), oy = v - T(0.5f);
            const T d2 = ox * ox + oy * oy;
            const T ax = ox * d2 * T(0.0015f), ay = oy * d2 * T(0.0015f);
            const int px = int(ax * T(W)), py = int(ay * T(H));
            auto sample = [&](int cx, int cy) {
                cx = std::min(cx, W - 1);
                cy = std::min(cy, H - 1);
                const V3<T> h = hdr.rgb(cx, cy);
                const V3<T> b = bl.rgb(std::min(cx / 2, bl.w - 1), std::min(cy / 2, bl.h - 1));
                return V3<T>{h.r + st * b.r, h.g + st * b.g, h.b + st * b.b};
            };
            V3<T> c;
            c.r = sample(std::clamp(x + px, 0, W - 1), std::clamp(y + py, 0, H - 1)).r;
            c.g = sample(x, y).g;
            c.b = sample(std::clamp(x - px, 0, W - 1), std::clamp(y - py, 0, H - 1)).b;
            c = aces(c);
            c = {srgb(c.r), srgb(c.g), srgb(c.b)};
            const T l = lum(c);
            const V3<T> cool{l * T(0.9f), l * T(0.95f), l * T(1.1f)};
            const T g = T(0.15f);
            c = {c.r + (cool.r - c.r) * g, c.g + (cool.g - c.g) * g, c.b + (cool.b - c.b) * g};
            const T vig = sat(T(1) - (ox * ox + oy * oy) * T(1.5f));
            c = {c.r * vig, c.g * vig, c.b * vig};
            float* o = out + (size_t(y) * W + x) * 4;
            const T cc[4] = {c.r, c.g, c.b, T(1)};
            for (int k = 0; k < 4; ++k) {
                const float f = float(cc[k]);
                o[k] = unorm8 ? std::nearbyint(sat(f) * 255.0f) / 255.0f : f;
            }
        }
    if (mips_out) {
        size_t o = 0;
        for (int i = 0; i < n; ++i)
            for (T vv : mip[i].px) mips_out[o++] = float(vv);
    }
    return n;
}

} // namespace

extern "C" {

// One frame of the chain.  hdr: H*W*4 float32; out: H*W*4; mips_out (optional)
// receives the final bloom mips, concatenated.  Returns the mip count (< 0 on
// bad arguments).
int orc_post_frame(int w, int h, const float* hdr, float threshold, float strength, int max_mips, float* out,
                   float* mips_out, int fp16_store, int unorm8, int dbl, int threads)
{
#ifdef _OPENMP
    const int prev = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    const int n = dbl ? post_frame<double>(w, h, hdr, threshold, strength, max_mips, out, mips_out, fp16_store, unorm8)
                      : post_frame<float>(w, h, hdr, threshold, strength, max_mips, out, mips_out, fp16_store, unorm8);
#ifdef _OPENMP
    omp_set_num_threads(prev);
#endif
    return n;
}

} // extern "C"
