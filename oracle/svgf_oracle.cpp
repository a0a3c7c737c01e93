// CPU oracle for the SVGF denoiser.  TEST INFRASTRUCTURE ONLY: this file is the
// checker that the CUDA path is compared against (and the timed CPU baseline);
// nothing in the product links, loads or calls it.
//
// Two algorithms live here, each templated on the arithmetic type T (float or
// double):
//
//  * REF-EXACT: a line-by-line restatement of the reference shader
//    `src/svgf_denoise.slang` (svgfMain, lines 152-275) driven the way the
//    reference host drives it (`src/main.cpp:929-944`: pass 0 init, then
//    passes 1..3 at strides 1, 2, 4).  Optional rounding to fp16 at every image
//    store reproduces the reference's rgba16f / rg16f images
//    (`src/svgf_denoise.slang:61-94`).
//
//  * FULL: the Schied et al. 2017 SVGF superset (motion-vector reprojection with
//    a bilinear 2x2 history fetch and depth/normal consistency test, history
//    length, colour + moment EMA with a mean-centred moment state, 7x7 spatial
//    variance fallback for short histories, a-trous levels with luminance /
//    normal / depth edge stops and squared-weight variance propagation, level-0
//    output written back as colour history).  The reference has no code for
//    this mode (it stops at `src/svgf_denoise.slang:170-175`, "no motion-vector
//    reprojection"), so the FULL half is pinned only by the closed-form
//    known-answer tests in tests/ and by float-vs-double agreement.
//
// Parity status: the reference ships no tests, golden images or fixtures for
// this path and its shader compiler (slangc) is absent, so the restatement is
// pinned by (a) the reference shader source compiled as C++ through
// oracle/build.py when the reference checkout is present, and (b) closed-form
// known-answer tests.  Without (a) the REF-EXACT half is "parity unpinned".
//
// Compile with -ffp-contract=off: the GPU path evaluates every threshold
// decision with explicitly unfused operations, and the oracle must do the same.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- helpers ----

inline float to_half_float(float x)
{
    // Round-to-nearest-even to IEEE binary16, returned widened to float.
    return static_cast<float>(static_cast<_Float16>(x));
}

inline float to_half_satfinite(float x)
{
    const float hmax = 65504.0f;
    if (x > hmax) x = hmax;
    if (x < -hmax) x = -hmax;
    return to_half_float(x);
}

template <class T> inline T q16(T x, bool on) { return on ? T(to_half_float(float(x))) : x; }
template <class T> inline T q16s(T x, bool on) { return on ? T(to_half_satfinite(float(x))) : x; }
template <class T> inline T q32(T x, bool on) { return on ? T(float(x)) : x; }

// Rec.709 luminance, `src/svgf_denoise.slang:109-112`.  Evaluated left to right
// as three products and two sums (no fused multiply-add).
template <class T> inline T lum(T r, T g, T b)
{
    return r * T(0.2126f) + g * T(0.7152f) + b * T(0.0722f);
}

// Octahedral normal encoding to two snorm16 values (Meyer et al. 2010,
// "On Floating-Point Normal Vectors"), and its decode.  Used to emulate the
// FP16 storage form's 2x16-bit normals.
inline float sgn_nz(float v) { return v >= 0.0f ? 1.0f : -1.0f; }

inline void oct16_encode(float nx, float ny, float nz, int16_t& ex, int16_t& ey)
{
    float l1 = std::fabs(nx) + std::fabs(ny) + std::fabs(nz);
    float px = l1 > 0.0f ? nx / l1 : 0.0f;
    float py = l1 > 0.0f ? ny / l1 : 0.0f;
    if (nz < 0.0f) {
        float ox = (1.0f - std::fabs(py)) * sgn_nz(px);
        float oy = (1.0f - std::fabs(px)) * sgn_nz(py);
        px = ox;
        py = oy;
    }
    px = std::min(1.0f, std::max(-1.0f, px));
    py = std::min(1.0f, std::max(-1.0f, py));
    ex = static_cast<int16_t>(std::nearbyint(px * 32767.0f));
    ey = static_cast<int16_t>(std::nearbyint(py * 32767.0f));
}

inline void oct16_decode(int16_t ex, int16_t ey, float& nx, float& ny, float& nz)
{
    float px = std::max(-1.0f, static_cast<float>(ex) / 32767.0f);
    float py = std::max(-1.0f, static_cast<float>(ey) / 32767.0f);
    float vz = 1.0f - std::fabs(px) - std::fabs(py);
    if (vz < 0.0f) {
        float ox = (1.0f - std::fabs(py)) * sgn_nz(px);
        float oy = (1.0f - std::fabs(px)) * sgn_nz(py);
        px = ox;
        py = oy;
    }
    float d = px * px + py * py + vz * vz;
    float inv = 1.0f / std::sqrt(d);
    nx = px * inv;
    ny = py * inv;
    nz = vz * inv;
}

// Unnormalised octahedral decode: the point on the unit octahedron.  The
// FP16 storage form keeps normals this way; the reprojection normal test is
// scale-free, and the edge-stopping weights normalise on use.
inline void oct16_decode_raw(int16_t ex, int16_t ey, float& nx, float& ny, float& nz)
{
    const float kInv = 1.0f / 32767.0f;
    float px = std::max(-1.0f, static_cast<float>(ex) * kInv);
    float py = std::max(-1.0f, static_cast<float>(ey) * kInv);
    float vz = 1.0f - std::fabs(px) - std::fabs(py);
    if (vz < 0.0f) {
        float ox = (1.0f - std::fabs(py)) * sgn_nz(px);
        float oy = (1.0f - std::fabs(px)) * sgn_nz(py);
        px = ox;
        py = oy;
    }
    nx = px;
    ny = py;
    nz = vz;
}

template <class T> inline void oct16_roundtrip(T& x, T& y, T& z)
{
    int16_t ex, ey;
    oct16_encode(float(x), float(y), float(z), ex, ey);
    float a, b, c;
    oct16_decode_raw(ex, ey, a, b, c);
    x = T(a);
    y = T(b);
    z = T(c);
}

// Reprojection normal test, scale-free: the angle between a and b is at most
// acos(0.9) iff a.b >= 0 and (a.b)^2 >= 0.81 |a|^2 |b|^2.
template <class T> inline bool normal_close(T ax, T ay, T az, T bx, T by, T bz)
{
    T d = ax * bx + ay * by + az * bz;
    if (!(d >= T(0))) return false;
    T aa = ax * ax + ay * ay + az * az;
    T bb = bx * bx + by * by + bz * bz;
    return d * d >= (T(0.81f) * aa) * bb;
}

// The unit normal used by the edge-stopping weights.
template <class T> inline void unit_normal(const T* g, bool f16, T& x, T& y, T& z)
{
    x = g[0];
    y = g[1];
    z = g[2];
    if (f16) {
        T inv = T(1) / std::sqrt(x * x + y * y + z * z);
        x *= inv;
        y *= inv;
        z *= inv;
    }
}

inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

struct Threads {
    explicit Threads(int n)
    {
#ifdef _OPENMP
        prev = omp_get_max_threads();
        if (n > 0) omp_set_num_threads(n);
#else
        (void)n;
#endif
    }
    ~Threads()
    {
#ifdef _OPENMP
        omp_set_num_threads(prev);
#endif
    }
    int prev = 1;
};

// ------------------------------------------------------------- REF-EXACT ----
//
// Restates src/svgf_denoise.slang.  Images are dense row-major arrays of 4
// (rgba16f images) or 2 (rg16f moments) channels.

template <class T> struct RefConst {
    // src/svgf_denoise.slang:118 (WAVELET_KERNEL), :137, :144, :150.
    static constexpr float kernel[5] = {1.0f / 16.0f, 4.0f / 16.0f, 6.0f / 16.0f, 4.0f / 16.0f, 1.0f / 16.0f};
};

// Pass 0, src/svgf_denoise.slang:176-191.
template <class T>
void ref_init(int w, int h, const T* raw, const T* mom_prev, T* mom_curr, T* wav_a, T alpha_m, T var_eps, bool f16)
{
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t i = size_t(y) * w + x;
            T r = raw[4 * i + 0], g = raw[4 * i + 1], b = raw[4 * i + 2];
            T l = lum(r, g, b);
            T m1p = mom_prev[2 * i + 0], m2p = mom_prev[2 * i + 1];
            // Slang lerp(a, b, t) = a + (b - a) * t.
            T m1 = m1p + (l - m1p) * alpha_m;
            T m2 = m2p + (l * l - m2p) * alpha_m;
            // Slang max() on a NaN first operand returns the other operand
            // (IEEE maxNum), as std::fmax does; the fp16 moments overflow to
            // inf / NaN for luminance above ~256 and this keeps that path exact.
            T var = std::fmax(m2 - m1 * m1, T(0));
            mom_curr[2 * i + 0] = q16(m1, f16);
            mom_curr[2 * i + 1] = q16(m2, f16);
            wav_a[4 * i + 0] = q16(r, f16);
            wav_a[4 * i + 1] = q16(g, f16);
            wav_a[4 * i + 2] = q16(b, f16);
            wav_a[4 * i + 3] = q16(T(std::sqrt(var + var_eps)), f16);
        }
    }
}

// Passes 1..3, src/svgf_denoise.slang:209-274.  `final_pass` selects the
// denoised_indirect write (alpha = 1, :264-267); otherwise alpha carries the
// centre's sqrt-variance unchanged (:268-273).
template <class T>
void ref_level(int w, int h, const T* src, T* dst, int stride, bool final_pass, T phi, T var_eps, bool f16)
{
    const int max_x = w - 1, max_y = h - 1;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t i = size_t(y) * w + x;
            T cr = src[4 * i + 0], cg = src[4 * i + 1], cb = src[4 * i + 2], ca = src[4 * i + 3];
            T cl = lum(cr, cg, cb);
            T sigma = std::fmax(phi * ca, var_eps);
            T sr = 0, sg = 0, sb = 0, ws = 0;
            for (int dy = -2; dy <= 2; ++dy) {
                for (int dx = -2; dx <= 2; ++dx) {
                    int sx = clampi(x + dx * stride, 0, max_x);
                    int sy = clampi(y + dy * stride, 0, max_y);
                    size_t j = size_t(sy) * w + sx;
                    T qr = src[4 * j + 0], qg = src[4 * j + 1], qb = src[4 * j + 2];
                    T ql = lum(qr, qg, qb);
                    T kw = T(RefConst<T>::kernel[dx + 2]) * T(RefConst<T>::kernel[dy + 2]);
                    T diff = std::fabs(ql - cl);
                    T ew = std::exp(-diff / sigma);
                    T tw = kw * ew;
                    sr += qr * tw;
                    sg += qg * tw;
                    sb += qb * tw;
                    ws += tw;
                }
            }
            T fr, fg, fb;
            if (ws > T(1e-6f)) {
                fr = sr / ws;
                fg = sg / ws;
                fb = sb / ws;
            } else {
                fr = cr;
                fg = cg;
                fb = cb;
            }
            dst[4 * i + 0] = q16(fr, f16);
            dst[4 * i + 1] = q16(fg, f16);
            dst[4 * i + 2] = q16(fb, f16);
            dst[4 * i + 3] = final_pass ? T(1) : q16(ca, f16);
        }
    }
}

// One reference frame: init, then `levels` wavelet passes at strides 1, 2, 4, ...
// ping-ponging a -> b -> a -> ... with the last pass writing `out`
// (src/main.cpp:929-944; src/svgf_denoise.slang:200-204).
template <class T>
void ref_frame(int w, int h, const T* raw, const T* mom_prev, T* mom_curr, T* out, int levels, T phi, T alpha_m, T var_eps,
               bool f16)
{
    size_t n = size_t(w) * h;
    std::vector<T> a(4 * n), b(4 * n);
    ref_init(w, h, raw, mom_prev, mom_curr, a.data(), alpha_m, var_eps, f16);
    T* src = a.data();
    T* oth = b.data();
    for (int lv = 0; lv < levels; ++lv) {
        bool last = lv == levels - 1;
        T* dst = last ? out : oth;
        ref_level(w, h, src, dst, 1 << lv, last, phi, var_eps, f16);
        std::swap(src, oth);
    }
    if (levels == 0) {
        // No wavelet pass: the reference would never write its output.  Define
        // the output as the init image with alpha forced to 1.
        for (size_t i = 0; i < n; ++i) {
            out[4 * i + 0] = a[4 * i + 0];
            out[4 * i + 1] = a[4 * i + 1];
            out[4 * i + 2] = a[4 * i + 2];
            out[4 * i + 3] = T(1);
        }
    }
}

// ------------------------------------------------------------------ FULL ----

struct FullParams {
    double alpha;           // colour EMA weight
    double moments_alpha;   // moment EMA weight
    double sigma_l;         // luminance edge-stop scale
    double sigma_n;         // normal edge-stop exponent
    double sigma_z;         // depth edge-stop scale
    int32_t levels;         // a-trous levels (strides 1, 2, 4, ...)
    int32_t max_history;    // history-length cap
    int32_t fallback_frames;// spatial variance below this history length
    int32_t reserved;
};

// Stores of the FULL algorithm that the FP16 storage form rounds: the oracle
// emulates each one separately, so that its share of the error against the
// float64 result can be measured on its own.
enum : int {
    Q_INPUT = 1,   // radiance input rounded to binary16
    Q_NORMAL = 2,  // guide normals as octahedral 2 x 16-bit codes
    Q_TC = 4,      // temporally integrated colour (the level-0 input) in binary16
    Q_HIST = 8,    // colour history in binary16
    Q_MOM = 16,    // luminance moments in binary16
    Q_RECORD = 32, // a-trous scratch records (colour, variance) in binary16
    Q_OUTPUT = 64, // the denoised output in binary16
};

// Constants of the FULL algorithm (shared verbatim with the CUDA kernels).
constexpr float kEpsL = 1e-4f;         // luminance edge-stop denominator floor
constexpr float kEpsZ = 1e-3f;         // depth edge-stop denominator floor (metres)
constexpr float kDepthRel = 0.05f;     // reprojection depth test: relative term
constexpr float kDepthGrad = 4.0f;     // reprojection depth test: gradient term
constexpr float kDepthAbs = 0.1f;      // reprojection depth test: absolute term
constexpr float kNormalCos = 0.9f;     // reprojection normal test: min cosine (tested squared, 0.81)
constexpr float kB3[5] = {1.0f / 16.0f, 1.0f / 4.0f, 3.0f / 8.0f, 1.0f / 4.0f, 1.0f / 16.0f};
constexpr float kG3[3] = {0.25f, 0.5f, 0.25f};

// One-sided depth difference with the smaller magnitude (0 when the image is
// one pixel wide in that axis).
template <class T> inline T grad1(const T* zrow, int x, int w, int step)
{
    bool has_l = x > 0, has_r = x < w - 1;
    T z = zrow[0];
    T dl = has_l ? z - zrow[-step] : T(0);
    T dr = has_r ? zrow[step] - z : T(0);
    if (has_l && has_r) return std::fabs(dl) <= std::fabs(dr) ? dl : dr;
    if (has_l) return dl;
    if (has_r) return dr;
    return T(0);
}

// max(0, d)^sigma_n.  sigma_n = 2^k (k <= 10) uses k squarings, as the GPU does.
template <class T> inline T normal_weight(T d, double sigma_n)
{
    if (!(d > T(0))) return T(0);
    double s = sigma_n;
    int k = -1;
    for (int i = 0; i <= 10; ++i)
        if (s == double(1 << i)) k = i;
    if (k >= 0) {
        T v = d;
        for (int i = 0; i < k; ++i) v = v * v;
        return v;
    }
    return T(std::exp2(T(sigma_n) * std::log2(d)));
}

template <class T> struct FullBuffers {
    // guide: n.xyz, z ; hist: rgb, len ; mom: mu, var ; col: rgb, var ; tc: rgb, len
    std::vector<T> tc, colA, colB, gx, gy;
};

template <class T>
void full_frame(const FullParams& P, int w, int h, const T* radiance4, const T* depth, const T* normal3, const T* motion2,
                const T* guide_prev, const T* hist_prev, const T* mom_prev, T* guide_cur, T* hist_cur, T* mom_cur,
                T* out4, T* var_out, int q)
{
    // Which stores of the FP16 storage form are emulated (a mask of the Q_* bits).
    const bool q_in = q & Q_INPUT, q_nrm = q & Q_NORMAL, q_tc = q & Q_TC, q_hist = q & Q_HIST, q_mom = q & Q_MOM,
               q_rec = q & Q_RECORD, q_out = q & Q_OUTPUT;
    const size_t n = size_t(w) * h;
    FullBuffers<T> B;
    B.tc.resize(4 * n);
    B.colA.resize(4 * n);
    B.colB.resize(4 * n);
    B.gx.resize(n);
    B.gy.resize(n);
    const T alpha = T(P.alpha), alpha_m = T(P.moments_alpha);
    const int cap = P.max_history;

    // ---- K1: guide, temporal reprojection, history length, colour + moment EMA.
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t i = size_t(y) * w + x;
            T nx = normal3[3 * i + 0], ny = normal3[3 * i + 1], nz = normal3[3 * i + 2];
            T z = q32(depth[i], q_nrm);
            if (q_nrm) oct16_roundtrip(nx, ny, nz);
            guide_cur[4 * i + 0] = nx;
            guide_cur[4 * i + 1] = ny;
            guide_cur[4 * i + 2] = nz;
            guide_cur[4 * i + 3] = z;
        }
    }
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t i = size_t(y) * w + x;
            const T* zr = guide_cur + 4 * i + 3;
            B.gx[i] = grad1(zr, x, w, 4);
            B.gy[i] = grad1(zr, y, h, 4 * w);
        }
    }
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t i = size_t(y) * w + x;
            T cr = q16(radiance4[4 * i + 0], q_in), cg = q16(radiance4[4 * i + 1], q_in), cb = q16(radiance4[4 * i + 2], q_in);
            T nx = guide_cur[4 * i + 0], ny = guide_cur[4 * i + 1], nz = guide_cur[4 * i + 2], z = guide_cur[4 * i + 3];
            T gsum = std::fabs(B.gx[i]) + std::fabs(B.gy[i]);
            T ztol = T(kDepthRel) * z + T(kDepthGrad) * gsum + T(kDepthAbs);
            // Previous-frame position of this pixel's centre, minus 0.5.
            T px = T(x) + motion2[2 * i + 0];
            T py = T(y) + motion2[2 * i + 1];
            T fx0 = std::floor(px), fy0 = std::floor(py);
            T fx = px - fx0, fy = py - fy0;
            // Integer tap origin; coordinates far outside the image are
            // clamped before conversion so that the conversion is defined.
            T lim = T(1 << 30);
            int x0 = int(std::max(-lim, std::min(lim, fx0)));
            int y0 = int(std::max(-lim, std::min(lim, fy0)));
            T bw[4] = {(T(1) - fx) * (T(1) - fy), fx * (T(1) - fy), (T(1) - fx) * fy, fx * fy};
            int tx[4] = {x0, x0 + 1, x0, x0 + 1};
            int ty[4] = {y0, y0, y0 + 1, y0 + 1};
            T sw = 0;
            T hr = 0, hg = 0, hb = 0, hmu = 0;
            int lmax = 0;
            bool ok[4];
            size_t ti[4];
            for (int k = 0; k < 4; ++k) {
                ok[k] = false;
                ti[k] = 0;
                if (tx[k] < 0 || ty[k] < 0 || tx[k] >= w || ty[k] >= h) continue;
                size_t j = size_t(ty[k]) * w + tx[k];
                ti[k] = j;
                T len_t = hist_prev[4 * j + 3];
                if (!(len_t > T(0))) continue;
                T zt = guide_prev[4 * j + 3];
                if (!(std::fabs(zt - z) <= ztol)) continue;
                if (!normal_close(guide_prev[4 * j + 0], guide_prev[4 * j + 1], guide_prev[4 * j + 2], nx, ny, nz))
                    continue;
                ok[k] = true;
                sw += bw[k];
                hr += bw[k] * hist_prev[4 * j + 0];
                hg += bw[k] * hist_prev[4 * j + 1];
                hb += bw[k] * hist_prev[4 * j + 2];
                hmu += bw[k] * mom_prev[2 * j + 0];
                lmax = std::max(lmax, int(len_t));
            }
            T l = lum(cr, cg, cb);
            T outr, outg, outb, mu, var;
            int len;
            if (sw > T(0)) {
                T inv = T(1) / sw;
                hr *= inv;
                hg *= inv;
                hb *= inv;
                hmu *= inv;
                // Mixture variance of the taps, mean-centred.
                T hv = 0;
                for (int k = 0; k < 4; ++k) {
                    if (!ok[k]) continue;
                    T dm = mom_prev[2 * ti[k] + 0] - hmu;
                    hv += bw[k] * (mom_prev[2 * ti[k] + 1] + dm * dm);
                }
                hv *= inv;
                len = std::min(lmax + 1, cap);
                T ac = std::max(alpha, T(1) / T(len));
                T am = std::max(alpha_m, T(1) / T(len));
                outr = hr + ac * (cr - hr);
                outg = hg + ac * (cg - hg);
                outb = hb + ac * (cb - hb);
                T dl = l - hmu;
                mu = hmu + am * dl;
                var = (T(1) - am) * (hv + am * dl * dl);
            } else {
                len = 1;
                outr = cr;
                outg = cg;
                outb = cb;
                mu = l;
                var = T(0);
            }
            B.tc[4 * i + 0] = q16(outr, q_tc);
            B.tc[4 * i + 1] = q16(outg, q_tc);
            B.tc[4 * i + 2] = q16(outb, q_tc);
            B.tc[4 * i + 3] = T(len);
            mom_cur[2 * i + 0] = q16s(mu, q_mom);
            mom_cur[2 * i + 1] = q16s(var, q_mom);
        }
    }

    // ---- K2: variance (temporal, or 7x7 spatial for short histories).
    const T sz = T(P.sigma_z);
#pragma omp parallel for schedule(static)
    for (int y = 0; y < h; ++y) {
        for (int x = 0; x < w; ++x) {
            size_t i = size_t(y) * w + x;
            int len = int(B.tc[4 * i + 3]);
            T var;
            if (len < P.fallback_frames) {
                T nx, ny, nz;
                unit_normal(guide_cur + 4 * i, q_nrm, nx, ny, nz);
                T z = guide_cur[4 * i + 3];
                T gx = B.gx[i], gy = B.gy[i];
                T mup = mom_cur[2 * i + 0];
                T s0 = 0, s1 = 0, s2 = 0;
                for (int dy = -3; dy <= 3; ++dy) {
                    int qy = y + dy;
                    if (qy < 0 || qy >= h) continue;
                    for (int dx = -3; dx <= 3; ++dx) {
                        int qx = x + dx;
                        if (qx < 0 || qx >= w) continue;
                        size_t j = size_t(qy) * w + qx;
                        T qx_, qy_, qz_;
                        unit_normal(guide_cur + 4 * j, q_nrm, qx_, qy_, qz_);
                        T d = qx_ * nx + qy_ * ny + qz_ * nz;
                        T wn = normal_weight(d, P.sigma_n);
                        if (!(wn > T(0))) continue;
                        T den = sz * std::fabs(T(dx) * gx + T(dy) * gy) + T(kEpsZ);
                        T ez = std::fabs(guide_cur[4 * j + 3] - z) / den;
                        T wgt = wn * std::exp(-ez);
                        T dm = mom_cur[2 * j + 0] - mup;
                        s0 += wgt;
                        s1 += wgt * dm;
                        s2 += wgt * (dm * dm + mom_cur[2 * j + 1]);
                    }
                }
                if (s0 > T(0)) {
                    T m1 = s1 / s0;
                    var = std::max(T(0), s2 / s0 - m1 * m1);
                } else {
                    var = mom_cur[2 * i + 1];
                }
            } else {
                var = mom_cur[2 * i + 1];
            }
            B.colA[4 * i + 0] = B.tc[4 * i + 0];
            B.colA[4 * i + 1] = B.tc[4 * i + 1];
            B.colA[4 * i + 2] = B.tc[4 * i + 2];
            B.colA[4 * i + 3] = q16s(var, q_rec);
        }
    }

    // ---- K3: a-trous levels.
    const T sl = T(P.sigma_l);
    T* src = B.colA.data();
    T* dst = B.colB.data();
    for (int lv = 0; lv < P.levels; ++lv) {
        const int s = 1 << lv;
        const bool last = lv == P.levels - 1;
#pragma omp parallel for schedule(static)
        for (int y = 0; y < h; ++y) {
            for (int x = 0; x < w; ++x) {
                size_t i = size_t(y) * w + x;
                T cr = src[4 * i + 0], cg = src[4 * i + 1], cb = src[4 * i + 2], cv = src[4 * i + 3];
                T cl = lum(cr, cg, cb);
                T nx, ny, nz;
                unit_normal(guide_cur + 4 * i, q_nrm, nx, ny, nz);
                T z = guide_cur[4 * i + 3];
                T gx = B.gx[i], gy = B.gy[i];
                // 3x3 Gaussian of the variance around the centre (inside taps only).
                T gv = 0, gw = 0;
                for (int a = -1; a <= 1; ++a) {
                    int qy = y + a;
                    if (qy < 0 || qy >= h) continue;
                    for (int b = -1; b <= 1; ++b) {
                        int qx = x + b;
                        if (qx < 0 || qx >= w) continue;
                        T k = T(kG3[a + 1]) * T(kG3[b + 1]);
                        gv += k * src[4 * (size_t(qy) * w + qx) + 3];
                        gw += k;
                    }
                }
                gv = gv / gw;
                T inv_l = T(1) / (sl * std::sqrt(std::max(gv, T(0))) + T(kEpsL));
                T sr = 0, sg = 0, sb = 0, sw = 0, sv = 0;
                for (int dy = -2; dy <= 2; ++dy) {
                    int qy = y + dy * s;
                    if (qy < 0 || qy >= h) continue;
                    for (int dx = -2; dx <= 2; ++dx) {
                        int qx = x + dx * s;
                        if (qx < 0 || qx >= w) continue;
                        size_t j = size_t(qy) * w + qx;
                        T ux, uy, uz;
                        unit_normal(guide_cur + 4 * j, q_nrm, ux, uy, uz);
                        T d = ux * nx + uy * ny + uz * nz;
                        T wn = normal_weight(d, P.sigma_n);
                        if (!(wn > T(0))) continue;
                        T qr = src[4 * j + 0], qg = src[4 * j + 1], qb = src[4 * j + 2], qv = src[4 * j + 3];
                        T ql = lum(qr, qg, qb);
                        T el = std::fabs(cl - ql) * inv_l;
                        T den = sz * std::fabs(T(s) * (T(dx) * gx + T(dy) * gy)) + T(kEpsZ);
                        T ez = std::fabs(z - guide_cur[4 * j + 3]) / den;
                        T wgt = T(kB3[dx + 2]) * T(kB3[dy + 2]) * wn * std::exp(-(el + ez));
                        sr += wgt * qr;
                        sg += wgt * qg;
                        sb += wgt * qb;
                        sw += wgt;
                        sv += wgt * wgt * qv;
                    }
                }
                T orr, og, ob, ov;
                if (sw > T(0)) {
                    T inv = T(1) / sw;
                    orr = sr * inv;
                    og = sg * inv;
                    ob = sb * inv;
                    ov = sv * (inv * inv);
                } else {
                    orr = cr;
                    og = cg;
                    ob = cb;
                    ov = cv;
                }
                if (lv == 0) {
                    hist_cur[4 * i + 0] = q16(orr, q_hist);
                    hist_cur[4 * i + 1] = q16(og, q_hist);
                    hist_cur[4 * i + 2] = q16(ob, q_hist);
                    hist_cur[4 * i + 3] = B.tc[4 * i + 3];
                }
                if (last) {
                    out4[4 * i + 0] = q16(orr, q_out);
                    out4[4 * i + 1] = q16(og, q_out);
                    out4[4 * i + 2] = q16(ob, q_out);
                    out4[4 * i + 3] = T(1);
                    if (var_out) var_out[i] = ov;
                } else {
                    dst[4 * i + 0] = q16(orr, q_rec);
                    dst[4 * i + 1] = q16(og, q_rec);
                    dst[4 * i + 2] = q16(ob, q_rec);
                    dst[4 * i + 3] = q16s(ov, q_rec);
                }
            }
        }
        std::swap(src, dst);
    }
    if (P.levels == 0) {
        for (size_t i = 0; i < n; ++i) {
            for (int c = 0; c < 3; ++c) {
                hist_cur[4 * i + c] = B.colA[4 * i + c];
                out4[4 * i + c] = B.colA[4 * i + c];
            }
            hist_cur[4 * i + 3] = B.tc[4 * i + 3];
            out4[4 * i + 3] = T(1);
            if (var_out) var_out[i] = B.colA[4 * i + 3];
        }
    }
}

} // namespace

extern "C" {

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

// REF-EXACT frame.  raw: h*w*4, mom_prev/mom_curr: h*w*2, out: h*w*4.
int orc_ref_frame_f32(int w, int h, const float* raw, const float* mom_prev, float* mom_curr, float* out, int levels,
                      float phi, float alpha_m, float var_eps, int fp16_store, int threads)
{
    if (w <= 0 || h <= 0 || levels < 0 || levels > 12) return 1;
    Threads t(threads);
    ref_frame<float>(w, h, raw, mom_prev, mom_curr, out, levels, phi, alpha_m, var_eps, fp16_store != 0);
    return 0;
}

int orc_ref_frame_f64(int w, int h, const double* raw, const double* mom_prev, double* mom_curr, double* out,
                      int levels, double phi, double alpha_m, double var_eps, int fp16_store, int threads)
{
    if (w <= 0 || h <= 0 || levels < 0 || levels > 12) return 1;
    Threads t(threads);
    ref_frame<double>(w, h, raw, mom_prev, mom_curr, out, levels, phi, alpha_m, var_eps, fp16_store != 0);
    return 0;
}

// FULL frame.  radiance: h*w*4, depth: h*w, normal: h*w*3, motion: h*w*2;
// guide: h*w*4 (n.xyz, z), hist: h*w*4 (rgb, len), mom: h*w*2 (mu, var),
// out: h*w*4, var_out: h*w or NULL.  fp16_store: the Q_* mask of the stores
// that are rounded as the FP16 storage form rounds them (0: none).
int orc_full_frame_f32(const FullParams* p, int w, int h, const float* radiance, const float* depth,
                       const float* normal, const float* motion, const float* guide_prev, const float* hist_prev,
                       const float* mom_prev, float* guide_cur, float* hist_cur, float* mom_cur, float* out,
                       float* var_out, int fp16_store, int threads)
{
    if (!p || w <= 0 || h <= 0 || p->levels < 0 || p->levels > 12 || p->max_history < 1) return 1;
    Threads t(threads);
    full_frame<float>(*p, w, h, radiance, depth, normal, motion, guide_prev, hist_prev, mom_prev, guide_cur, hist_cur,
                      mom_cur, out, var_out, fp16_store);
    return 0;
}

int orc_full_frame_f64(const FullParams* p, int w, int h, const double* radiance, const double* depth,
                       const double* normal, const double* motion, const double* guide_prev, const double* hist_prev,
                       const double* mom_prev, double* guide_cur, double* hist_cur, double* mom_cur, double* out,
                       double* var_out, int fp16_store, int threads)
{
    if (!p || w <= 0 || h <= 0 || p->levels < 0 || p->levels > 12 || p->max_history < 1) return 1;
    Threads t(threads);
    full_frame<double>(*p, w, h, radiance, depth, normal, motion, guide_prev, hist_prev, mom_prev, guide_cur, hist_cur,
                       mom_cur, out, var_out, fp16_store);
    return 0;
}

// Octahedral snorm16 encode / decode of n normals (for tests of the GPU codec).
void orc_oct16_encode(int n, const float* nrm3, int16_t* enc2)
{
    for (int i = 0; i < n; ++i) oct16_encode(nrm3[3 * i], nrm3[3 * i + 1], nrm3[3 * i + 2], enc2[2 * i], enc2[2 * i + 1]);
}

void orc_oct16_decode(int n, const int16_t* enc2, float* nrm3)
{
    for (int i = 0; i < n; ++i) oct16_decode(enc2[2 * i], enc2[2 * i + 1], nrm3[3 * i], nrm3[3 * i + 1], nrm3[3 * i + 2]);
}

} // extern "C"
