// CPU oracle for the volumetric-fog froxel filter.  TEST INFRASTRUCTURE ONLY:
// this file is the checker that the CUDA path is compared against (and the
// timed CPU baseline of the fog line); nothing in the product links, loads or
// calls it.
//
// A restatement of the reference shader `src/volumetric_filter.slang`
// (filterMain, lines 142-226) as the reference host drives it
// (`src/main.cpp:993-1005`: one invocation per froxel of a
// ceil(W/8) x ceil(H/8) x D grid, the (history, output) pair alternated by the
// caller between two images, `history_valid` 0 on the first frame), templated
// on the arithmetic type T (float for parity, double for accuracy):
//
//  1. 3x3 box mean of the injected froxels in the froxel's own slice, over the
//     neighbours inside the grid (lines 152-166);
//  2. without valid history, that mean is the output (lines 170-173);
//  3. the froxel centre is placed in the world: NDC of the column, view depth
//     of the slice from the logarithmic slice distribution, along the
//     normalised camera ray scaled by view_z / max(ray . forward, 1e-4)
//     (lines 74-106, 177);
//  4. it is projected with the previous view-projection; w <= 1e-4, a view
//     depth outside [near, far] or a position outside the grid keeps the
//     spatial mean (lines 178-213).  The previous x/y froxel coordinates are
//     taken in edge units ((ndc * 0.5 + 0.5) * W), the z coordinate in centre
//     units (t * D - 0.5), as the shader does;
//  5. trilinear fetch of the history with clamp-to-edge indices (lines
//     111-140) and out = history + (spatial - history) * alpha (lines 216-225).
//
// Matrices are column-major 4x4 (element (col, row) at index col * 4 + row,
// the reference's MathLib::Mat4 storage, `libs/math/include/math/matrix.hpp:26-47`);
// clip = M (x, y, z, 1) sums the four column terms left to right.  Images are
// float32 arrays of rgba texels, index ((z * H) + y) * W + x; fp16_store rounds
// every stored texel to binary16 (the reference's rgba16f froxel images,
// `src/main.cpp:1918-1924`).
//
// Compile with -ffp-contract=off (as the rest of the oracle).

#include <cmath>
#include <cstdint>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

template <class T> struct Fog {
    T ivp[16], pvp[16], cam[3];
    T alpha, znear, zfar;
    int W, H, D, valid;
};

template <class T> inline void mat_vec(const T* m, T x, T y, T z, T w, T o[4])
{
    for (int r = 0; r < 4; ++r) o[r] = m[0 * 4 + r] * x + m[1 * 4 + r] * y + m[2 * 4 + r] * z + m[3 * 4 + r] * w;
}

template <class T> inline T fpow(T a, T b) { return std::pow(a, b); }
template <class T> inline T flog(T a) { return std::log(a); }

inline float store_round(float v, bool f16) { return f16 ? static_cast<float>(static_cast<_Float16>(v)) : v; }

template <class T>
void fog_froxel(const Fog<T>& p, const float* raw, const float* hist, float* out, int x, int y, int z, bool f16)
{
    const int W = p.W, H = p.H, D = p.D;
    auto at = [&](int xx, int yy, int zz) { return ((size_t(zz) * H + yy) * W + xx) * 4; };
    // 1. spatial 3x3 mean (same slice)
    T s[4] = {0, 0, 0, 0}, n = 0;
    for (int dy = -1; dy <= 1; ++dy)
        for (int dx = -1; dx <= 1; ++dx) {
            const int qx = x + dx, qy = y + dy;
            if (qx < 0 || qx > W - 1 || qy < 0 || qy > H - 1) continue;
            const float* q = raw + at(qx, qy, z);
            for (int c = 0; c < 4; ++c) s[c] += T(q[c]);
            n += T(1);
        }
    const T cnt = n > T(1) ? n : T(1);
    T sp[4];
    for (int c = 0; c < 4; ++c) sp[c] = s[c] / cnt;
    float* o = out + at(x, y, z);
    auto emit = [&](const T* v) {
        for (int c = 0; c < 4; ++c) o[c] = store_round(float(v[c]), f16);
    };
    if (!p.valid) return emit(sp);

    // 3. froxel centre in the world
    const T u = (T(x) + T(0.5)) / T(W), v = (T(y) + T(0.5)) / T(H);
    const T nx = u * T(2) - T(1), ny = T(1) - v * T(2);
    const T tz = (T(z) + T(0.5)) / T(D);
    const T view_z = p.znear * fpow(p.zfar / p.znear, tz);
    T nh[4], fh[4];
    mat_vec(p.ivp, nx, ny, T(0), T(1), nh);
    mat_vec(p.ivp, T(0), T(0), T(0), T(1), fh);
    T ray[3], fwd[3];
    for (int k = 0; k < 3; ++k) {
        ray[k] = nh[k] / nh[3] - p.cam[k];
        fwd[k] = fh[k] / fh[3] - p.cam[k];
    }
    const T rl = std::sqrt(ray[0] * ray[0] + ray[1] * ray[1] + ray[2] * ray[2]);
    const T fl = std::sqrt(fwd[0] * fwd[0] + fwd[1] * fwd[1] + fwd[2] * fwd[2]);
    for (int k = 0; k < 3; ++k) {
        ray[k] = ray[k] / rl;
        fwd[k] = fwd[k] / fl;
    }
    T rdf = ray[0] * fwd[0] + ray[1] * fwd[1] + ray[2] * fwd[2];
    rdf = rdf > T(1e-4f) ? rdf : T(1e-4f);
    const T t = view_z / rdf;
    const T wx = p.cam[0] + ray[0] * t, wy = p.cam[1] + ray[1] * t, wz = p.cam[2] + ray[2] * t;

    // 4. previous-frame froxel coordinates
    T pc[4];
    mat_vec(p.pvp, wx, wy, wz, T(1), pc);
    if (pc[3] <= T(1e-4f)) return emit(sp);
    const T ndx = pc[0] / pc[3], ndy = pc[1] / pc[3];
    const T fx = (ndx * T(0.5) + T(0.5)) * T(W);
    const T fy = (-ndy * T(0.5) + T(0.5)) * T(H);
    const T pz = pc[3];
    if (pz < p.znear || pz > p.zfar) return emit(sp);
    const T lt = flog(pz / p.znear) / flog(p.zfar / p.znear);
    const T fz = lt * T(D) - T(0.5);
    if (fx < T(0) || fx >= T(W) || fy < T(0) || fy >= T(H) || fz < T(0) || fz >= T(D)) return emit(sp);

    // 5. trilinear history, clamp-to-edge
    const int ix = int(std::floor(fx)), iy = int(std::floor(fy)), iz = int(std::floor(fz));
    const T ax = fx - T(ix), ay = fy - T(iy), az = fz - T(iz);
    auto cl = [](int v, int hi) { return v < 0 ? 0 : (v > hi ? hi : v); };
    const int x0 = cl(ix, W - 1), x1 = cl(ix + 1, W - 1);
    const int y0 = cl(iy, H - 1), y1 = cl(iy + 1, H - 1);
    const int z0 = cl(iz, D - 1), z1 = cl(iz + 1, D - 1);
    T res[4];
    for (int c = 0; c < 4; ++c) {
        auto hv = [&](int xx, int yy, int zz) { return T(hist[at(xx, yy, zz) + c]); };
        auto lr = [](T a, T b, T w) { return a + (b - a) * w; };
        const T c00 = lr(hv(x0, y0, z0), hv(x1, y0, z0), ax);
        const T c10 = lr(hv(x0, y1, z0), hv(x1, y1, z0), ax);
        const T c01 = lr(hv(x0, y0, z1), hv(x1, y0, z1), ax);
        const T c11 = lr(hv(x0, y1, z1), hv(x1, y1, z1), ax);
        const T c0 = lr(c00, c10, ay), c1 = lr(c01, c11, ay);
        const T h = lr(c0, c1, az);
        res[c] = h + (sp[c] - h) * p.alpha;
    }
    emit(res);
}

template <class T> int fog_frame(const float* params, const float* raw, const float* hist, float* out, int fp16_store,
                                 int threads)
{
    // params: the 176-byte block as 44 floats / words (tg_fog_filter_params layout)
    Fog<T> p;
    for (int k = 0; k < 16; ++k) {
        p.ivp[k] = T(params[k]);
        p.pvp[k] = T(params[16 + k]);
    }
    for (int k = 0; k < 3; ++k) p.cam[k] = T(params[32 + k]);
    p.alpha = T(params[35]);
    uint32_t u[4];
    std::memcpy(u, params + 36, sizeof u);
    p.W = int(u[0]);
    p.H = int(u[1]);
    p.D = int(u[2]);
    p.valid = u[3] != 0;
    p.znear = T(params[40]);
    p.zfar = T(params[41]);
    if (p.W <= 0 || p.H <= 0 || p.D <= 0) return 1;
#ifdef _OPENMP
    const int prev = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
#pragma omp parallel for collapse(2) schedule(static)
    for (int z = 0; z < p.D; ++z)
        for (int y = 0; y < p.H; ++y)
            for (int x = 0; x < p.W; ++x) fog_froxel<T>(p, raw, hist, out, x, y, z, fp16_store != 0);
#ifdef _OPENMP
    omp_set_num_threads(prev);
#endif
    return 0;
}

} // namespace

extern "C" {

// One filter pass.  params: 44 x 4 bytes in the tg_fog_filter_params layout;
// raw / hist / out: D*H*W*4 float32.  dbl selects double arithmetic.
int orc_fog_filter(const float* params, const float* raw, const float* hist, float* out, int fp16_store, int dbl,
                   int threads)
{
    return dbl ? fog_frame<double>(params, raw, hist, out, fp16_store, threads)
               : fog_frame<float>(params, raw, hist, out, fp16_store, threads);
}

} // extern "C"
