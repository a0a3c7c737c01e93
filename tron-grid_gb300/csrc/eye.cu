// Eye-frame readback (include/tg_eye.h) on sm_103a.
//
// One launch per frame packs every eye into a device copy of the frame's slot:
// the work is the concatenation of the eyes' pixel groups (4 consecutive
// pixels of one eye per thread), an eye is found by binary search over the
// group prefix sums of a small per-slot table, and the thread writes its 12 RGB
// bytes as three aligned 32-bit stores and its 4 depths as one 16-byte store (a
// group cut short by the end of an eye stores byte by byte).  One copy-engine
// transfer then moves the whole slot to the page-locked host ring: SM stores
// into host memory reach only a few GB/s over the chip-to-chip link, the copy
// engines its full bandwidth.  Eyes and slots start on 16-byte boundaries.
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <new>
#include <vector>

#include "svgf_internal.h"
#include "tg_eye.h"

namespace tg {
namespace {

struct EyeEntry {
    const char* col;
    const char* dep;
    long long col_pitch, dep_pitch;
    long long rgb_off, dep_off;  // byte offsets within a slot
    int w, h, fmt, pad;
};

inline size_t al16(size_t v) { return (v + 15) / 16 * 16; }

__device__ __forceinline__ uint32_t q8(float f)
{
    f = f < 0.f ? 0.f : (f > 1.f ? 1.f : f);
    return __float2uint_rn(__fmul_rn(f, 255.0f));
}

// r | g << 8 | b << 16 of pixel (x, y)
__device__ __forceinline__ uint32_t load_rgb(const EyeEntry& e, int x, int y)
{
    const char* row = e.col + y * e.col_pitch;
    if (e.fmt == TG_FMT_RGBA8 || e.fmt == TG_FMT_BGRA8) {
        const uint32_t v = reinterpret_cast<const uint32_t*>(row)[x];
        return e.fmt == TG_FMT_RGBA8 ? (v & 0xffffffu) : (((v >> 16) & 0xffu) | (v & 0xff00u) | ((v & 0xffu) << 16));
    }
    float r, g, b;
    if (e.fmt == TG_FMT_RGBA16F) {
        const uint2 u = reinterpret_cast<const uint2*>(row)[x];
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&u.x));
        r = a.x;
        g = a.y;
        b = __half2float(*reinterpret_cast<const __half*>(&u.y));
    } else {
        const float4 v = reinterpret_cast<const float4*>(row)[x];
        r = v.x;
        g = v.y;
        b = v.z;
    }
    return q8(r) | (q8(g) << 8) | (q8(b) << 16);
}

__global__ void __launch_bounds__(256) k_eye_pack(const EyeEntry* ents, const long long* prefix, int n, char* slot)
{
    const long long g = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= prefix[n]) return;
    int lo = 0, hi = n;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (prefix[mid] <= g)
            lo = mid;
        else
            hi = mid;
    }
    const EyeEntry e = ents[lo];
    const long long npx = (long long)e.w * e.h;
    const long long p0 = (g - prefix[lo]) * 4;
    const int cnt = int(min(4LL, npx - p0));
    uint32_t rgb[4];
    float dep[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        if (k < cnt) {
            const int x = int((p0 + k) % e.w), y = int((p0 + k) / e.w);
            rgb[k] = load_rgb(e, x, y);
            dep[k] = reinterpret_cast<const float*>(e.dep + y * e.dep_pitch)[x];
        } else {
            rgb[k] = 0;
            dep[k] = 0.f;
        }
    }
    char* rp = slot + e.rgb_off + 3 * p0;
    float* dp = reinterpret_cast<float*>(slot + e.dep_off) + p0;
    if (cnt == 4) {
        uint32_t* w = reinterpret_cast<uint32_t*>(rp);
        w[0] = rgb[0] | (rgb[1] << 24);
        w[1] = (rgb[1] >> 8) | (rgb[2] << 16);
        w[2] = (rgb[2] >> 16) | (rgb[3] << 8);
        *reinterpret_cast<float4*>(dp) = make_float4(dep[0], dep[1], dep[2], dep[3]);
    } else {
        for (int k = 0; k < cnt; ++k) {
            rp[3 * k] = char(rgb[k] & 0xff);
            rp[3 * k + 1] = char((rgb[k] >> 8) & 0xff);
            rp[3 * k + 2] = char((rgb[k] >> 16) & 0xff);
            dp[k] = dep[k];
        }
    }
}

} // namespace
} // namespace tg

using namespace tg;

struct tg_eye {
    int device = 0;
    uint32_t n = 0, ring = 3;
    std::vector<uint32_t> w, h;
    std::vector<double> fov;
    std::vector<long long> rgb_off, dep_off;
    size_t slot_bytes = 0;
    char* host = nullptr;      // ring * slot_bytes, page-locked
    char* dev = nullptr;       // ring * slot_bytes in device memory (the packed slots before their copy)
    bool own_host = false;
    size_t table_bytes = 0;
    std::vector<char*> tab_host, tab_dev;
    std::vector<cudaEvent_t> ev;
    std::vector<long long> slot_frame;
    long long last = -1;
};

namespace {

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev)
    {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard()
    {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

size_t layout(uint32_t n, const uint32_t* w, const uint32_t* h, std::vector<long long>* ro, std::vector<long long>* dof)
{
    size_t off = 0;
    for (uint32_t i = 0; i < n; ++i) {
        const size_t px = size_t(w[i]) * h[i];
        if (ro) ro->push_back((long long)off);
        off += al16(px * 3);
        if (dof) dof->push_back((long long)off);
        off += al16(px * 4);
    }
    return off;
}

void release(tg_eye* s)
{
    for (cudaEvent_t e : s->ev)
        if (e) cudaEventDestroy(e);
    for (char* p : s->tab_host)
        if (p) cudaFreeHost(p);
    for (char* p : s->tab_dev)
        if (p) cudaFree(p);
    if (s->host) {
        if (s->own_host)
            cudaFreeHost(s->host);
        else
            cudaHostUnregister(s->host);
    }
    if (s->dev) cudaFree(s->dev);
    cudaGetLastError();
}

} // namespace

uint64_t tg_eye_host_bytes(uint32_t n_eyes, const uint32_t* widths, const uint32_t* heights, uint32_t ring)
{
    if (!widths || !heights || n_eyes == 0) return 0;
    return uint64_t(layout(n_eyes, widths, heights, nullptr, nullptr)) * (ring ? ring : 3);
}

int tg_eye_create(const tg_eye_desc* d, tg_eye** out)
{
    if (!out) return fail(TG_ERR_INVALID, "null output handle");
    *out = nullptr;
    if (!d || !d->widths || !d->heights || d->n_eyes == 0 || d->n_eyes > TG_EYE_MAX_EYES)
        return fail(TG_ERR_INVALID, "need 1..%d eyes with sizes", TG_EYE_MAX_EYES);
    unsigned long long total_px = 0;
    for (uint32_t i = 0; i < d->n_eyes; ++i) {
        if (d->widths[i] == 0 || d->heights[i] == 0 || d->widths[i] > 16384 || d->heights[i] > 16384)
            return fail(TG_ERR_INVALID, "eye %u size %ux%u outside 1..16384", i, d->widths[i], d->heights[i]);
        total_px += (unsigned long long)d->widths[i] * d->heights[i];
    }
    if (total_px > (1ull << 32)) return fail(TG_ERR_INVALID, "%llu eye pixels per frame exceed 2^32", total_px);
    int dev = d->device;
    if (dev < 0 && cudaGetDevice(&dev) != cudaSuccess) return fail(TG_ERR_CUDA, "no current CUDA device");
    DeviceGuard g(dev);
    tg_eye* s = new (std::nothrow) tg_eye();
    if (!s) return fail(TG_ERR_OOM, "host allocation failed");
    s->device = dev;
    s->n = d->n_eyes;
    s->ring = d->ring ? d->ring : 3;
    s->w.assign(d->widths, d->widths + s->n);
    s->h.assign(d->heights, d->heights + s->n);
    s->fov.assign(s->n, 0.0);
    if (d->fov_horizontal) s->fov.assign(d->fov_horizontal, d->fov_horizontal + s->n);
    s->slot_bytes = layout(s->n, d->widths, d->heights, &s->rgb_off, &s->dep_off);
    const size_t total = s->slot_bytes * s->ring;
    auto bail = [&](int st) {
        release(s);
        delete s;
        return st;
    };
    if (d->host_buffer) {
        if (d->host_bytes < total) return bail(fail(TG_ERR_INVALID, "host_buffer holds %llu bytes, %zu needed",
                                                    (unsigned long long)d->host_bytes, total));
        if (reinterpret_cast<uintptr_t>(d->host_buffer) % 16) return bail(fail(TG_ERR_INVALID, "host_buffer not 16-byte aligned"));
        if (cudaHostRegister(d->host_buffer, total, cudaHostRegisterPortable) != cudaSuccess) {
            cudaGetLastError();
            return bail(fail(TG_ERR_CUDA, "cudaHostRegister of the caller's buffer failed"));
        }
        s->host = static_cast<char*>(d->host_buffer);
    } else {
        if (cudaHostAlloc(&s->host, total, cudaHostAllocPortable) != cudaSuccess) {
            cudaGetLastError();
            s->host = nullptr;
            return bail(fail(TG_ERR_OOM, "cudaHostAlloc of %zu bytes failed", total));
        }
        s->own_host = true;
        std::memset(s->host, 0, total);
    }
    if (cudaMalloc(&s->dev, total) != cudaSuccess) {
        cudaGetLastError();
        s->dev = nullptr;
        return bail(fail(TG_ERR_OOM, "cudaMalloc of %zu eye slot bytes failed", total));
    }
    s->table_bytes = al16(sizeof(EyeEntry) * s->n) + sizeof(long long) * (s->n + 1);
    s->tab_host.assign(s->ring, nullptr);
    s->tab_dev.assign(s->ring, nullptr);
    s->ev.assign(s->ring, nullptr);
    s->slot_frame.assign(s->ring, -1);
    for (uint32_t k = 0; k < s->ring; ++k) {
        if (cudaHostAlloc(&s->tab_host[k], s->table_bytes, cudaHostAllocPortable) != cudaSuccess ||
            cudaMalloc(&s->tab_dev[k], s->table_bytes) != cudaSuccess ||
            cudaEventCreateWithFlags(&s->ev[k], cudaEventDisableTiming) != cudaSuccess) {
            cudaGetLastError();
            return bail(fail(TG_ERR_OOM, "eye tables could not be allocated"));
        }
    }
    *out = s;
    return TG_OK;
}

int tg_eye_submit(tg_eye* s, uint64_t frame, const tg_image* colour, const tg_image* depth, void* stream)
{
    if (!s || !colour || !depth) return fail(TG_ERR_INVALID, "null handle or images");
    if (s->last >= 0 && (long long)frame != s->last + 1)
        return fail(TG_ERR_STATE, "frame %llu submitted after %lld (frames are submitted in order)",
                    (unsigned long long)frame, s->last);
    static const int kCol[] = {TG_FMT_BGRA8, TG_FMT_RGBA8, TG_FMT_RGBA16F, TG_FMT_RGBA32F};
    static const int kDep[] = {TG_FMT_R32F};
    for (uint32_t i = 0; i < s->n; ++i) {
        int st;
        if ((st = check_image("eye colour", colour[i], s->w[i], s->h[i], kCol, 4))) return st;
        if ((st = check_image("eye depth", depth[i], s->w[i], s->h[i], kDep, 1))) return st;
    }
    DeviceGuard g(s->device);
    const uint32_t k = uint32_t(frame % s->ring);
    // the table of this slot was last uploaded for frame - ring
    if (s->slot_frame[k] >= 0 && cudaEventSynchronize(s->ev[k]) != cudaSuccess)
        return fail(TG_ERR_CUDA, "eye slot wait failed");
    EyeEntry* ent = reinterpret_cast<EyeEntry*>(s->tab_host[k]);
    long long* pf = reinterpret_cast<long long*>(s->tab_host[k] + al16(sizeof(EyeEntry) * s->n));
    long long acc = 0;
    for (uint32_t i = 0; i < s->n; ++i) {
        const int cb = fmt_bytes(colour[i].format);
        EyeEntry& e = ent[i];
        e.col = static_cast<const char*>(colour[i].ptr);
        e.col_pitch = colour[i].pitch_bytes ? colour[i].pitch_bytes : (long long)cb * s->w[i];
        e.dep = static_cast<const char*>(depth[i].ptr);
        e.dep_pitch = depth[i].pitch_bytes ? depth[i].pitch_bytes : 4LL * s->w[i];
        e.rgb_off = (long long)(k * s->slot_bytes) + s->rgb_off[i];
        e.dep_off = (long long)(k * s->slot_bytes) + s->dep_off[i];
        e.w = int(s->w[i]);
        e.h = int(s->h[i]);
        e.fmt = colour[i].format;
        e.pad = 0;
        pf[i] = acc;
        acc += ((long long)s->w[i] * s->h[i] + 3) / 4;
    }
    pf[s->n] = acc;
    cudaStream_t cs = static_cast<cudaStream_t>(stream);
    if (cudaMemcpyAsync(s->tab_dev[k], s->tab_host[k], s->table_bytes, cudaMemcpyHostToDevice, cs) != cudaSuccess)
        return fail(TG_ERR_CUDA, "eye table upload failed");
    const EyeEntry* de = reinterpret_cast<const EyeEntry*>(s->tab_dev[k]);
    const long long* dpf = reinterpret_cast<const long long*>(s->tab_dev[k] + al16(sizeof(EyeEntry) * s->n));
    const unsigned blocks = unsigned((acc + 255) / 256);
    k_eye_pack<<<blocks, 256, 0, cs>>>(de, dpf, int(s->n), s->dev);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(TG_ERR_CUDA, "eye pack launch failed: %s", cudaGetErrorString(e));
    const size_t so = size_t(k) * s->slot_bytes;
    if (cudaMemcpyAsync(s->host + so, s->dev + so, s->slot_bytes, cudaMemcpyDeviceToHost, cs) != cudaSuccess)
        return fail(TG_ERR_CUDA, "eye slot copy failed");
    if (cudaEventRecord(s->ev[k], cs) != cudaSuccess) return fail(TG_ERR_CUDA, "eye event record failed");
    s->slot_frame[k] = (long long)frame;
    s->last = (long long)frame;
    return TG_OK;
}

int tg_eye_acquire(tg_eye* s, uint64_t frame, tg_vision_data* out)
{
    if (!s || !out) return fail(TG_ERR_INVALID, "null handle or output");
    const uint32_t k = uint32_t(frame % s->ring);
    if (s->slot_frame[k] != (long long)frame)
        return fail(TG_ERR_STATE, "frame %llu is not in the ring (never submitted, or overwritten)",
                    (unsigned long long)frame);
    DeviceGuard g(s->device);
    if (cudaEventSynchronize(s->ev[k]) != cudaSuccess) return fail(TG_ERR_CUDA, "eye frame wait failed");
    const char* base = s->host + size_t(k) * s->slot_bytes;
    for (uint32_t i = 0; i < s->n; ++i) {
        out[i].rgb = reinterpret_cast<const uint8_t*>(base + s->rgb_off[i]);
        out[i].depth = reinterpret_cast<const float*>(base + s->dep_off[i]);
        out[i].width = s->w[i];
        out[i].height = s->h[i];
        out[i].fov_horizontal = s->fov[i];
    }
    return TG_OK;
}

void tg_eye_destroy(tg_eye* s)
{
    if (!s) return;
    {
        DeviceGuard g(s->device);
        cudaDeviceSynchronize();
        release(s);
    }
    delete s;
}
