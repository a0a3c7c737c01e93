// tg_svgf.hpp - C++ RAII wrappers over the C ABI of include/tg_svgf.h,
// tg_fog.h, tg_post.h and tg_eye.h.
//
// SvgfDenoiser mirrors how the reference engine uses its SVGF pass: one object
// per swapchain (src/main.cpp:1326-1397 creates the pass's images), `denoise`
// once per frame in place of the four svgfMain dispatches (src/main.cpp:906-947),
// `resize` on swapchain recreation (src/main.cpp:1547-1603).  PostProcessor owns
// the bloom image as the engine does (src/main.cpp:1298-1321), fog_filter is
// one froxel-filter dispatch (src/main.cpp:993-1005), EyeReadback the designed
// vision readback ring (docs/AI_INTERFACE.md:385-400).  Errors become tg::Error
// exceptions on the C++ side only; nothing throws across the C ABI.
#pragma once

#include <stdexcept>
#include <string>
#include <utility>

#include "tg_eye.h"
#include "tg_fog.h"
#include "tg_post.h"
#include "tg_svgf.h"

namespace tg {

class Error : public std::runtime_error {
public:
    Error(int status, const std::string& what) : std::runtime_error(what), status_(status) {}
    int status() const noexcept { return status_; }

private:
    int status_;
};

inline void check(int status)
{
    if (status != TG_OK)
        throw Error(status, std::string(tg_status_string(status)) + ": " + tg_last_error());
}

class SvgfDenoiser {
public:
    SvgfDenoiser(uint32_t width, uint32_t height, int32_t mode = TG_SVGF_MODE_FULL,
                 int32_t storage = TG_SVGF_STORAGE_FP32, int32_t device = -1)
    {
        tg_svgf_desc d{};
        d.width = width;
        d.height = height;
        d.device = device;
        check(tg_svgf_params_default(mode, storage, &d.params));
        check(tg_svgf_create(&d, &h_));
    }

    SvgfDenoiser(uint32_t width, uint32_t height, const tg_svgf_params& params, int32_t device = -1)
    {
        tg_svgf_desc d{};
        d.width = width;
        d.height = height;
        d.device = device;
        d.params = params;
        check(tg_svgf_create(&d, &h_));
    }

    SvgfDenoiser(const SvgfDenoiser&) = delete;
    SvgfDenoiser& operator=(const SvgfDenoiser&) = delete;
    SvgfDenoiser(SvgfDenoiser&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    SvgfDenoiser& operator=(SvgfDenoiser&& o) noexcept
    {
        if (this != &o) {
            tg_svgf_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    ~SvgfDenoiser() { tg_svgf_destroy(h_); }

    // One frame on `stream` (a cudaStream_t), device buffers.
    void denoise(const tg_svgf_inputs& in, const tg_svgf_outputs& out, void* stream = nullptr)
    {
        check(tg_svgf_denoise(h_, &in, &out, stream));
    }

    // One frame with host buffers; call synchronize() before reading the output.
    void denoise_host(const tg_svgf_inputs& in, const tg_svgf_outputs& out, void* stream = nullptr)
    {
        check(tg_svgf_denoise_host(h_, &in, &out, stream));
    }

    void synchronize() { check(tg_svgf_synchronize(h_)); }
    void reset(void* stream = nullptr) { check(tg_svgf_reset(h_, stream)); }
    void resize(uint32_t width, uint32_t height) { check(tg_svgf_resize(h_, width, height)); }

    tg_svgf_info info() const
    {
        tg_svgf_info i{};
        check(tg_svgf_get_info(h_, &i));
        return i;
    }

    tg_svgf* handle() const noexcept { return h_; }

private:
    tg_svgf* h_ = nullptr;
};

// One froxel-filter pass (the reference's filterMain dispatch); the params block is the engine's push block.
inline void fog_filter(const tg_fog_filter_params& params, const tg_volume& inject_raw, const tg_volume& history,
                       const tg_volume& output, void* stream = nullptr)
{
    check(tg_fog_filter(&params, &inject_raw, &history, &output, stream));
}

// The bloom + post-process chain; owns the bloom mips.
class PostProcessor {
public:
    PostProcessor(uint32_t width, uint32_t height, int device = -1)
    {
        tg_post_params p{};
        check(tg_post_params_default(&p));
        check(tg_post_create(width, height, &p, device, &h_));
    }
    PostProcessor(uint32_t width, uint32_t height, const tg_post_params& params, int device = -1)
    {
        check(tg_post_create(width, height, &params, device, &h_));
    }
    PostProcessor(const PostProcessor&) = delete;
    PostProcessor& operator=(const PostProcessor&) = delete;
    PostProcessor(PostProcessor&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    PostProcessor& operator=(PostProcessor&& o) noexcept
    {
        if (this != &o) {
            tg_post_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    ~PostProcessor() { tg_post_destroy(h_); }

    // The whole chain of one frame on `stream`: HDR image in, display image out (device buffers).
    void process(const tg_image& hdr, const tg_image& out, void* stream = nullptr)
    {
        check(tg_post_process(h_, &hdr, &out, stream));
    }
    void resize(uint32_t width, uint32_t height) { check(tg_post_resize(h_, width, height)); }
    tg_post_info info() const
    {
        tg_post_info i{};
        check(tg_post_get_info(h_, &i));
        return i;
    }
    tg_post* handle() const noexcept { return h_; }

private:
    tg_post* h_ = nullptr;
};

// The eye-frame readback ring: submit a tick's eye images, acquire a finished tick's TgVisionData views.
class EyeReadback {
public:
    explicit EyeReadback(const tg_eye_desc& desc) { check(tg_eye_create(&desc, &h_)); }
    EyeReadback(const EyeReadback&) = delete;
    EyeReadback& operator=(const EyeReadback&) = delete;
    EyeReadback(EyeReadback&& o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
    EyeReadback& operator=(EyeReadback&& o) noexcept
    {
        if (this != &o) {
            tg_eye_destroy(h_);
            h_ = std::exchange(o.h_, nullptr);
        }
        return *this;
    }
    ~EyeReadback() { tg_eye_destroy(h_); }

    // colour[i] / depth[i] of every eye, in the order of the descriptor's sizes.
    void submit(uint64_t frame, const tg_image* colour, const tg_image* depth, void* stream = nullptr)
    {
        check(tg_eye_submit(h_, frame, colour, depth, stream));
    }
    // Fills out[0 .. n_eyes - 1]; the views stay valid until frame + ring is submitted.
    void acquire(uint64_t frame, tg_vision_data* out) { check(tg_eye_acquire(h_, frame, out)); }
    tg_eye* handle() const noexcept { return h_; }

private:
    tg_eye* h_ = nullptr;
};

} // namespace tg
