// tg_svgf.hpp - C++ RAII wrapper over the C ABI of include/tg_svgf.h.
//
// Mirrors how the reference engine uses its SVGF pass: one object per swapchain
// (src/main.cpp:1326-1397 creates the pass's images), `denoise` once per frame
// in place of the four svgfMain dispatches (src/main.cpp:906-947), `resize` on
// swapchain recreation (src/main.cpp:1547-1603).  Errors become tg::Error
// exceptions on the C++ side only; nothing throws across the C ABI.
#pragma once

#include <stdexcept>
#include <string>
#include <utility>

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

} // namespace tg
