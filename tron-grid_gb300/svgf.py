"""Python mirror of the SVGF pass over the C ABI (include/tg_svgf.h).

`Denoiser` plays the role of the reference's SVGF block in recordFrame
(src/main.cpp:906-947) plus the images it owns (src/main.cpp:1326-1397): one
object per camera stream, one `denoise` call per frame, `reset` / `resize` for
the zero-clear and swapchain-resize paths (src/main.cpp:1399-1496, :1547-1603).
Device buffers are torch tensors (torch supplies memory and streams only; the
work runs in libtg_svgf.so).
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L


def _fmt(role: str, t: torch.Tensor) -> int:
    dt, nd = t.dtype, t.dim()
    ch = t.shape[2] if nd == 3 else 1
    if role in ("radiance", "denoised"):
        if ch == 4 and dt == torch.float32:
            return L.FMT_RGBA32F
        if ch == 4 and dt == torch.float16:
            return L.FMT_RGBA16F
    elif role == "depth":
        if ch == 1 and dt == torch.float32:
            return L.FMT_R32F
    elif role == "normal":
        if ch == 3 and dt == torch.float32:
            return L.FMT_RGB32F
        if ch == 4 and dt == torch.float32:
            return L.FMT_RGBA32F
        if ch == 2 and dt == torch.int16:
            return L.FMT_OCT16
    elif role == "motion":
        if ch == 2 and dt == torch.float32:
            return L.FMT_RG32F
        if ch == 2 and dt == torch.float16:
            return L.FMT_RG16F
    raise ValueError(f"{role}: unsupported tensor layout {tuple(t.shape)} {dt}")


def image(role: str, t: torch.Tensor | None) -> L.Image:
    """tg_image view of an (H, W[, C]) tensor whose pixels are contiguous within a row."""
    if t is None:
        return L.Image(None, 0, L.FMT_NONE, 0)
    fmt = _fmt(role, t)
    if t.dim() == 3 and (t.stride(2) != 1 or t.stride(1) != t.shape[2]):
        raise ValueError(f"{role}: pixels must be contiguous within a row")
    if t.dim() == 2 and t.stride(1) != 1:
        raise ValueError(f"{role}: pixels must be contiguous within a row")
    return L.Image(t.data_ptr(), t.stride(0) * t.element_size(), fmt, 0)


def _stream_ptr(stream) -> int | None:
    if stream is None:
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, torch.cuda.Stream):
        return stream.cuda_stream
    return int(stream)


class Denoiser:
    """One SVGF stream (a handle of the C ABI)."""

    def __init__(self, width: int, height: int, mode: int = L.MODE_FULL, storage: int = L.STORAGE_FP32,
                 device: int | None = None, flags: int = 0, **params):
        self.lib = L.load()
        self.params = L.default_params(mode, storage, **params)
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        d = L.Desc(width, height, self.params, device, flags)
        h = C.c_void_p()
        L.check(self.lib.tg_svgf_create(C.byref(d), C.byref(h)))
        self.handle = h
        self.width, self.height = width, height

    # ---------------------------------------------------------------- frames
    def denoise(self, radiance, depth=None, normal=None, motion=None, out=None, stream=None):
        """Denoises one frame of device tensors; returns `out` (allocated RGBA32F if None)."""
        if out is None:
            out = torch.empty((self.height, self.width, 4), dtype=torch.float32, device=radiance.device)
        ins = L.Inputs(image("radiance", radiance), image("depth", depth), image("normal", normal),
                       image("motion", motion))
        outs = L.Outputs(image("denoised", out))
        L.check(self.lib.tg_svgf_denoise(self.handle, C.byref(ins), C.byref(outs), _stream_ptr(stream)))
        return out

    def denoise_host(self, radiance, depth=None, normal=None, motion=None, out=None, stream=None):
        """Host-memory variant (CPU tensors, ideally pinned); call synchronize() before reading `out`."""
        if out is None:
            out = torch.empty((self.height, self.width, 4), dtype=torch.float32, pin_memory=True)
        ins = L.Inputs(image("radiance", radiance), image("depth", depth), image("normal", normal),
                       image("motion", motion))
        outs = L.Outputs(image("denoised", out))
        L.check(self.lib.tg_svgf_denoise_host(self.handle, C.byref(ins), C.byref(outs), _stream_ptr(stream)))
        return out

    def synchronize(self):
        L.check(self.lib.tg_svgf_synchronize(self.handle))

    def reset(self, stream=None):
        L.check(self.lib.tg_svgf_reset(self.handle, _stream_ptr(stream)))

    def resize(self, width: int, height: int):
        L.check(self.lib.tg_svgf_resize(self.handle, width, height))
        self.width, self.height = width, height

    def info(self) -> dict:
        i = L.Info()
        L.check(self.lib.tg_svgf_get_info(self.handle, C.byref(i)))
        return {k: getattr(i, k) for k, _ in L.Info._fields_ if k != "reserved"}

    def profile(self, enable: bool = True):
        """Brackets every kernel launch with a CUDA event pair (see profile_read)."""
        L.check(self.lib.tg_svgf_profile_enable(self.handle, int(enable)))

    def profile_read(self, reset: bool = True) -> dict:
        """{family: {launches, total_ms, algo_bytes}} accumulated since the last reset."""
        arr = (L.KernelStat * 8)()
        n = C.c_int(0)
        L.check(self.lib.tg_svgf_profile_read(self.handle, arr, 8, C.byref(n), int(reset)))
        return {arr[i].name.decode(): dict(launches=arr[i].launches, total_ms=arr[i].total_ms,
                                           algo_bytes=arr[i].algo_bytes) for i in range(min(n.value, 8))}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.tg_svgf_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def state_bytes(width: int, height: int, mode: int = L.MODE_FULL, storage: int = L.STORAGE_FP32, **params) -> int:
    p = L.default_params(mode, storage, **params)
    return int(L.load().tg_svgf_state_bytes(C.byref(p), width, height))
