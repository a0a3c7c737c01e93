"""Bloom + post-process chain over torch device tensors (include/tg_post.h).

`PostProcessor` owns the half-resolution rgba16f bloom mip chain, as the
reference owns its bloom image (`src/main.cpp:1298-1321`); `process` is one
frame of the reference's bloom and post-process dispatches
(`src/main.cpp:306-430`): HDR (h, w, 4) float16 / float32 in, display image
(h, w, 4) uint8 (BGRA by default, the reference's B8G8R8A8_UNORM swapchain;
or RGBA) or float32 out.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L


def default_params(**overrides) -> L.PostParams:
    p = L.PostParams()
    L.check(L.load().tg_post_params_default(C.byref(p)))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p


def _image(t, fmt) -> L.Image:
    if not t.is_cuda or t.dim() != 3 or t.shape[-1] != 4 or t.stride(-1) != 1 or t.stride(-2) != 4:
        raise ValueError("images are CUDA tensors (h, w, 4) with contiguous texels")
    return L.Image(t.data_ptr(), t.stride(0) * t.element_size(), fmt, 0)


class PostProcessor:
    def __init__(self, width: int, height: int, device: int | None = None, **params):
        self.lib = L.load()
        self.params = default_params(**params)
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        h = C.c_void_p()
        L.check(self.lib.tg_post_create(width, height, C.byref(self.params), device, C.byref(h)))
        self.handle = h
        self.width, self.height = width, height

    def process(self, hdr, out=None, order: str = "bgra", stream=None):
        """One frame; `out` uint8 (`order` "bgra" or "rgba") or float32, allocated BGRA8 when None."""
        if out is None:
            out = torch.empty((self.height, self.width, 4), dtype=torch.uint8, device=hdr.device)
        if hdr.dtype == torch.float16:
            hf = L.FMT_RGBA16F
        elif hdr.dtype == torch.float32:
            hf = L.FMT_RGBA32F
        else:
            raise TypeError("hdr is float16 or float32")
        if out.dtype == torch.uint8:
            of = L.FMT_BGRA8 if order == "bgra" else L.FMT_RGBA8
        elif out.dtype == torch.float32:
            of = L.FMT_RGBA32F
        else:
            raise TypeError("out is uint8 or float32")
        s = stream if stream is not None else torch.cuda.current_stream(hdr.device)
        hi, oi = _image(hdr, hf), _image(out, of)
        L.check(self.lib.tg_post_process(self.handle, C.byref(hi), C.byref(oi), C.c_void_p(s.cuda_stream)))
        return out

    def resize(self, width: int, height: int):
        L.check(self.lib.tg_post_resize(self.handle, width, height))
        self.width, self.height = width, height

    def info(self) -> dict:
        i = L.PostInfo()
        L.check(self.lib.tg_post_get_info(self.handle, C.byref(i)))
        n = i.mip_count
        return {"width": i.width, "height": i.height, "mip_count": n, "bloom_bytes": i.bloom_bytes,
                "mips": [(i.mip_width[k], i.mip_height[k], i.mip_ptr[k]) for k in range(n)]}

    def bloom_mips(self):
        """Copies of the bloom mips (float32 (h, w, 4) CPU arrays) after the frames enqueued so far."""
        torch.cuda.synchronize(self.device)
        res = []
        for (w, h, ptr) in self.info()["mips"]:
            view = torch.as_tensor(_DeviceArray(ptr, (h, w, 4), "<f2"), device=torch.device("cuda", self.device))
            res.append(view.float().cpu().numpy())
        return res

    def close(self):
        if self.handle:
            self.lib.tg_post_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _DeviceArray:
    """A view of handle-owned device memory for torch.as_tensor (CUDA array interface); callers only read it."""

    def __init__(self, ptr, shape, typestr):
        self.__cuda_array_interface__ = {"shape": shape, "typestr": typestr, "data": (int(ptr), False), "version": 2,
                                         "strides": None}
