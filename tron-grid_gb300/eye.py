"""Eye-frame readback for AI entities (include/tg_eye.h) over torch device tensors.

`EyeReadback` packs every entity's eye image (colour + depth, at the resolution
its brain asked for) into a ring of mapped host slots each frame, as the
reference designs its vision path (`docs/AI_INTERFACE.md:338-400`: RGB888 and
float32 depth in CPU-visible memory, triple-buffered, read two frames behind).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib as L


def _image(t, fmt):
    return L.Image(t.data_ptr(), t.stride(0) * t.element_size(), fmt, 0)


def colour_format(t, order="bgra"):
    if t.dtype == torch.uint8:
        return L.FMT_BGRA8 if order == "bgra" else L.FMT_RGBA8
    if t.dtype == torch.float16:
        return L.FMT_RGBA16F
    if t.dtype == torch.float32:
        return L.FMT_RGBA32F
    raise TypeError(f"eye colour images are uint8, float16 or float32, not {t.dtype}")


class EyeReadback:
    def __init__(self, sizes, fovs=None, ring: int = 3, device: int | None = None, host_buffer=None):
        """sizes: [(width, height)] per eye; host_buffer: optional 16-byte-aligned writable numpy array that the
        ring lives in (e.g. a shared-memory mapping), page-locked for the copies."""
        self.lib = L.load()
        self.n = len(sizes)
        self.sizes = [(int(w), int(h)) for w, h in sizes]
        self._w = (C.c_uint32 * self.n)(*[w for w, _ in self.sizes])
        self._h = (C.c_uint32 * self.n)(*[h for _, h in self.sizes])
        self._fov = (C.c_double * self.n)(*(fovs if fovs is not None else [0.0] * self.n))
        if device is None:
            device = torch.cuda.current_device()
        self.device = device
        self.ring = ring
        self._buf = host_buffer
        hb = host_buffer.ctypes.data if host_buffer is not None else None
        nb = host_buffer.nbytes if host_buffer is not None else 0
        d = L.EyeDesc(self.n, self._w, self._h, self._fov, ring, device, hb, nb)
        h = C.c_void_p()
        L.check(self.lib.tg_eye_create(C.byref(d), C.byref(h)))
        self.handle = h

    def host_bytes(self) -> int:
        return int(self.lib.tg_eye_host_bytes(self.n, self._w, self._h, self.ring))

    def submit(self, frame: int, colours, depths, order="bgra", stream=None):
        """colours: per eye (h, w, 4) uint8 / float16 / float32 CUDA tensors; depths: per eye (h, w) float32."""
        if len(colours) != self.n or len(depths) != self.n:
            raise ValueError(f"{self.n} eyes, {len(colours)} colour and {len(depths)} depth images given")
        ci = (L.Image * self.n)(*[_image(c, colour_format(c, order)) for c in colours])
        di = (L.Image * self.n)(*[_image(d, L.FMT_R32F) for d in depths])
        s = stream if stream is not None else torch.cuda.current_stream(self.device)
        L.check(self.lib.tg_eye_submit(self.handle, frame, ci, di, C.c_void_p(s.cuda_stream)))

    def acquire(self, frame: int):
        """[(rgb (h, w, 3) uint8, depth (h, w) float32, fov)] views into the host slot of `frame`."""
        out = (L.VisionData * self.n)()
        L.check(self.lib.tg_eye_acquire(self.handle, frame, out))
        res = []
        for v in out:
            rgb = np.ctypeslib.as_array(v.rgb, shape=(v.height, v.width, 3))
            dep = np.ctypeslib.as_array(v.depth, shape=(v.height, v.width))
            res.append((rgb, dep, v.fov_horizontal))
        return res

    def close(self):
        if self.handle:
            self.lib.tg_eye_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
