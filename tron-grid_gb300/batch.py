"""Python mirror of the batched SVGF (many streams, one persistent launch per step)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .svgf import _stream_ptr, image


class Batch:
    """N camera streams of their own resolutions, FULL mode, denoised step by step."""

    def __init__(self, sizes, storage: int = L.STORAGE_FP16, device: int | None = None, rows_per_thread: int = 0,
                 ctas_per_sm: int = 0, use_graph: bool = True, strategy: int = 0, barrier_timeout_us: int = 0,
                 debug_barrier_extra: int = 0, **params):
        self.lib = L.load()
        self.sizes = [(int(w), int(h)) for (w, h) in sizes]
        n = len(self.sizes)
        ws = (C.c_uint32 * n)(*[w for w, _ in self.sizes])
        hs = (C.c_uint32 * n)(*[h for _, h in self.sizes])
        if device is None:
            device = torch.cuda.current_device()
        self.params = L.default_params(L.MODE_FULL, storage, **params)
        d = L.BatchDesc(n, ws, hs, self.params, device, rows_per_thread, ctas_per_sm, int(use_graph), strategy,
                        barrier_timeout_us, debug_barrier_extra)
        h = C.c_void_p()
        L.check(self.lib.tg_svgf_batch_create(C.byref(d), C.byref(h)))
        self.handle = h
        self._keep = (ws, hs)

    @staticmethod
    def _arrays(ids, frames, outs):
        n = len(ids)
        ida = (C.c_uint32 * n)(*ids)
        ins = (L.Inputs * n)()
        ous = (L.Outputs * n)()
        for k, (fr, o) in enumerate(zip(frames, outs)):
            ins[k] = L.Inputs(image("radiance", fr["radiance"]), image("depth", fr["depth"]),
                              image("normal", fr["normal"]), image("motion", fr["motion"]))
            ous[k] = L.Outputs(image("denoised", o))
        return n, ida, ins, ous

    def denoise(self, ids, frames, outs, stream=None):
        """One step: stream ids[k] consumes frames[k] (dict of device tensors) and writes outs[k]."""
        n, ida, ins, ous = self._arrays(ids, frames, outs)
        L.check(self.lib.tg_svgf_batch_denoise(self.handle, n, ida, ins, ous, _stream_ptr(stream)))
        return outs

    def autotune(self, ids, frames, outs, steps: int = 3, stream=None):
        n, ida, ins, ous = self._arrays(ids, frames, outs)
        L.check(self.lib.tg_svgf_batch_autotune(self.handle, n, ida, ins, ous, steps, _stream_ptr(stream)))
        return self.info()

    def reset_stream(self, sid: int, stream=None):
        L.check(self.lib.tg_svgf_batch_reset_stream(self.handle, sid, _stream_ptr(stream)))

    def synchronize(self):
        L.check(self.lib.tg_svgf_batch_synchronize(self.handle))

    def info(self) -> dict:
        i = L.BatchInfo()
        L.check(self.lib.tg_svgf_batch_get_info(self.handle, C.byref(i)))
        return {k: getattr(i, k) for k, _ in L.BatchInfo._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.tg_svgf_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
