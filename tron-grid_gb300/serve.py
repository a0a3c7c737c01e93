"""Python mirror of the serving loop (continuous batching under an HBM budget)."""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib as L
from .svgf import image


class Server:
    """Sessions submit frames (host tensors, ideally pinned); results land in the given host outputs."""

    def __init__(self, budget_bytes: int, max_sessions: int = 1024, max_batch: int = 64, batching: bool = True,
                 storage: int = L.STORAGE_FP16, device: int | None = None, use_graph: bool = True,
                 strategy: int = 0, max_batch_pixels: int = 0, **params):
        self.lib = L.load()
        if device is None:
            device = torch.cuda.current_device()
        self.params = L.default_params(L.MODE_FULL, storage, **params)
        d = L.ServerDesc(self.params, int(budget_bytes), max_sessions, max_batch, device, int(batching),
                         int(use_graph), strategy, int(max_batch_pixels))
        h = C.c_void_p()
        L.check(self.lib.tg_svgf_server_create(C.byref(d), C.byref(h)))
        self.handle = h
        self._alive = {}

    def submit(self, session: int, frame: dict, out: torch.Tensor) -> int:
        h, w = out.shape[:2]
        ins = L.Inputs(image("radiance", frame["radiance"]), image("depth", frame["depth"]),
                       image("normal", frame["normal"]), image("motion", frame["motion"]))
        outs = L.Outputs(image("denoised", out))
        t = C.c_uint64(0)
        L.check(self.lib.tg_svgf_server_submit(self.handle, session, w, h, C.byref(ins), C.byref(outs), C.byref(t)))
        self._alive[t.value] = (frame, out)
        return t.value

    def wait(self, ticket: int, timeout_us: int = 120_000_000) -> dict:
        info = L.RequestInfo()
        L.check(self.lib.tg_svgf_server_wait(self.handle, ticket, timeout_us, C.byref(info)))
        self._alive.pop(ticket, None)
        return {k: getattr(info, k) for k, _ in L.RequestInfo._fields_}

    def end_session(self, session: int):
        L.check(self.lib.tg_svgf_server_end_session(self.handle, session))

    def stats(self, reset: bool = False) -> dict:
        s = L.ServerStats()
        L.check(self.lib.tg_svgf_server_get_stats(self.handle, C.byref(s), int(reset)))
        return {k: getattr(s, k) for k, _ in L.ServerStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.tg_svgf_server_destroy(self.handle)
            self.handle = None
            self._alive.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
