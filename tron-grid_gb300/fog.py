"""Volumetric-fog froxel filter over torch device tensors (include/tg_fog.h).

`fog_filter` is one pass of the reference's filter dispatch
(`src/main.cpp:993-1005`, `src/volumetric_filter.slang:142-226`);
`FogFilter` owns the (history, output) pair and alternates it every frame as
the reference host alternates its two filter descriptor sets
(`src/main.cpp:2233-2253`).  Volumes are (depth, height, width, 4) float16
(the reference's rgba16f) or float32 CUDA tensors.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L


def make_params(inv_view_projection, prev_view_projection, camera_pos, alpha, width, height, depth, history_valid,
                near_plane, far_plane) -> L.FogParams:
    """The parameter block; matrices are 4x4 in mathematical order (clip = M @ [x, y, z, 1]) and are stored
    column-major (element (col, row) at col * 4 + row), as the reference's MathLib::Mat4."""
    p = L.FogParams()
    p.inv_view_projection[:] = [float(v) for v in np.asarray(inv_view_projection, np.float64).reshape(4, 4).T.reshape(16)]
    p.prev_view_projection[:] = [float(v) for v in np.asarray(prev_view_projection, np.float64).reshape(4, 4).T.reshape(16)]
    p.camera_pos[:] = [float(v) for v in np.asarray(camera_pos, np.float64).reshape(3)]
    p.alpha = float(alpha)
    p.froxel_width, p.froxel_height, p.froxel_depth = int(width), int(height), int(depth)
    p.history_valid = int(history_valid)
    p.near_plane, p.far_plane = float(near_plane), float(far_plane)
    return p


def param_bytes(p: L.FogParams) -> bytes:
    return C.string_at(C.addressof(p), C.sizeof(p))


def _fmt(t):
    import torch

    if t.dtype == torch.float16:
        return L.FMT_RGBA16F, 8
    if t.dtype == torch.float32:
        return L.FMT_RGBA32F, 16
    raise TypeError(f"froxel volumes are float16 or float32, not {t.dtype}")


def volume(t) -> L.Volume:
    """A (d, h, w, 4) CUDA tensor whose texels are contiguous along w (rows and slices may be strided)."""
    if not t.is_cuda or t.dim() != 4 or t.shape[-1] != 4 or t.stride(-1) != 1 or t.stride(-2) != 4:
        raise ValueError("froxel volume must be a CUDA tensor (d, h, w, 4) with contiguous texels along w")
    fmt, tb = _fmt(t)
    es = t.element_size()
    return L.Volume(t.data_ptr(), t.stride(1) * es, t.stride(0) * es, fmt, 0)


def fog_filter(params: L.FogParams, inject_raw, history, out=None, stream=None):
    """One filter pass; returns `out` (allocated like `history` when None)."""
    import torch

    if out is None:
        out = torch.empty_like(history)
    for t in (inject_raw, history, out):
        if tuple(t.shape[:3]) != (params.froxel_depth, params.froxel_height, params.froxel_width):
            raise ValueError(f"volume shape {tuple(t.shape)} does not match the froxel grid")
    s = stream if stream is not None else torch.cuda.current_stream(out.device)
    lib = L.load()
    vr, vh, vo = volume(inject_raw), volume(history), volume(out)
    L.check(lib.tg_fog_filter(C.byref(params), C.byref(vr), C.byref(vh), C.byref(vo), C.c_void_p(s.cuda_stream)))
    return out


class FogFilter:
    """Owns the two froxel volumes that alternate as (history, output), as the reference host does."""

    def __init__(self, width: int, height: int, depth: int, dtype=None, device="cuda"):
        import torch

        dtype = dtype or torch.float16
        self.vol = [torch.zeros((depth, height, width, 4), dtype=dtype, device=device) for _ in range(2)]
        self.frame = 0

    def step(self, params: L.FogParams, inject_raw, stream=None):
        """Filters one frame; returns this frame's output (the next frame's history)."""
        cur = self.frame & 1
        out = fog_filter(params, inject_raw, self.vol[cur ^ 1], self.vol[cur], stream=stream)
        self.frame += 1
        return out
