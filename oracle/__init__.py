"""ctypes front end of the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module; the product never imports it.  Arrays are numpy, row-major (h, w, c).

* ``ref_frame``  - restatement of the reference shader chain
  (`src/svgf_denoise.slang:152-275`, host order `src/main.cpp:929-944`).
* ``ref_frame_reference`` - the reference shader source itself compiled as C++
  (oracle/build.py), when the translation could be built.
* ``full_frame`` - the full Schied-2017 SVGF superset, float32 or float64.
* ``fog_filter`` - restatement of the volumetric-fog froxel filter
  (`src/volumetric_filter.slang:142-226`), float32 or float64;
  ``fog_filter_reference`` - that shader compiled as C++ (oracle/build.py).
  Froxel volumes are numpy (d, h, w, 4).
* ``post_frame`` - restatement of the bloom + post-process chain
  (`src/bloom_downsample.slang`, `src/postprocess.slang`, host order
  `src/main.cpp:306-430`); ``post_frame_reference`` - those shaders compiled
  as C++.
* ``eye_pack`` - the eye-frame packing (RGB888 + float32 depth; numpy).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_orc = None
_ref = None
_fogref = None
_postref = None


class FullParams(C.Structure):
    _fields_ = [
        ("alpha", C.c_double),
        ("moments_alpha", C.c_double),
        ("sigma_l", C.c_double),
        ("sigma_n", C.c_double),
        ("sigma_z", C.c_double),
        ("levels", C.c_int32),
        ("max_history", C.c_int32),
        ("fallback_frames", C.c_int32),
        ("reserved", C.c_int32),
    ]


def full_params(alpha=0.2, moments_alpha=0.2, sigma_l=4.0, sigma_n=128.0, sigma_z=1.0, levels=5, max_history=32,
                fallback_frames=4) -> FullParams:
    return FullParams(alpha, moments_alpha, sigma_l, sigma_n, sigma_z, levels, max_history, fallback_frames, 0)


_orc_timing = None


def _lib(timing: bool = False):
    """The checker build, or with ``timing`` the timed CPU baseline's build (oracle/build.py TIMING_CXXFLAGS)."""
    global _orc, _orc_timing
    if timing:
        if _orc_timing is None:
            path = _build.ORC_TIMING_LIB
            if not os.path.exists(path):
                path = _build.build_oracle_timing()
            _orc_timing = _declare(C.CDLL(path))
        return _orc_timing
    if _orc is None:
        path = _build.ORC_LIB
        if not os.path.exists(path):
            path = _build.build_oracle()
        _orc = _declare(C.CDLL(path))
    return _orc


def timing_flags() -> str:
    return " ".join(_build.TIMING_CXXFLAGS)


def _declare(lib):
    """Argument types of the oracle's C entry points (the same in both builds)."""
    P = C.c_void_p
    lib.orc_ref_frame_f32.argtypes = [C.c_int, C.c_int, P, P, P, P, C.c_int, C.c_float, C.c_float, C.c_float,
                                      C.c_int, C.c_int]
    lib.orc_ref_frame_f64.argtypes = [C.c_int, C.c_int, P, P, P, P, C.c_int, C.c_double, C.c_double,
                                      C.c_double, C.c_int, C.c_int]
    for nm in ("orc_full_frame_f32", "orc_full_frame_f64"):
        getattr(lib, nm).argtypes = [C.POINTER(FullParams), C.c_int, C.c_int] + [P] * 12 + [C.c_int, C.c_int]
    lib.orc_oct16_encode.argtypes = [C.c_int, P, P]
    lib.orc_oct16_decode.argtypes = [C.c_int, P, P]
    lib.orc_num_threads.restype = C.c_int
    lib.orc_fog_filter.argtypes = [C.c_char_p, P, P, P, C.c_int, C.c_int, C.c_int]
    lib.orc_post_frame.argtypes = [C.c_int, C.c_int, P, C.c_float, C.c_float, C.c_int, P, P, C.c_int, C.c_int,
                                   C.c_int, C.c_int]
    lib.orc_post_frame.restype = C.c_int
    return lib


def reference_available() -> bool:
    return _reflib() is not None


def _reflib():
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_reference()
            except Exception:
                path = None
        if path is None or not os.path.exists(path):
            return None
        _ref = C.CDLL(path)
        P = C.c_void_p
        _ref.ref_svgf_frame.argtypes = [C.c_int, C.c_int, P, P, P, P, C.c_int, C.c_int]
    return _ref


def num_threads() -> int:
    return int(_lib().orc_num_threads())


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _p(a):
    return a.ctypes.data_as(C.c_void_p)


def ref_frame(raw, mom_prev, levels=3, phi=2.0, alpha_m=0.2, var_eps=1e-4, fp16_store=True, dtype=np.float32,
              threads=0, timing=False):
    """One reference frame.  raw (h,w,4), mom_prev (h,w,2) -> (out (h,w,4), mom_curr (h,w,2))."""
    raw = _c(raw, dtype)
    mom_prev = _c(mom_prev, dtype)
    h, w = raw.shape[:2]
    out = np.zeros((h, w, 4), dtype)
    mom = np.zeros((h, w, 2), dtype)
    lib = _lib(timing)
    f = lib.orc_ref_frame_f32 if dtype == np.float32 else lib.orc_ref_frame_f64
    rc = f(w, h, _p(raw), _p(mom_prev), _p(mom), _p(out), levels, phi, alpha_m, var_eps, int(bool(fp16_store)),
           threads)
    if rc:
        raise ValueError("oracle ref_frame rejected its arguments")
    return out, mom


def ref_frame_reference(raw, mom_prev, fp16_store=True, threads=0):
    """The reference shader itself (compiled as C++): init + 3 levels."""
    lib = _reflib()
    if lib is None:
        raise RuntimeError("reference shader translation not built (oracle/_ref)")
    raw = _c(raw, np.float32).copy()
    mom_prev = _c(mom_prev, np.float32).copy()
    h, w = raw.shape[:2]
    out = np.zeros((h, w, 4), np.float32)
    mom = np.zeros((h, w, 2), np.float32)
    rc = lib.ref_svgf_frame(w, h, _p(raw), _p(mom_prev), _p(mom), _p(out), int(bool(fp16_store)), threads)
    if rc:
        raise ValueError("reference frame rejected its arguments")
    return out, mom


class FullState:
    """Per-stream state of the FULL oracle (zero = no history)."""

    def __init__(self, h, w, dtype=np.float64):
        self.guide = np.zeros((h, w, 4), dtype)
        self.hist = np.zeros((h, w, 4), dtype)
        self.mom = np.zeros((h, w, 2), dtype)


# Stores of the FULL algorithm that FP16 storage rounds (the Q_* mask of oracle/svgf_oracle.cpp): each can be
# emulated on its own to measure its share of the error against float64.
Q_INPUT, Q_NORMAL, Q_TC, Q_HIST, Q_MOM, Q_RECORD, Q_OUTPUT = 1, 2, 4, 8, 16, 32, 64
Q_ALL = 127


def fp16_storage_mask(fp16_output: bool) -> int:
    """The stores the CUDA path's FP16 storage form rounds: radiance, octahedral normals, the temporally integrated
    colour, history and moments in binary16; the a-trous scratch records stay float32; the output is rounded only
    when the caller's output image is RGBA16F."""
    return (Q_ALL & ~(Q_RECORD | Q_OUTPUT)) | (Q_OUTPUT if fp16_output else 0)


def full_frame(params: FullParams, state: FullState, radiance, depth, normal, motion, fp16_store=False, threads=0,
               timing=False):
    """One FULL frame; updates ``state`` in place and returns (out (h,w,4), var (h,w)).

    ``fp16_store``: False / 0 = no emulation, True = every store of the FP16 storage form (Q_ALL), or a mask of
    Q_* bits naming the stores to round.  ``timing``: run the timed CPU baseline's build instead of the checker's."""
    mask = (Q_ALL if fp16_store else 0) if isinstance(fp16_store, (bool, np.bool_)) else int(fp16_store)
    dt = state.guide.dtype
    radiance = _c(radiance, dt)
    depth = _c(depth, dt)
    normal = _c(normal, dt)
    motion = _c(motion, dt)
    h, w = depth.shape[:2]
    g = np.zeros_like(state.guide)
    hs = np.zeros_like(state.hist)
    m = np.zeros_like(state.mom)
    out = np.zeros((h, w, 4), dt)
    var = np.zeros((h, w), dt)
    lib = _lib(timing)
    f = lib.orc_full_frame_f32 if dt == np.float32 else lib.orc_full_frame_f64
    rc = f(C.byref(params), w, h, _p(radiance), _p(depth), _p(normal), _p(motion), _p(state.guide), _p(state.hist),
           _p(state.mom), _p(g), _p(hs), _p(m), _p(out), _p(var), mask, threads)
    if rc:
        raise ValueError("oracle full_frame rejected its arguments")
    state.guide, state.hist, state.mom = g, hs, m
    return out, var


def oct16_encode(normals):
    n = _c(normals, np.float32).reshape(-1, 3)
    out = np.zeros((n.shape[0], 2), np.int16)
    _lib().orc_oct16_encode(n.shape[0], _p(n), _p(out))
    return out.reshape(tuple(np.shape(normals)[:-1]) + (2,))


def oct16_decode(enc):
    e = _c(enc, np.int16).reshape(-1, 2)
    out = np.zeros((e.shape[0], 3), np.float32)
    _lib().orc_oct16_decode(e.shape[0], _p(e), _p(out))
    return out.reshape(tuple(np.shape(enc)[:-1]) + (3,))


# ------------------------------------------------------ volumetric-fog filter ----

FOG_PARAM_BYTES = 176


def fog_param_block(inv_view_projection, prev_view_projection, camera_pos, alpha, width, height, depth,
                    history_valid, near_plane, far_plane) -> bytes:
    """The 176-byte parameter block of the froxel filter (the reference's
    VolumetricFilterPushConstants layout, `src/main.cpp:221-234`).

    The matrices are given as 4x4 arrays in mathematical order (clip = M @ [x, y, z, 1]) and stored
    column-major, element (col, row) at index col * 4 + row, as the reference's MathLib::Mat4.
    """
    import struct

    def cm(m):
        m = np.asarray(m, dtype=np.float64).reshape(4, 4)
        return [float(v) for v in m.T.reshape(16)]

    cam = [float(v) for v in np.asarray(camera_pos, dtype=np.float64).reshape(3)]
    blk = struct.pack("<16f16f3ff4I4f", *cm(inv_view_projection), *cm(prev_view_projection), *cam, float(alpha),
                      int(width), int(height), int(depth), int(history_valid), float(near_plane), float(far_plane),
                      0.0, 0.0)
    assert len(blk) == FOG_PARAM_BYTES
    return blk


def _fog_dims(block: bytes):
    import struct

    w, h, d, _ = struct.unpack_from("<4I", block, 36 * 4)
    return w, h, d


def fog_filter(block: bytes, raw, history, fp16_store=True, dtype=np.float32, threads=0):
    """One froxel-filter pass (restatement).  raw / history (d, h, w, 4) -> out (d, h, w, 4) float32."""
    w, h, d = _fog_dims(block)
    raw = _c(raw, np.float32).reshape(d, h, w, 4)
    history = _c(history, np.float32).reshape(d, h, w, 4)
    out = np.zeros((d, h, w, 4), np.float32)
    rc = _lib().orc_fog_filter(block, _p(raw), _p(history), _p(out), int(bool(fp16_store)),
                               int(dtype == np.float64), threads)
    if rc:
        raise ValueError("oracle fog_filter rejected its arguments")
    return out


def fog_reference_available() -> bool:
    return _fogreflib() is not None


def _fogreflib():
    global _fogref
    if _fogref is None:
        path = _build.FOG_REF_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_fog_reference()
            except Exception:
                path = None
        if path is None or not os.path.exists(path):
            return None
        _fogref = C.CDLL(path)
        P = C.c_void_p
        _fogref.ref_fog_filter.argtypes = [C.c_char_p, P, P, P, C.c_int, C.c_int]
    return _fogref


def fog_filter_reference(block: bytes, raw, history, fp16_store=True, threads=0):
    """The reference froxel-filter shader itself (compiled as C++)."""
    lib = _fogreflib()
    if lib is None:
        raise RuntimeError("reference froxel-filter translation not built (oracle/_ref)")
    w, h, d = _fog_dims(block)
    raw = _c(raw, np.float32).reshape(d, h, w, 4).copy()
    history = _c(history, np.float32).reshape(d, h, w, 4).copy()
    out = np.zeros((d, h, w, 4), np.float32)
    rc = lib.ref_fog_filter(block, _p(raw), _p(history), _p(out), int(bool(fp16_store)), threads)
    if rc:
        raise ValueError("reference fog filter rejected its arguments")
    return out


# ------------------------------------------------------ bloom + post-process ----

def bloom_mip_sizes(width, height, max_mips=6):
    """Mip sizes of the bloom image (half the frame, at least 1x1; `src/main.cpp:271-278, 1298-1301`)."""
    import math

    bw, bh = max(width // 2, 1), max(height // 2, 1)
    n = min(int(math.floor(math.log2(float(np.float32(max(bw, bh)))))) + 1, max_mips)
    return [(max(bw >> i, 1), max(bh >> i, 1)) for i in range(n)]


def _split_mips(flat, sizes):
    out, o = [], 0
    for (w, h) in sizes:
        out.append(flat[o:o + w * h * 4].reshape(h, w, 4))
        o += w * h * 4
    return out


def post_frame(hdr, threshold=1.0, strength=0.095, max_mips=6, fp16_store=True, unorm8=True, dtype=np.float32,
               threads=0):
    """One frame of the chain (restatement).  hdr (h, w, 4) -> (out (h, w, 4) float32, [bloom mips])."""
    hdr = _c(hdr, np.float32)
    h, w = hdr.shape[:2]
    sizes = bloom_mip_sizes(w, h, max_mips)
    out = np.zeros((h, w, 4), np.float32)
    mips = np.zeros(sum(a * b * 4 for a, b in sizes), np.float32)
    n = _lib().orc_post_frame(w, h, _p(hdr), threshold, strength, max_mips, _p(out), _p(mips), int(bool(fp16_store)),
                              int(bool(unorm8)), int(dtype == np.float64), threads)
    if n != len(sizes):
        raise ValueError("oracle post_frame rejected its arguments")
    return out, _split_mips(mips, sizes)


def post_reference_available() -> bool:
    return _postreflib() is not None


def _postreflib():
    global _postref
    if _postref is None:
        path = _build.POST_REF_LIB
        if not os.path.exists(path):
            try:
                path = _build.build_post_reference()
            except Exception:
                path = None
        if path is None or not os.path.exists(path):
            return None
        _postref = C.CDLL(path)
        P = C.c_void_p
        _postref.ref_post_frame.argtypes = [C.c_int, C.c_int, P, C.c_float, C.c_float, C.c_int, P, P, C.c_int]
        _postref.ref_post_frame.restype = C.c_int
    return _postref


def post_frame_reference(hdr, threshold=1.0, strength=0.095, max_mips=6, threads=0):
    """The reference bloom + post-process shaders themselves (compiled as C++): rgba16f bloom, UNORM8 output."""
    lib = _postreflib()
    if lib is None:
        raise RuntimeError("reference bloom / post-process translation not built (oracle/_ref)")
    hdr = _c(hdr, np.float32)
    h, w = hdr.shape[:2]
    sizes = bloom_mip_sizes(w, h, max_mips)
    out = np.zeros((h, w, 4), np.float32)
    mips = np.zeros(sum(a * b * 4 for a, b in sizes), np.float32)
    n = lib.ref_post_frame(w, h, _p(hdr), threshold, strength, max_mips, _p(out), _p(mips), threads)
    if n != len(sizes):
        raise ValueError("reference post frame rejected its arguments")
    return out, _split_mips(mips, sizes)


# ------------------------------------------------------------ eye readback ----

def eye_pack(colour, depth, order="bgra"):
    """The eye frame a brain reads (docs/AI_INTERFACE.md:368-381): RGB888 (h, w, 3) and depth (h, w) float32.
    colour is (h, w, 4) uint8 (BGRA or RGBA) or float (clamped to [0, 1], scaled by 255 in float32 and rounded
    to nearest, ties to even)."""
    colour = np.asarray(colour)
    if colour.dtype == np.uint8:
        rgb = colour[..., [2, 1, 0]] if order == "bgra" else colour[..., :3]
    else:
        c = np.clip(colour[..., :3].astype(np.float32), np.float32(0), np.float32(1))
        rgb = np.rint(c * np.float32(255)).astype(np.uint8)
    return np.ascontiguousarray(rgb), np.asarray(depth, np.float32).copy()
