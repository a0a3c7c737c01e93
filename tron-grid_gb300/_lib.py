"""ctypes declarations of include/tg_svgf.h, tg_fog.h, tg_post.h, tg_eye.h and the loader of libtg_svgf.so.

The library is the product: if it is missing the import of this package fails
with an error that says how to build it.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libtg_svgf.so")

# tg_status
OK, ERR_INVALID, ERR_OOM, ERR_CUDA, ERR_TIMEOUT, ERR_BUDGET, ERR_UNSUPPORTED, ERR_STATE = range(8)
# tg_format
FMT_NONE, FMT_RGBA32F, FMT_RGBA16F, FMT_R32F, FMT_RGB32F, FMT_OCT16, FMT_RG32F, FMT_RG16F, FMT_RGBA8, FMT_BGRA8 = range(10)
FMT_BYTES = {FMT_RGBA32F: 16, FMT_RGBA16F: 8, FMT_R32F: 4, FMT_RGB32F: 12, FMT_OCT16: 4, FMT_RG32F: 8, FMT_RG16F: 4,
             FMT_RGBA8: 4, FMT_BGRA8: 4}
# tg_svgf_mode / tg_svgf_storage
MODE_REF_EXACT, MODE_FULL = 0, 1
BATCH_STAGES, BATCH_PERSISTENT = 0, 1
FLAG_NO_TMA = 1
STORAGE_FP32, STORAGE_FP16 = 0, 1


class Image(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("pitch_bytes", C.c_int64), ("format", C.c_int32), ("reserved", C.c_int32)]


class Params(C.Structure):
    _fields_ = [
        ("mode", C.c_int32), ("storage", C.c_int32), ("levels", C.c_int32), ("max_history", C.c_int32),
        ("fallback_frames", C.c_int32), ("reserved0", C.c_int32),
        ("alpha", C.c_float), ("moments_alpha", C.c_float), ("sigma_l", C.c_float), ("sigma_n", C.c_float),
        ("sigma_z", C.c_float), ("variance_epsilon", C.c_float), ("reserved", C.c_float * 4),
    ]


class Desc(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("params", Params), ("device", C.c_int32),
                ("flags", C.c_int32)]


class Inputs(C.Structure):
    _fields_ = [("radiance", Image), ("depth", Image), ("normal", Image), ("motion", Image)]


class Outputs(C.Structure):
    _fields_ = [("denoised", Image)]


class Info(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("frame_index", C.c_uint64),
                ("state_bytes", C.c_uint64), ("scratch_bytes", C.c_uint64), ("staging_bytes", C.c_uint64),
                ("kernels_per_frame", C.c_uint32), ("device_errors", C.c_uint32), ("tma", C.c_uint32),
                ("reserved", C.c_uint32)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint32), ("reserved", C.c_uint32),
                ("total_ms", C.c_double), ("algo_bytes", C.c_double)]


class BatchDesc(C.Structure):
    _fields_ = [("n_streams", C.c_uint32), ("widths", C.POINTER(C.c_uint32)), ("heights", C.POINTER(C.c_uint32)),
                ("params", Params), ("device", C.c_int32), ("rows_per_thread", C.c_int32),
                ("ctas_per_sm", C.c_int32), ("use_graph", C.c_int32), ("strategy", C.c_int32),
                ("barrier_timeout_us", C.c_uint32), ("debug_barrier_extra", C.c_int32)]


class BatchInfo(C.Structure):
    _fields_ = [("n_streams", C.c_uint32), ("rows_per_thread", C.c_int32), ("ctas_per_sm", C.c_int32),
                ("grid_ctas", C.c_int32), ("graphs", C.c_int32), ("strategy", C.c_int32),
                ("state_bytes", C.c_uint64), ("scratch_bytes", C.c_uint64), ("steps", C.c_uint64),
                ("barrier_timeouts", C.c_uint64), ("tuned_ms", C.c_double)]


class ServerDesc(C.Structure):
    _fields_ = [("params", Params), ("hbm_budget_bytes", C.c_uint64), ("max_sessions", C.c_uint32),
                ("max_batch", C.c_uint32), ("device", C.c_int32), ("batching", C.c_int32),
                ("use_graph", C.c_int32), ("strategy", C.c_int32), ("max_batch_pixels", C.c_uint64)]


class RequestInfo(C.Structure):
    _fields_ = [("status", C.c_int32), ("batch_size", C.c_uint32), ("latency_ms", C.c_double),
                ("queue_ms", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("failed", C.c_uint64),
                ("admissions", C.c_uint64), ("evictions", C.c_uint64), ("launches", C.c_uint64),
                ("resident_bytes", C.c_uint64), ("peak_resident_bytes", C.c_uint64),
                ("resident_sessions", C.c_uint32), ("max_batch_seen", C.c_uint32),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("mpx_per_s", C.c_double), ("wall_s", C.c_double)]


class TgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{message} (status {status})")
        self.status = status


class FogParams(C.Structure):
    """tg_fog_filter_params: the reference's 176-byte VolumetricFilterPushConstants layout."""
    _fields_ = [("inv_view_projection", C.c_float * 16), ("prev_view_projection", C.c_float * 16),
                ("camera_pos", C.c_float * 3), ("alpha", C.c_float), ("froxel_width", C.c_uint32),
                ("froxel_height", C.c_uint32), ("froxel_depth", C.c_uint32), ("history_valid", C.c_uint32),
                ("near_plane", C.c_float), ("far_plane", C.c_float), ("pad0", C.c_float), ("pad1", C.c_float)]


class Volume(C.Structure):
    _fields_ = [("ptr", C.c_void_p), ("row_pitch_bytes", C.c_int64), ("slice_pitch_bytes", C.c_int64),
                ("format", C.c_int32), ("reserved", C.c_int32)]


class PostParams(C.Structure):
    _fields_ = [("bloom_threshold", C.c_float), ("bloom_strength", C.c_float), ("max_mips", C.c_uint32),
                ("reserved", C.c_uint32)]


class PostInfo(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("mip_count", C.c_uint32), ("reserved0", C.c_uint32),
                ("bloom_bytes", C.c_uint64), ("mip_width", C.c_uint32 * 16), ("mip_height", C.c_uint32 * 16),
                ("mip_ptr", C.c_void_p * 16)]


class VisionData(C.Structure):
    _fields_ = [("rgb", C.POINTER(C.c_uint8)), ("depth", C.POINTER(C.c_float)), ("width", C.c_uint32),
                ("height", C.c_uint32), ("fov_horizontal", C.c_double)]


class EyeDesc(C.Structure):
    _fields_ = [("n_eyes", C.c_uint32), ("widths", C.POINTER(C.c_uint32)), ("heights", C.POINTER(C.c_uint32)),
                ("fov_horizontal", C.POINTER(C.c_double)), ("ring", C.c_uint32), ("device", C.c_int),
                ("host_buffer", C.c_void_p), ("host_bytes", C.c_uint64)]


# (name, restype, argtypes) of every entry point declared in include/*.h.
_P = C.c_void_p
SIGNATURES = {
    "tg_svgf_params_default": (C.c_int, [C.c_int32, C.c_int32, C.POINTER(Params)]),
    "tg_svgf_create": (C.c_int, [C.POINTER(Desc), C.POINTER(_P)]),
    "tg_svgf_denoise": (C.c_int, [_P, C.POINTER(Inputs), C.POINTER(Outputs), _P]),
    "tg_svgf_denoise_host": (C.c_int, [_P, C.POINTER(Inputs), C.POINTER(Outputs), _P]),
    "tg_svgf_synchronize": (C.c_int, [_P]),
    "tg_svgf_reset": (C.c_int, [_P, _P]),
    "tg_svgf_resize": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "tg_svgf_get_info": (C.c_int, [_P, C.POINTER(Info)]),
    "tg_svgf_destroy": (None, [_P]),
    "tg_status_string": (C.c_char_p, [C.c_int]),
    "tg_last_error": (C.c_char_p, []),
    "tg_svgf_state_bytes": (C.c_uint64, [C.POINTER(Params), C.c_uint32, C.c_uint32]),
    "tg_svgf_profile_enable": (C.c_int, [_P, C.c_int]),
    "tg_svgf_profile_read": (C.c_int, [_P, C.POINTER(KernelStat), C.c_int, C.POINTER(C.c_int), C.c_int]),
    "tg_svgf_batch_create": (C.c_int, [C.POINTER(BatchDesc), C.POINTER(_P)]),
    "tg_svgf_batch_denoise": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(Inputs),
                                        C.POINTER(Outputs), _P]),
    "tg_svgf_batch_autotune": (C.c_int, [_P, C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(Inputs),
                                         C.POINTER(Outputs), C.c_uint32, _P]),
    "tg_svgf_batch_reset_stream": (C.c_int, [_P, C.c_uint32, _P]),
    "tg_svgf_batch_synchronize": (C.c_int, [_P]),
    "tg_svgf_batch_get_info": (C.c_int, [_P, C.POINTER(BatchInfo)]),
    "tg_svgf_batch_destroy": (None, [_P]),
    "tg_svgf_server_create": (C.c_int, [C.POINTER(ServerDesc), C.POINTER(_P)]),
    "tg_svgf_server_submit": (C.c_int, [_P, C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(Inputs),
                                        C.POINTER(Outputs), C.POINTER(C.c_uint64)]),
    "tg_svgf_server_wait": (C.c_int, [_P, C.c_uint64, C.c_int64, C.POINTER(RequestInfo)]),
    "tg_svgf_server_end_session": (C.c_int, [_P, C.c_uint64]),
    "tg_svgf_server_get_stats": (C.c_int, [_P, C.POINTER(ServerStats), C.c_int]),
    "tg_svgf_server_destroy": (None, [_P]),
    "tg_svgf_denoise_ref_noalloc": (C.c_int, [C.POINTER(Params), C.c_uint32, C.c_uint32, C.POINTER(Image),
                                              C.POINTER(Image), C.POINTER(Image), C.POINTER(Image), _P]),
    "tg_fog_filter": (C.c_int, [C.POINTER(FogParams), C.POINTER(Volume), C.POINTER(Volume), C.POINTER(Volume), _P]),
    "tg_post_params_default": (C.c_int, [C.POINTER(PostParams)]),
    "tg_post_create": (C.c_int, [C.c_uint32, C.c_uint32, C.POINTER(PostParams), C.c_int, C.POINTER(_P)]),
    "tg_post_process": (C.c_int, [_P, C.POINTER(Image), C.POINTER(Image), _P]),
    "tg_post_resize": (C.c_int, [_P, C.c_uint32, C.c_uint32]),
    "tg_post_get_info": (C.c_int, [_P, C.POINTER(PostInfo)]),
    "tg_post_destroy": (None, [_P]),
    "tg_eye_host_bytes": (C.c_uint64, [C.c_uint32, C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.c_uint32]),
    "tg_eye_create": (C.c_int, [C.POINTER(EyeDesc), C.POINTER(_P)]),
    "tg_eye_submit": (C.c_int, [_P, C.c_uint64, C.POINTER(Image), C.POINTER(Image), _P]),
    "tg_eye_acquire": (C.c_int, [_P, C.c_uint64, C.POINTER(VisionData)]),
    "tg_eye_destroy": (None, [_P]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Loads libtg_svgf.so (once) and declares every signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(the SVGF denoiser has no CPU fallback)")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int):
    if status != OK:
        msg = load().tg_last_error()
        raise TgError(status, msg.decode() if msg else "tg_svgf error")
    return status


def default_params(mode: int = MODE_FULL, storage: int = STORAGE_FP32, **overrides) -> Params:
    p = Params()
    check(load().tg_svgf_params_default(mode, storage, C.byref(p)))
    for k, v in overrides.items():
        setattr(p, k, v)
    return p
