"""GB300-native SVGF denoiser for TronGrid (`src/svgf_denoise.slang`).

The compute lives in libtg_svgf.so (hand-written sm_103a CUDA behind the C ABI
of include/tg_svgf.h); this package is the host-side mirror used by tests and
benchmarks, plus the synthetic scene generator.
"""
from . import _lib
from ._lib import (MODE_FULL, MODE_REF_EXACT, STORAGE_FP16, STORAGE_FP32, TgError, default_params)
from .svgf import Denoiser, image, state_bytes

__all__ = ["Denoiser", "TgError", "MODE_FULL", "MODE_REF_EXACT", "STORAGE_FP16", "STORAGE_FP32", "default_params",
           "image", "state_bytes", "_lib"]
