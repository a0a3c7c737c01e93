"""GB300-native SVGF denoiser for TronGrid (`src/svgf_denoise.slang`), its
volumetric-fog froxel filter (`src/volumetric_filter.slang`), its bloom +
post-process chain (`src/bloom_downsample.slang`, `src/postprocess.slang`) and the
readback of AI entities' eye frames (`docs/AI_INTERFACE.md`, design only there).

The compute lives in libtg_svgf.so (hand-written sm_103a CUDA behind the C ABI
of include/tg_svgf.h, tg_fog.h, tg_post.h and tg_eye.h); this package is the host-side
mirror used by tests and benchmarks, plus the synthetic scene generators.
"""
from . import _lib
from ._lib import (MODE_FULL, MODE_REF_EXACT, STORAGE_FP16, STORAGE_FP32, TgError, default_params)
from .fog import FogFilter, fog_filter, make_params as fog_params
from .eye import EyeReadback
from .post import PostProcessor
from .svgf import Denoiser, image, state_bytes

__all__ = ["Denoiser", "TgError", "MODE_FULL", "MODE_REF_EXACT", "STORAGE_FP16", "STORAGE_FP32", "default_params",
           "image", "state_bytes", "FogFilter", "fog_filter", "fog_params", "PostProcessor", "EyeReadback", "_lib"]
