"""The entry point that allocates nothing (tg_svgf_denoise_ref_noalloc).

It serves callers that cannot allocate device memory while they denoise (a
real-time render thread, a plug-in host with a fixed budget): they pass every
image, moments included, and the wavelet scratch lives in a fixed array inside
the library.  Checked through the C ABI against the handle-based entry point on
two frames in a row, with the tolerance of the other parity tests.  This file is
collected last so that a run that stops at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest
import torch

import tron_grid_gb300 as tg
from tron_grid_gb300 import _lib as L
from tron_grid_gb300 import scene
from tron_grid_gb300.svgf import image
from tests.helpers import REL_TOL, rel_err

pytestmark = pytest.mark.gpu


def _mom_image(t, fmt):
    return L.Image(t.data_ptr(), 0, fmt, 0)


def _call(lib, params, W, H, raw, prev, cur, out, mom_fmt, stream):
    return lib.tg_svgf_denoise_ref_noalloc(C.byref(params), W, H, C.byref(image("radiance", raw)),
                                           C.byref(_mom_image(prev, mom_fmt)), C.byref(_mom_image(cur, mom_fmt)),
                                           C.byref(image("denoised", out)), stream)


# (storage, width, height, levels): a small frame, the largest frames the header names for the default 3 levels
# (1280x720 fp16 needs 14.7 MB of the 16 MiB, 960x540 fp32 16.6 MB), and two non-default level counts.
CASES = [(L.STORAGE_FP16, 320, 180, 3), (L.STORAGE_FP32, 320, 180, 3), (L.STORAGE_FP16, 1280, 720, 3),
         (L.STORAGE_FP32, 960, 540, 3), (L.STORAGE_FP16, 640, 360, 5), (L.STORAGE_FP32, 320, 180, 7)]


@pytest.mark.parametrize("storage,W,H,levels", CASES)
def test_noalloc_matches_handle_on_two_frames(cuda_dev, storage, W, H, levels):
    lib = L.load()
    f16 = storage == L.STORAGE_FP16
    dt = torch.float16 if f16 else torch.float32
    mom_fmt = L.FMT_RG16F if f16 else L.FMT_RG32F
    params = L.default_params(L.MODE_REF_EXACT, storage, levels=levels)
    ref = tg.Denoiser(W, H, mode=L.MODE_REF_EXACT, storage=storage, levels=levels)
    moms = [torch.zeros((H, W, 2), dtype=dt, device=cuda_dev) for _ in range(2)]
    sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=21), device=cuda_dev)
    for t in range(2):
        raw = sc.frame(t)["radiance"].to(dt)
        want = torch.empty((H, W, 4), dtype=dt, device=cuda_dev)
        ref.denoise(raw, out=want)
        got = torch.empty((H, W, 4), dtype=dt, device=cuda_dev)
        prev, cur = moms[(t + 1) % 2], moms[t % 2]
        st = _call(lib, params, W, H, raw, prev, cur, got, mom_fmt, torch.cuda.current_stream().cuda_stream)
        assert st == L.OK, lib.tg_last_error()
        g = got.float().cpu().numpy()
        w = want.float().cpu().numpy()
        assert np.all(np.isfinite(g))
        assert rel_err(g, w).max() <= REL_TOL, f"frame {t}"
    ref.close()


# (storage, levels, largest frame that fits, the frame one pixel wider that does not)
LIMITS = [(L.STORAGE_FP32, 3, (968, 540), (969, 540)), (L.STORAGE_FP16, 3, (1456, 720), (1457, 720)),
          (L.STORAGE_FP32, 10, (384, 216), (960, 540))]


@pytest.mark.parametrize("storage,levels,fits,too_big", LIMITS)
def test_noalloc_rejects_frames_beyond_its_scratch(cuda_dev, storage, levels, fits, too_big):
    """A frame whose two wavelet images (padded for every level's layout) exceed the 16 MiB array is rejected
    before anything is launched; the largest frame that fits runs."""
    lib = L.load()
    f16 = storage == L.STORAGE_FP16
    dt = torch.float16 if f16 else torch.float32
    mom_fmt = L.FMT_RG16F if f16 else L.FMT_RG32F
    params = L.default_params(L.MODE_REF_EXACT, storage, levels=levels)
    for (W, H), want in ((too_big, L.ERR_INVALID), (fits, L.OK)):
        raw = torch.zeros((H, W, 4), dtype=dt, device=cuda_dev)
        prev = torch.zeros((H, W, 2), dtype=dt, device=cuda_dev)
        cur = torch.empty_like(prev)
        out = torch.empty_like(raw)
        st = _call(lib, params, W, H, raw, prev, cur, out, mom_fmt, None)
        assert st == want, (W, H, lib.tg_last_error())
        if want == L.ERR_INVALID:
            assert b"scratch" in lib.tg_last_error()
        else:
            torch.cuda.synchronize()
            assert torch.all(out[..., 3] == 1)
