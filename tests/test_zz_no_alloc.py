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


@pytest.mark.parametrize("storage", [L.STORAGE_FP16, L.STORAGE_FP32])
def test_noalloc_matches_handle_on_two_frames(cuda_dev, storage):
    W, H = 320, 180
    lib = L.load()
    f16 = storage == L.STORAGE_FP16
    dt = torch.float16 if f16 else torch.float32
    mom_fmt = L.FMT_RG16F if f16 else L.FMT_RG32F
    params = L.default_params(L.MODE_REF_EXACT, storage)
    ref = tg.Denoiser(W, H, mode=L.MODE_REF_EXACT, storage=storage)
    moms = [torch.zeros((H, W, 2), dtype=dt, device=cuda_dev) for _ in range(2)]
    sc = scene.PlaneScene(scene.config0(seed=21))
    for t in range(2):
        raw = sc.frame(t)["radiance"].to(dt).to(cuda_dev)
        want = torch.empty((H, W, 4), dtype=dt, device=cuda_dev)
        ref.denoise(raw, out=want)
        got = torch.empty((H, W, 4), dtype=dt, device=cuda_dev)
        prev, cur = moms[(t + 1) % 2], moms[t % 2]
        st = lib.tg_svgf_denoise_ref_noalloc(C.byref(params), W, H, C.byref(image("radiance", raw)),
                                             C.byref(_mom_image(prev, mom_fmt)), C.byref(_mom_image(cur, mom_fmt)),
                                             C.byref(image("denoised", got)),
                                             torch.cuda.current_stream().cuda_stream)
        assert st == L.OK, lib.tg_last_error()
        g = got.float().cpu().numpy()
        w = want.float().cpu().numpy()
        assert rel_err(g, w).max() <= REL_TOL, f"frame {t}"
        assert np.all(np.isfinite(g))
    ref.close()


def test_noalloc_rejects_frames_beyond_its_scratch(cuda_dev):
    lib = L.load()
    W, H = 1920, 1080
    params = L.default_params(L.MODE_REF_EXACT, L.STORAGE_FP16)
    raw = torch.zeros((H, W, 4), dtype=torch.float16, device=cuda_dev)
    mom = torch.zeros((H, W, 2), dtype=torch.float16, device=cuda_dev)
    out = torch.empty_like(raw)
    st = lib.tg_svgf_denoise_ref_noalloc(C.byref(params), W, H, C.byref(image("radiance", raw)),
                                         C.byref(_mom_image(mom, L.FMT_RG16F)), C.byref(_mom_image(mom, L.FMT_RG16F)),
                                         C.byref(image("denoised", out)), None)
    assert st == L.ERR_INVALID
    assert b"scratch" in lib.tg_last_error()
