"""GPU parity at the benchmarked sizes: the FULL chain through the C ABI against the CPU oracle on the
60-frame camera sequence (yaw 0.5 deg + 0.05 m per frame, a plane that appears at frame 30).

What only full-size frames exercise: the stride-16 level's 240 x 135 sub-lattice at 4K (tiles 88% full),
grids of 16-18k CTAs, interior and border tiles side by side across a whole frame, and the frame-30
disocclusion and the cut back to frame 0 at full resolution.  Frames are generated on the GPU, denoised
there, and copied to the host for the oracle, which runs every frame so that its state carries over.

Tolerances (as in test_gpu_parity.py)
* FP32 storage: per-pixel relative luminance error <= 1e-4 against the float32 oracle; relative L2
  luminance error <= 1e-4 against the float64 oracle where it runs (1920x1080).
* FP16 storage (binary16 radiance, history, moments, octahedral normals; float32 a-trous scratch):
  per-pixel <= 2^-8 and mean <= 1e-4 against the float32 oracle that rounds the same stores.  Against the
  float64 oracle, with an RGBA32F output image: per-pixel relative luminance error <= 1e-3 when the float64
  oracle denoises the same binary16 radiance and octahedral normals (the error of the FP16 state itself:
  history, moments, temporally integrated colour), and relative L2 <= 1e-4 with per-pixel <= 1.5e-3 when
  it denoises the full-precision inputs (the rounding of the radiance to binary16 alone moves a pixel by up
  to about 0.9e-3 at 1920x1080).
"""
import numpy as np
import pytest
import torch

import oracle
import tron_grid_gb300 as tg
from tron_grid_gb300 import scene
from tests.helpers import REL_TOL, rel_err, rel_l2, report

pytestmark = pytest.mark.gpu

KEYS = ("radiance", "depth", "normal", "motion")
FP16_REL_TOL = 1e-3         # against float64 on the same binary16 / octahedral inputs
FP16_INPUT_REL_TOL = 1.5e-3  # against float64 on the full-precision inputs


def _sequence(W, H, order, storage, check, with_f64, dev):
    """Denoises frames `order` of the 60-frame sequence at W x H in that order on the GPU and in the oracle
    (float32 with the storage form's rounding; with `with_f64` also float64 on the full-precision inputs and,
    for FP16 storage, float64 on the same binary16 radiance and octahedral normals the GPU gets), calling
    check(t, gpu, r32, r64, r64q) for each frame (r64q is r64 for FP32 storage)."""
    sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=0), device=dev)
    f16 = storage == tg.STORAGE_FP16
    den = tg.Denoiser(W, H, mode=tg.MODE_FULL, storage=storage)
    P = oracle.full_params()
    st32 = oracle.FullState(H, W, np.float32)
    st64 = oracle.FullState(H, W, np.float64) if with_f64 else None
    st64q = oracle.FullState(H, W, np.float64) if with_f64 and f16 else None
    out = torch.empty((H, W, 4), dtype=torch.float32, device=dev)
    mask = oracle.fp16_storage_mask(False) if f16 else 0
    for t in order:
        fr = sc.frame(t)
        rad, dep, nrm, mot = (fr[k] for k in KEYS)
        if f16:
            rad_d, nrm_d = rad.half(), scene.oct16_encode(nrm)
            rad_np = rad_d.float().cpu().numpy()
            nrm_np = oracle.oct16_decode(nrm_d.cpu().numpy())
        else:
            rad_d, nrm_d = rad, nrm
            rad_np, nrm_np = rad.cpu().numpy(), nrm.cpu().numpy()
        den.denoise(rad_d, dep, nrm_d, mot, out=out)
        g = out.cpu().numpy()
        dep_np, mot_np = dep.cpu().numpy(), mot.cpu().numpy()
        r32, _ = oracle.full_frame(P, st32, rad_np, dep_np, nrm_np, mot_np, fp16_store=mask)
        r64 = r64q = None
        if with_f64:
            r64, _ = oracle.full_frame(P, st64, rad.cpu().numpy(), dep_np, nrm.cpu().numpy(), mot_np)
            r64q = oracle.full_frame(P, st64q, rad_np, dep_np, nrm_np, mot_np)[0] if f16 else r64
        check(t, g, r32, r64, r64q)
    den.synchronize()
    assert den.info()["device_errors"] == 0
    den.close()


def _check_fp32(t, g, r32, r64, r64q):
    assert np.all(np.isfinite(g)), f"frame {t}: non-finite output"
    e = rel_err(g, r32)
    assert e.max() <= REL_TOL, f"frame {t}: max rel err {e.max():.3e} vs float32 oracle ({report(g, r32)})"
    assert np.all(g[..., 3] == 1.0)
    if r64 is not None:
        assert rel_l2(g, r64) <= 1e-4, f"frame {t}: rel L2 vs float64 {rel_l2(g, r64):.3e}"


def test_full_fp32_1080p_whole_sequence_and_cut(cuda_dev):
    """1920x1080, all 60 frames (the plane appears at frame 30), then frame 0 again: a camera cut, where every
    pixel loses its history and takes the 7x7 spatial variance."""
    _sequence(1920, 1080, list(range(60)) + [0], tg.STORAGE_FP32, _check_fp32, True, cuda_dev)


def test_full_fp32_4k_sequence(cuda_dev):
    """3840x2160, all 60 frames in order against the float32 oracle; frames 0, 1, 4, 29, 30, 31 and 59 are the
    events (first frame, first reprojection, the end of the spatial-variance window, the frames around the
    disocclusion, the last frame)."""
    _sequence(3840, 2160, list(range(60)), tg.STORAGE_FP32, _check_fp32, False, cuda_dev)


def _check_fp16(t, g, r32, r64, r64q):
    assert np.all(np.isfinite(g)), f"frame {t}: non-finite output"
    e = rel_err(g, r32)
    assert e.max() <= 2.0 ** -8, f"frame {t}: max rel {e.max():.3e} vs the emulating oracle"
    assert e.mean() <= 1e-4, f"frame {t}: mean rel {e.mean():.3e} vs the emulating oracle"
    if r64q is not None:
        eq = rel_err(g, r64q)
        assert eq.max() <= FP16_REL_TOL, f"frame {t}: max rel {eq.max():.3e} vs float64, same inputs ({report(g, r64q)})"
        e64 = rel_err(g, r64)
        assert e64.max() <= FP16_INPUT_REL_TOL, f"frame {t}: max rel {e64.max():.3e} vs float64 ({report(g, r64)})"
        assert rel_l2(g, r64) <= 1e-4, f"frame {t}: rel L2 vs float64 {rel_l2(g, r64):.3e}"


def test_full_fp16_4k_events(cuda_dev):
    """FP16 storage at 3840x2160, frames 0..31 in order (through the disocclusion) against the oracle that
    rounds the same stores."""
    _sequence(3840, 2160, list(range(32)), tg.STORAGE_FP16, _check_fp16, False, cuda_dev)


def test_full_fp16_1080p_against_float64(cuda_dev):
    """FP16 storage at 1920x1080 over the whole sequence: every pixel of every frame within 1e-3 relative
    luminance of the float64 oracle on the same inputs (RGBA32F output image)."""
    _sequence(1920, 1080, list(range(60)), tg.STORAGE_FP16, _check_fp16, True, cuda_dev)
