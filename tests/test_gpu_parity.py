"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Tolerances
* FP32 storage (both modes): per-pixel relative luminance error <= 1e-4
  (absolute floor 1e-7) against the oracle evaluated in float32.
* REF_EXACT with the reference's fp16 images: the GPU rounds to binary16 at
  every store exactly as the oracle does; a last-bit difference in an
  exponential can move one stored value by one fp16 step, so the bound is 2
  fp16 units in the last place per value and 99.9% of values identical.
* FULL with FP16 storage: against the float32 oracle with the same fp16 /
  octahedral storage emulation (per-pixel 2^-8, mean 1e-4: a last-place
  difference of an approximate SFU operation can flip one binary16 rounding of
  the history, and the flip persists through the EMA), and against the
  float64 oracle without emulation: relative L2 luminance error <= 1e-3
  (test_gpu_full_size.py bounds every pixel against float64).
"""
import numpy as np
import pytest
import torch

import oracle
import tron_grid_gb300 as tg
from tron_grid_gb300 import scene
from tests.helpers import LUM_FLOOR, REL_TOL, rel_err, rel_l2, report

pytestmark = pytest.mark.gpu

KEYS = ("radiance", "depth", "normal", "motion")


def _frames(spec, n):
    sc = scene.PlaneScene(spec)
    return [sc.frame(t) for t in range(n)]


def _run_full_pair(dev, spec, n_frames, storage=tg.STORAGE_FP32, fp16_inputs=False, check=None, params=None):
    W, H = spec.width, spec.height
    params = params or {}
    den = tg.Denoiser(W, H, mode=tg.MODE_FULL, storage=storage, **params)
    st32 = oracle.FullState(H, W, np.float32)
    st64 = oracle.FullState(H, W, np.float64)
    P = oracle.full_params(**params)
    f16 = storage == tg.STORAGE_FP16
    out_dt = torch.float16 if f16 else torch.float32
    results = []
    sc = scene.PlaneScene(spec)
    for t in range(n_frames):
        fr = sc.frame(t)
        rad, dep, nrm, mot = (fr[k] for k in KEYS)
        nrm_np = nrm.numpy()
        if fp16_inputs:
            rad_d = rad.to(torch.float16).to(dev)
            enc = oracle.oct16_encode(nrm_np)
            nrm_d = torch.from_numpy(enc).to(dev)
            rad_np = rad.to(torch.float16).float().numpy()
            nrm_np = oracle.oct16_decode(enc)
        else:
            rad_d, nrm_d = rad.to(dev), nrm.to(dev)
            rad_np = rad.numpy()
        out = torch.empty((H, W, 4), dtype=out_dt, device=dev)
        den.denoise(rad_d, dep.to(dev), nrm_d, mot.to(dev), out=out)
        g = out.float().cpu().numpy()
        r32, _ = oracle.full_frame(P, st32, rad_np, dep.numpy(), nrm_np, mot.numpy(),
                                   fp16_store=oracle.fp16_storage_mask(True) if f16 else 0)
        r64, _ = oracle.full_frame(P, st64, rad.numpy(), dep.numpy(), nrm.numpy(), mot.numpy(), fp16_store=False)
        results.append((g, r32, r64, fr))
        if check:
            check(t, g, r32, r64)
    den.close()
    return results


def _check_fp32(t, g, r32, r64):
    e = rel_err(g, r32)
    assert np.all(np.isfinite(g))
    assert e.max() <= REL_TOL, f"frame {t}: max rel err {e.max():.3e} vs float32 oracle ({report(g, r32)})"
    assert rel_l2(g, r64) <= 1e-4, f"frame {t}: rel L2 vs float64 {rel_l2(g, r64):.3e}"


def test_full_fp32_640x360_pan(cuda_dev):
    """640x360, 8 frames, yaw 0.2 deg/frame, 5 levels, sigma 4/128/1."""
    _run_full_pair(cuda_dev, scene.slow_pan(seed=1), 8, check=_check_fp32)


def test_full_fp32_motion_and_disocclusion(cuda_dev):
    """Yaw 0.5 deg + 0.05 m per frame with a plane appearing at frame 30 (320x180)."""
    spec = scene.pan_with_disocclusion(320, 180, seed=2)
    _run_full_pair(cuda_dev, spec, 33, check=_check_fp32)


@pytest.mark.parametrize("wh", [(1, 1), (2, 2), (7, 3), (33, 17), (5, 40)])
def test_full_fp32_odd_sizes(cuda_dev, wh):
    spec = scene.pan_with_disocclusion(wh[0], wh[1], seed=3)
    _run_full_pair(cuda_dev, spec, 5, check=_check_fp32)


def _check_fp16(t, g, r32, r64):
    e = rel_err(g, r32)
    assert np.all(np.isfinite(g))
    assert e.max() <= 2.0 ** -8, f"frame {t}: max rel {e.max():.3e} vs emulating oracle"
    assert e.mean() <= 1e-4, f"frame {t}: mean rel {e.mean():.3e} vs emulating oracle"
    l2 = rel_l2(g, r64)
    assert l2 <= 1e-3, f"frame {t}: rel L2 vs float64 oracle {l2:.3e}"


def test_full_fp16_storage(cuda_dev):
    """FP16 colour/moments, octahedral normals; FP16 radiance + OCT16 normal inputs."""
    _run_full_pair(cuda_dev, scene.pan_with_disocclusion(320, 180, seed=4), 33, storage=tg.STORAGE_FP16, fp16_inputs=True,
                   check=_check_fp16)


# Non-default parameters: every edge-stop width, both EMA weights, a shorter history cap and fallback window.
ODD_PARAMS = dict(sigma_l=2.5, sigma_n=64.0, sigma_z=0.5, alpha=0.1, moments_alpha=0.3, max_history=16,
                  fallback_frames=3)


@pytest.mark.parametrize("levels", [1, 2, 3, 4])
def test_full_fp32_level_counts_and_params(cuda_dev, levels):
    """Fewer a-trous levels (with one level, level 0 is also the last: staged from the planes, colour only)."""
    _run_full_pair(cuda_dev, scene.pan_with_disocclusion(96, 64, seed=5), 6, check=_check_fp32, params=dict(ODD_PARAMS, levels=levels))


@pytest.mark.parametrize("W", [96, 97])
def test_full_fp16_single_level(cuda_dev, W):
    """One FP16 level at an even width (level 0 by TMA from the planes) and an odd one (plain loads)."""
    _run_full_pair(cuda_dev, scene.pan_with_disocclusion(W, 64, seed=6), 6, storage=tg.STORAGE_FP16, fp16_inputs=True,
                   check=_check_fp16, params=dict(ODD_PARAMS, levels=1))


def _ref_pair(dev, spec, n, storage, check):
    W, H = spec.width, spec.height
    den = tg.Denoiser(W, H, mode=tg.MODE_REF_EXACT, storage=storage)
    f16 = storage == tg.STORAGE_FP16
    mom = np.zeros((H, W, 2), np.float32)
    sc = scene.PlaneScene(spec)
    for t in range(n):
        raw = sc.frame(t)["radiance"]
        if f16:
            raw = raw.to(torch.float16)
        out = torch.empty((H, W, 4), dtype=raw.dtype, device=dev)
        den.denoise(raw.to(dev), out=out)
        ref, mom = oracle.ref_frame(raw.float().numpy(), mom, fp16_store=f16)
        check(t, out.float().cpu().numpy(), ref)
    den.close()


def test_ref_exact_fp32(cuda_dev):
    def chk(t, g, r):
        e = rel_err(g, r)
        assert e.max() <= REL_TOL, f"frame {t}: {report(g, r)}"
        assert np.all(g[..., 3] == 1.0)

    _ref_pair(cuda_dev, scene.slow_pan(seed=5), 8, tg.STORAGE_FP32, chk)


def test_ref_exact_fp16_images(cuda_dev):
    """The reference's rgba16f / rg16f images (moments overflow to inf/NaN above luminance ~256, as in the reference)."""
    def chk(t, g, r):
        gb = g[..., :3].astype(np.float16).view(np.int16).astype(np.int32)
        rb = r[..., :3].astype(np.float16).view(np.int16).astype(np.int32)
        ulps = np.abs(gb - rb)  # all values are positive, so bit patterns are ordered
        assert ulps.max() <= 2, f"frame {t}: {ulps.max()} fp16 ulps apart"
        same = np.mean(g[..., :3] == r[..., :3])
        assert same >= 0.999, f"frame {t}: only {same:.5f} of values identical"

    _ref_pair(cuda_dev, scene.slow_pan(seed=6), 8, tg.STORAGE_FP16, chk)


@pytest.mark.parametrize("wh", [(1, 1), (2, 2), (7, 3), (33, 17)])
def test_ref_exact_odd_sizes(cuda_dev, wh):
    def chk(t, g, r):
        assert rel_err(g, r).max() <= REL_TOL

    _ref_pair(cuda_dev, scene.SceneSpec(wh[0], wh[1], seed=8), 4, tg.STORAGE_FP32, chk)


def _pinned(t, pad):
    """A pinned copy of `t` (H, W[, C]); with pad > 0 a view into rows of W + pad pixels (a pitched image)."""
    if not pad:
        return t.pin_memory()
    H, W = t.shape[0], t.shape[1]
    big = torch.zeros((H, W + pad) + tuple(t.shape[2:]), dtype=t.dtype).pin_memory()
    v = big[:, :W]
    v.copy_(t)
    return v


@pytest.mark.parametrize("pad", [0, 3])
@pytest.mark.parametrize("storage", [tg.STORAGE_FP32, tg.STORAGE_FP16])
def test_host_api_matches_device_api(cuda_dev, storage, pad):
    """tg_svgf_denoise_host (pinned host buffers, four frames through its ring of three staging sets) gives the
    device API's bits; FP16 storage with rgba16f radiance and octahedral normals.  pad > 0: every host image
    (inputs and output) is pitched (rows of W + pad pixels), which the host path copies row by row."""
    spec = scene.pan_with_disocclusion(200, 120, seed=9)
    frames = _frames(spec, 4)
    f16 = storage == tg.STORAGE_FP16
    if f16:
        for fr in frames:
            fr["radiance"] = fr["radiance"].half()
            fr["normal"] = torch.from_numpy(oracle.oct16_encode(fr["normal"].numpy()))
    dt = torch.float16 if f16 else torch.float32
    a = tg.Denoiser(200, 120, storage=storage)
    b = tg.Denoiser(200, 120, storage=storage)
    outs_h = []
    for fr in frames:
        ins = [_pinned(fr[k], pad) for k in KEYS]
        outs_h.append(b.denoise_host(*ins, out=_pinned(torch.zeros((120, 200, 4), dtype=dt), pad)))
    b.synchronize()
    for fr, oh in zip(frames, outs_h):
        od = a.denoise(*(fr[k].to(cuda_dev) for k in KEYS), out=torch.empty((120, 200, 4), dtype=dt, device=cuda_dev))
        assert torch.equal(od.cpu(), oh)
    a.close()
    b.close()


def test_reset_restarts_history(cuda_dev):
    spec = scene.pan_with_disocclusion(64, 48, seed=10)
    frames = _frames(spec, 3)
    d = tg.Denoiser(64, 48)
    first = d.denoise(*(frames[0][k].to(cuda_dev) for k in KEYS)).cpu()
    d.denoise(*(frames[1][k].to(cuda_dev) for k in KEYS))
    d.reset()
    again = d.denoise(*(frames[0][k].to(cuda_dev) for k in KEYS)).cpu()
    assert torch.equal(first, again)
    assert d.info()["frame_index"] == 1
    d.close()


@pytest.mark.parametrize("storage", [tg.STORAGE_FP32, tg.STORAGE_FP16])
def test_resize_rezeroes_state(cuda_dev, storage):
    """After resize (the reference's rebuildFrameBuffers, src/main.cpp:1547-1603) a handle behaves exactly as a
    fresh one of the new size; the caller's two outputs alternate as denoised_indirect[frame % 2]."""
    small = _frames(scene.pan_with_disocclusion(64, 48, seed=12), 2)
    big = _frames(scene.pan_with_disocclusion(96, 80, seed=13), 3)
    f16 = storage == tg.STORAGE_FP16

    def ins(fr):
        t = [fr[k].to(cuda_dev) for k in KEYS]
        if f16:
            t[0] = t[0].half()
            t[2] = scene.oct16_encode(t[2])
        return t

    dt = torch.float16 if f16 else torch.float32
    d = tg.Denoiser(64, 48, storage=storage)
    for fr in small:
        d.denoise(*ins(fr))
    d.resize(96, 80)
    fresh = tg.Denoiser(96, 80, storage=storage)
    outs = [torch.empty((80, 96, 4), dtype=dt, device=cuda_dev) for _ in range(2)]
    for t, fr in enumerate(big):
        a = d.denoise(*ins(fr), out=outs[t % 2])
        b = fresh.denoise(*ins(fr), out=torch.empty_like(outs[0]))
        assert torch.equal(a.cpu(), b.cpu()), f"frame {t}"
    assert d.info()["frame_index"] == 3
    d.close()
    fresh.close()


def test_input_layouts_agree(cuda_dev):
    """RGB32F vs RGBA32F vs pitched normals and pitched radiance give identical output."""
    W, H = 48, 40
    fr = _frames(scene.pan_with_disocclusion(W, H, seed=11), 1)[0]
    rad, dep, nrm, mot = (fr[k].to(cuda_dev) for k in KEYS)
    base = tg.Denoiser(W, H).denoise(rad, dep, nrm, mot).cpu()
    nrm4 = torch.cat([nrm, torch.zeros_like(nrm[..., :1])], -1)
    assert torch.equal(tg.Denoiser(W, H).denoise(rad, dep, nrm4, mot).cpu(), base)
    wide = torch.zeros((H, W + 7, 4), device=cuda_dev)
    wide[:, :W] = rad
    assert torch.equal(tg.Denoiser(W, H).denoise(wide[:, :W], dep, nrm, mot).cpu(), base)


def test_invalid_arguments_raise(cuda_dev):
    d = tg.Denoiser(32, 32)
    rad = torch.zeros((32, 32, 4), device=cuda_dev)
    dep = torch.zeros((32, 32), device=cuda_dev)
    nrm = torch.zeros((32, 32, 3), device=cuda_dev)
    with pytest.raises(tg.TgError) as e:  # FULL without motion
        d.denoise(rad, dep, nrm, None)
    assert e.value.status == tg._lib.ERR_INVALID
    with pytest.raises(ValueError):
        d.denoise(rad.double(), dep, nrm, torch.zeros((32, 32, 2), device=cuda_dev))
    d.close()


@pytest.mark.parametrize("storage", [tg.STORAGE_FP32, tg.STORAGE_FP16])
@pytest.mark.parametrize("W", [333, 334])
def test_tma_and_plain_staging_agree(cuda_dev, storage, W):
    """The a-trous tiles staged by the tensor-memory accelerator give the same bits as plain loads.  Level 0
    stages from the tc / guide / variance planes: by TMA at both widths for FP32, at the even width for FP16
    (8-byte texels need a row pitch that is a multiple of 16 bytes), with plain loads otherwise."""
    H = 197
    f16 = storage == tg.STORAGE_FP16
    a = tg.Denoiser(W, H, storage=storage)
    b = tg.Denoiser(W, H, storage=storage, flags=tg._lib.FLAG_NO_TMA)
    assert a.info()["tma"] == 1 and b.info()["tma"] == 0
    sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=12))
    dt = torch.float16 if f16 else torch.float32
    for t in range(6):
        fr = sc.frame(t)
        rad = fr["radiance"].to(dt).to(cuda_dev)
        nrm = torch.from_numpy(oracle.oct16_encode(fr["normal"].numpy())).to(cuda_dev) if f16 else fr["normal"].to(cuda_dev)
        args = (rad, fr["depth"].to(cuda_dev), nrm, fr["motion"].to(cuda_dev))
        oa = a.denoise(*args, out=torch.empty((H, W, 4), dtype=dt, device=cuda_dev))
        ob = b.denoise(*args, out=torch.empty((H, W, 4), dtype=dt, device=cuda_dev))
        assert torch.equal(oa, ob), f"frame {t}"
    a.synchronize()
    assert a.info()["device_errors"] == 0


@pytest.mark.parametrize("storage", [tg.STORAGE_FP32, tg.STORAGE_FP16])
@pytest.mark.parametrize("W,H,pitch_px", [(333, 197, 0), (334, 197, 0), (640, 360, 0), (640, 360, 648)])
def test_ref_exact_tma_and_plain_staging_agree(cuda_dev, storage, W, H, pitch_px):
    """REF_EXACT: interior tiles staged by the tensor-memory accelerator (the first pass from the caller's
    radiance, the later ones from the residue planes) give the same bits as plain loads, for radiance images
    that are tightly packed or pitched, in either storage format; a width whose plane rows are not a multiple
    of 16 bytes falls back to plain loads for that pass."""
    f16 = storage == tg.STORAGE_FP16
    dt = torch.float16 if f16 else torch.float32
    a = tg.Denoiser(W, H, mode=tg.MODE_REF_EXACT, storage=storage)
    b = tg.Denoiser(W, H, mode=tg.MODE_REF_EXACT, storage=storage, flags=tg._lib.FLAG_NO_TMA)
    assert a.info()["tma"] == 1 and b.info()["tma"] == 0
    sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=13), device=cuda_dev)
    for t in range(4):
        rad = sc.frame(t)["radiance"].to(dt)
        if pitch_px:
            big = torch.zeros((H, pitch_px, 4), dtype=dt, device=cuda_dev)
            big[:, :W] = rad
            rad = big[:, :W]
        oa = a.denoise(rad, out=torch.empty((H, W, 4), dtype=dt, device=cuda_dev))
        ob = b.denoise(rad, out=torch.empty((H, W, 4), dtype=dt, device=cuda_dev))
        assert torch.equal(oa, ob), f"frame {t}"
    a.synchronize()
    assert a.info()["device_errors"] == 0
    a.close()
    b.close()
