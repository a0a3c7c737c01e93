"""GPU parity of the froxel filter (tg_fog_filter) against the oracle and the reference shader's outputs.

Every add, multiply, divide and square root of the kernel's projection path is an IEEE-rounded operation
in the reference's order, as in the oracle; the slice depth pow and its inverse log are CUDA's powf / logf
against the host's, so results agree exactly except where those differ in the last place.  Tolerances
(written here): rgba16f outputs within 1 fp16 ulp, rgba32f outputs within 1e-5 relative to the volume's scale;
at most 0.05% of froxels may differ more (a froxel on a rejection boundary whose decision flips with the last
place of powf / logf).
"""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tron-grid_gb300"))

import oracle  # noqa: E402
import fog_scene  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "fog_*.npz")))
OUTLIER_FRAC = 5e-4


def _ulp16(a, b):
    ia = np.asarray(a, np.float16).view(np.int16).astype(np.int32)
    ib = np.asarray(b, np.float16).view(np.int16).astype(np.int32)
    ia = np.where(ia < 0, -32768 - ia, ia)
    ib = np.where(ib < 0, -32768 - ib, ib)
    return np.abs(ia - ib)


def check(got, want, f16, scale, what=""):
    got = np.asarray(got, np.float32)
    want = np.asarray(want, np.float32)
    if f16:
        bad = (_ulp16(got, want) > 1).any(-1)
    else:
        bad = (np.abs(got - want) > 1e-5 * max(scale, 1e-30)).any(-1)
    frac = float(bad.mean())
    exact = float((got == want).all(-1).mean())
    assert frac <= OUTLIER_FRAC, f"{what}: {frac:.2e} of froxels beyond tolerance (exact {exact:.4f})"
    return exact


def _run(tg, blk_args_or_params, raw, hist, out_dtype, dev, raw_dtype=None):
    import torch

    p = blk_args_or_params
    r = torch.from_numpy(raw).to(dev, raw_dtype or out_dtype)
    h = torch.from_numpy(hist).to(dev, out_dtype)
    o = torch.full_like(h, float("nan"))
    tg.fog_filter(p, r, h, o)
    torch.cuda.synchronize()
    return o.float().cpu().numpy()


def _params_from_block(blk):
    import ctypes as C

    from tron_grid_gb300 import _lib as L

    p = L.FogParams()
    C.memmove(C.addressof(p), blk, C.sizeof(p))
    return p


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("f16", [True, False])
def test_matches_reference_outputs(cuda_dev, path, f16):
    """The reference shader's own outputs (tests/golden), frame by frame along its history chain."""
    import torch

    import tron_grid_gb300 as tg

    z = np.load(path)
    blocks, raw, want = z["params"], z["raw"], z["out_f16" if f16 else "out_f32"]
    dt = torch.float16 if f16 else torch.float32
    hist = np.zeros_like(raw[0])
    for t in range(len(blocks)):
        got = _run(tg, _params_from_block(blocks[t].tobytes()), raw[t], hist, dt, cuda_dev)
        check(got, want[t], f16, float(np.abs(want[t]).max()), f"{os.path.basename(path)} frame {t}")
        hist = want[t]


@pytest.mark.parametrize("f16", [True, False])
def test_scene_sequence_against_oracle(cuda_dev, f16):
    """A moving camera over the reference's froxel depth range; the GPU's own output is the next history."""
    import torch

    import tron_grid_gb300 as tg

    sp = fog_scene.FogSpec(width=64, height=36, depth=24, yaw_deg=1.5, translation=(0.05, 0.0, -0.4))
    sc = fog_scene.FogScene(sp, device=cuda_dev)
    dt = torch.float16 if f16 else torch.float32
    ff = tg.FogFilter(sp.width, sp.height, sp.depth, dtype=dt, device=cuda_dev)
    hist = np.zeros((sp.depth, sp.height, sp.width, 4), np.float32)
    exact = []
    for t in range(6):
        args = sc.param_args(t)
        raw = sc.inject(t, dtype=torch.float16)
        out = ff.step(tg.fog_params(**args), raw)
        torch.cuda.synchronize()
        got = out.float().cpu().numpy()
        want = oracle.fog_filter(oracle.fog_param_block(**args), raw.float().cpu().numpy(), hist, fp16_store=f16)
        exact.append(check(got, want, f16, float(np.abs(want).max()), f"frame {t}"))
        hist = got
    # fp16 stores absorb the last-place powf / logf differences almost everywhere; fp32 stores show them
    assert min(exact) > (0.99 if f16 else 0.9)


@pytest.mark.parametrize("raw16,out16", [(False, True), (True, False)])
def test_mixed_formats_and_padded_pitches(cuda_dev, raw16, out16):
    import torch

    import tron_grid_gb300 as tg

    sp = fog_scene.FogSpec(width=37, height=23, depth=9, yaw_deg=2.0)
    sc = fog_scene.FogScene(sp)
    args = sc.param_args(1)
    rng = np.random.default_rng(5)
    raw = rng.uniform(0, 3, (9, 23, 37, 4)).astype(np.float16).astype(np.float32)
    hist = rng.uniform(0, 3, (9, 23, 37, 4)).astype(np.float16).astype(np.float32)
    rdt = torch.float16 if raw16 else torch.float32
    odt = torch.float16 if out16 else torch.float32
    # padded rows and slices: views into larger allocations
    rbig = torch.zeros((9, 25, 41, 4), dtype=rdt, device=cuda_dev)
    hbig = torch.zeros((10, 23, 40, 4), dtype=odt, device=cuda_dev)
    obig = torch.full((9, 24, 39, 4), float("nan"), dtype=odt, device=cuda_dev)
    r = rbig[:, :23, :37]
    h = hbig[:9, :, :37]
    o = obig[:, :23, :37]
    r.copy_(torch.from_numpy(raw).to(cuda_dev, rdt))
    h.copy_(torch.from_numpy(hist).to(cuda_dev, odt))
    tg.fog_filter(tg.fog_params(**args), r, h, o)
    torch.cuda.synchronize()
    want = oracle.fog_filter(oracle.fog_param_block(**args), raw, hist, fp16_store=out16)
    check(o.float().cpu().numpy(), want, out16, 3.0, "mixed formats")
    assert torch.isnan(obig[:, 23:]).all() and torch.isnan(obig[:, :, 37:]).all()  # padding untouched


@pytest.mark.parametrize("dims", [(1, 1, 1), (3, 2, 1), (1, 7, 5), (33, 9, 2)])
def test_small_and_ragged_grids(cuda_dev, dims):
    import torch

    import tron_grid_gb300 as tg

    w, h, d = dims
    sc = fog_scene.FogScene(fog_scene.FogSpec(width=w, height=h, depth=d, yaw_deg=1.0))
    rng = np.random.default_rng(w * 100 + h * 10 + d)
    raw = rng.uniform(0, 1, (d, h, w, 4)).astype(np.float16).astype(np.float32)
    hist = rng.uniform(0, 1, (d, h, w, 4)).astype(np.float16).astype(np.float32)
    for t in (0, 1):
        args = sc.param_args(t)
        got = _run(tg, tg.fog_params(**args), raw, hist, torch.float16, cuda_dev)
        want = oracle.fog_filter(oracle.fog_param_block(**args), raw, hist, fp16_store=True)
        check(got, want, True, 1.0, f"{dims} frame {t}")


def test_reference_grid_full_size(cuda_dev):
    """The reference's 320x180x64 grid against the oracle over every froxel."""
    import torch

    import tron_grid_gb300 as tg

    sp = fog_scene.fog_config()
    sc = fog_scene.FogScene(sp, device=cuda_dev)
    ff = tg.FogFilter(sp.width, sp.height, sp.depth, device=cuda_dev)
    hist = np.zeros((sp.depth, sp.height, sp.width, 4), np.float32)
    for t in range(3):
        args = sc.param_args(t)
        raw = sc.inject(t)
        got = ff.step(tg.fog_params(**args), raw).float().cpu().numpy()
        want = oracle.fog_filter(oracle.fog_param_block(**args), raw.float().cpu().numpy(), hist)
        exact = check(got, want, True, 1.0, f"frame {t}")
        assert exact > 0.99
        hist = got


def test_invalid_arguments(cuda_dev):
    import torch

    import tron_grid_gb300 as tg
    from tron_grid_gb300 import _lib as L

    sc = fog_scene.FogScene(fog_scene.FogSpec(width=8, height=4, depth=2))
    p = tg.fog_params(**sc.param_args(1))
    v = torch.zeros((2, 4, 8, 4), dtype=torch.float16, device=cuda_dev)
    w = torch.zeros_like(v)
    with pytest.raises(L.TgError) as e:
        tg.fog_filter(p, v, w, v)  # output overlaps inject_raw
    assert e.value.status == L.ERR_INVALID
    with pytest.raises(L.TgError):
        tg.fog_filter(p, v, w.float(), v.clone())  # history and output formats differ
    bad = tg.fog_params(**dict(sc.param_args(1), near_plane=5.0, far_plane=1.0))
    with pytest.raises(L.TgError):
        tg.fog_filter(bad, v, w, v.clone())
    import ctypes as C

    vol = L.Volume(v.data_ptr() + 2, 0, 0, L.FMT_RGBA16F, 0)  # misaligned
    good = L.Volume(w.data_ptr(), 0, 0, L.FMT_RGBA16F, 0)
    out = torch.zeros_like(v)
    vo = L.Volume(out.data_ptr(), 0, 0, L.FMT_RGBA16F, 0)
    assert L.load().tg_fog_filter(C.byref(p), C.byref(vol), C.byref(good), C.byref(vo), None) == L.ERR_INVALID
