"""The froxel-filter oracle (a restatement of src/volumetric_filter.slang:142-226), pinned against the
reference shader itself: its outputs recorded in tests/golden/fog_*.npz and, where the reference checkout is
present, the shader compiled as C++; plus closed-form known answers."""
import glob
import os
import struct
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tron-grid_gb300"))

import oracle  # noqa: E402
import fog_scene  # noqa: E402

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "fog_*.npz")))


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 4


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("f16", [True, False])
def test_restatement_matches_reference_outputs(path, f16):
    """Bit-exact against the reference shader's own outputs, frame by frame along its history chain."""
    z = np.load(path)
    blocks, raw, want = z["params"], z["raw"], z["out_f16" if f16 else "out_f32"]
    hist = np.zeros_like(raw[0])
    for t in range(len(blocks)):
        got = oracle.fog_filter(blocks[t].tobytes(), raw[t], hist, fp16_store=f16)
        np.testing.assert_array_equal(got, want[t], err_msg=f"frame {t}")
        hist = want[t]


@pytest.mark.skipif(not oracle.fog_reference_available(), reason="reference checkout not present")
def test_restatement_matches_compiled_reference_on_scene():
    sp = fog_scene.FogSpec(width=40, height=24, depth=12, yaw_deg=2.0, translation=(0.1, 0.0, -0.3))
    sc = fog_scene.FogScene(sp)
    import torch

    hist = np.zeros((sp.depth, sp.height, sp.width, 4), np.float32)
    for t in range(4):
        blk = oracle.fog_param_block(**sc.param_args(t))
        raw = sc.inject(t, dtype=torch.float16).float().numpy()
        a = oracle.fog_filter(blk, raw, hist)
        b = oracle.fog_filter_reference(blk, raw, hist)
        np.testing.assert_array_equal(a, b)
        hist = a


def _block(**kw):
    args = dict(inv_view_projection=np.eye(4), prev_view_projection=np.eye(4), camera_pos=[0, 0, 0], alpha=0.25,
                width=7, height=5, depth=6, history_valid=1, near_plane=0.1, far_plane=120.0)
    args.update(kw)
    return oracle.fog_param_block(**args), args


def test_no_history_is_the_box_mean():
    blk, a = _block(history_valid=0)
    raw = np.zeros((6, 5, 7, 4), np.float32)
    raw[2, 2, 3] = 9.0      # interior impulse
    raw[4, 0, 0] = 4.0      # corner impulse
    out = oracle.fog_filter(blk, raw, np.full_like(raw, 7.0), fp16_store=False)
    np.testing.assert_allclose(out[2, 1:4, 2:5], 1.0)          # 9 / 9 over the interior 3x3
    assert out[2, 0, 0].max() == 0.0 and out[1].max() == 0.0  # other slices untouched
    # the corner froxel averages its 4 in-grid members, its edge neighbours 6, the next diagonal 9
    np.testing.assert_allclose(out[4, 0:2, 0:2, 0], [[4 / 4, 4 / 6], [4 / 6, 4 / 9]], rtol=1e-6)
    np.testing.assert_allclose(out[4, 0, 2], 0.0)


def _camera(yaw_deg=0.0, eye=(0.0, 1.7, 0.0), w=7, h=5):
    sp = fog_scene.FogSpec(width=w, height=h)
    proj = fog_scene.perspective(np.radians(60.0), w / h, sp.near, sp.far)
    th = np.radians(yaw_deg)
    e = np.asarray(eye, np.float64)
    view = fog_scene.look_at(e, e + np.array([-np.sin(th), 0.0, -np.cos(th)]))
    return proj @ view, e


def test_static_camera_blends_constant_history():
    """Identical cameras: every froxel of the inner slices reprojects inside the grid; with constant raw and
    history the trilinear fetch is exact, so out = h + (r - h) * alpha."""
    vp, eye = _camera()
    blk, a = _block(inv_view_projection=np.linalg.inv(vp), prev_view_projection=vp, camera_pos=eye)
    raw = np.full((6, 5, 7, 4), 2.0, np.float32)
    hist = np.full_like(raw, 10.0)
    out = oracle.fog_filter(blk, raw, hist, fp16_store=False)
    want = np.float32(10.0) + (np.float32(2.0) - np.float32(10.0)) * np.float32(0.25)
    np.testing.assert_array_equal(out[1:-1], want)


@pytest.mark.parametrize("case", ["behind", "beyond_far"])
def test_rejected_history_keeps_the_spatial_mean(case):
    vp, eye = _camera()
    if case == "behind":
        pvp, _ = _camera(yaw_deg=180.0)
    else:
        pvp, _ = _camera(eye=(0.0, 1.7, 300.0))
    blk, _ = _block(inv_view_projection=np.linalg.inv(vp), prev_view_projection=pvp, camera_pos=eye)
    raw = np.random.default_rng(0).uniform(0, 1, (6, 5, 7, 4)).astype(np.float32)
    out = oracle.fog_filter(blk, raw, np.full_like(raw, 50.0), fp16_store=False)
    blk0 = bytearray(blk)
    struct.pack_into("<I", blk0, 39 * 4, 0)
    np.testing.assert_array_equal(out, oracle.fog_filter(bytes(blk0), raw, raw, fp16_store=False))


def test_float_and_double_agree():
    sp = fog_scene.FogSpec(width=24, height=14, depth=8, yaw_deg=1.0)
    sc = fog_scene.FogScene(sp)
    import torch

    blk = oracle.fog_param_block(**sc.param_args(2))
    raw = sc.inject(2, dtype=torch.float32).numpy()
    hist = sc.inject(1, dtype=torch.float32).numpy()
    a = oracle.fog_filter(blk, raw, hist, fp16_store=False)
    b = oracle.fog_filter(blk, raw, hist, fp16_store=False, dtype=np.float64)
    assert np.abs(a - b).max() <= 1e-5 * max(1.0, float(np.abs(b).max()))


def test_product_param_block_is_the_oracle_block():
    """The product's tg_fog_filter_params bytes equal the oracle's (and the reference's 176-byte layout)."""
    import ctypes as C

    from tron_grid_gb300 import fog

    sc = fog_scene.FogScene(fog_scene.FogSpec(width=24, height=14, depth=8))
    args = sc.param_args(3)
    p = fog.make_params(**args)
    assert C.sizeof(p) == oracle.FOG_PARAM_BYTES == 176
    assert fog.param_bytes(p) == oracle.fog_param_block(**args)
