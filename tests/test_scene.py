"""The synthetic sequence generator (inputs of every parity test and the bench)."""
import math

import numpy as np
import torch

from tron_grid_gb300 import scene


def test_static_camera_has_zero_motion():
    sc = scene.PlaneScene(scene.SceneSpec(64, 36, seed=1, yaw_deg=0.0))
    fr = sc.frame(3)
    assert float(fr["motion"].abs().max()) < 1e-3


def test_geometry_is_valid():
    sc = scene.PlaneScene(scene.pan_with_disocclusion(80, 45, seed=2))
    fr = sc.frame(0)
    assert torch.all(fr["depth"] > 0) and torch.all(torch.isfinite(fr["depth"]))
    n = fr["normal"].norm(dim=-1)
    assert torch.allclose(n, torch.ones_like(n), atol=1e-5)
    assert torch.all(fr["radiance"][..., 3] == 1)


def test_noise_is_unit_mean_exponential():
    sc = scene.PlaneScene(scene.SceneSpec(256, 128, seed=3))
    fr = sc.frame(0)
    ratio = (fr["radiance"][..., :3] / fr["truth"][..., :3].clamp_min(1e-6)).flatten()
    assert abs(float(ratio.mean()) - 1.0) < 0.02
    assert abs(float(ratio.var()) - 1.0) < 0.05


def test_motion_vectors_reproject_to_same_surface():
    """A pixel moved by its motion vector lands, in the previous frame, on the same plane."""
    spec = scene.pan_with_disocclusion(160, 90, seed=4)
    sc = scene.PlaneScene(spec)
    prev, cur = sc.frame(9), sc.frame(10)
    H, W = 90, 160
    ys, xs = torch.meshgrid(torch.arange(H), torch.arange(W), indexing="ij")
    px = (xs + 0.5 + cur["motion"][..., 0]).floor().long()
    py = (ys + 0.5 + cur["motion"][..., 1]).floor().long()
    inside = (px >= 0) & (px < W) & (py >= 0) & (py < H)
    same = prev["plane"][py.clamp(0, H - 1), px.clamp(0, W - 1)] == cur["plane"]
    assert float(same[inside].float().mean()) > 0.97


def test_plane_appears_at_frame_30():
    spec = scene.pan_with_disocclusion(160, 90, seed=5)
    sc = scene.PlaneScene(spec)
    rect_id = len(sc.planes)
    assert not bool((sc.frame(29)["plane"] == rect_id).any())
    assert bool((sc.frame(30)["plane"] == rect_id).any())


def test_oct16_torch_encoder_matches_oracle():
    import oracle

    rng = np.random.default_rng(0)
    n = rng.normal(size=(4000, 3)).astype(np.float32)
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    a = scene.oct16_encode(torch.from_numpy(n)).numpy().astype(np.int32)
    b = oracle.oct16_encode(n).astype(np.int32)
    assert np.abs(a - b).max() <= 1


def test_stream_specs_are_seeded():
    a = scene.stream_specs(8, [(160, 90), (320, 180)], seed=3)
    b = scene.stream_specs(8, [(160, 90), (320, 180)], seed=3)
    assert [(s.width, s.height, s.seed) for s in a] == [(s.width, s.height, s.seed) for s in b]
    assert all(math.isfinite(s.yaw_deg) for s in a)
