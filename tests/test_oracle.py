"""The CPU oracle, pinned before it is trusted.

* REF-EXACT restatement vs the reference shader itself (src/svgf_denoise.slang
  compiled as C++): bit-identical, through committed golden vectors (always)
  and live (when the reference translation is available).
* Closed-form known-answer tests for both modes.
* float32 vs float64 agreement of the FULL oracle.
"""
import glob
import os

import numpy as np
import pytest

import oracle
from tests.helpers import rel_err, rel_l2

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "ref_exact_*.npz")))


def test_golden_vectors_present():
    assert len(GOLDEN) >= 5


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
@pytest.mark.parametrize("f16", [True, False])
def test_restatement_matches_reference_golden(path, f16):
    g = np.load(path)
    raw = g["raw"]
    tag = "f16" if f16 else "f32"
    h, w = raw.shape[1:3]
    mom = np.zeros((h, w, 2), np.float32)
    for t in range(raw.shape[0]):
        out, mom = oracle.ref_frame(raw[t], mom, fp16_store=f16)
        np.testing.assert_array_equal(out, g[f"out_{tag}"][t])
        np.testing.assert_array_equal(mom, g[f"mom_{tag}"][t])


@pytest.mark.skipif(not oracle.reference_available(), reason="reference shader translation not built")
@pytest.mark.parametrize("wh", [(1, 1), (2, 2), (7, 3), (33, 17), (97, 61)])
@pytest.mark.parametrize("f16", [True, False])
def test_restatement_matches_reference_live(wh, f16):
    w, h = wh
    rng = np.random.default_rng(w * 1000 + h)
    mom_a = np.zeros((h, w, 2), np.float32)
    mom_b = mom_a.copy()
    for t in range(6):
        raw = rng.exponential(1.0, (h, w, 4)) * rng.uniform(0.05, 40.0, (h, w, 1))
        raw = raw.astype(np.float16).astype(np.float32)
        a, mom_a = oracle.ref_frame(raw, mom_a, fp16_store=f16)
        b, mom_b = oracle.ref_frame_reference(raw, mom_b, fp16_store=f16)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(mom_a, mom_b)


def test_ref_fp16_moment_overflow_matches_reference():
    """Luminance above ~256 overflows the rg16f second moment to inf, then NaN (as in the reference)."""
    raw = np.full((4, 4, 4), 600.0, np.float32)
    mom = np.zeros((4, 4, 2), np.float32)
    for _ in range(3):
        out, mom = oracle.ref_frame(raw, mom, fp16_store=True)
        assert np.all(np.isfinite(out))
    assert np.all(np.isnan(mom[..., 1]))


# ------------------------------------------------------------ REF-EXACT KATs


def test_ref_constant_image_is_fixed_point():
    raw = np.zeros((9, 13, 4), np.float64)
    raw[...] = [0.3, 0.5, 0.2, 1.0]
    mom = np.zeros((9, 13, 2))
    for _ in range(3):
        out, mom = oracle.ref_frame(raw, mom, fp16_store=False, dtype=np.float64)
        np.testing.assert_allclose(out[..., :3], raw[..., :3], rtol=1e-14)
        assert np.all(out[..., 3] == 1.0)


def _atrous_b3_clamped(img, stride):
    """Independent numpy a-trous B3 blur with clamp-to-edge taps."""
    k = np.array([1, 4, 6, 4, 1], np.float64) / 16
    h, w = img.shape[:2]
    out = np.zeros_like(img)
    for dy in range(-2, 3):
        ys = np.clip(np.arange(h) + dy * stride, 0, h - 1)
        for dx in range(-2, 3):
            xs = np.clip(np.arange(w) + dx * stride, 0, w - 1)
            out += k[dx + 2] * k[dy + 2] * img[ys][:, xs]
    return out


def test_ref_isoluminant_image_is_pure_b3_atrous():
    """Equal luminance everywhere -> every edge weight is 1 -> three B3 a-trous passes (strides 1, 2, 4)."""
    rng = np.random.default_rng(0)
    h, w = 19, 23
    Y = np.array([0.2126, 0.7152, 0.0722], np.float32).astype(np.float64)  # the shader's float constants
    rgb = rng.uniform(0.1, 1.0, (h, w, 3))
    rgb *= (0.5 / (rgb @ Y))[..., None]  # luminance exactly 0.5 up to rounding
    raw = np.concatenate([rgb, np.ones((h, w, 1))], -1)
    out, _ = oracle.ref_frame(raw, np.zeros((h, w, 2)), fp16_store=False, dtype=np.float64)
    exp = rgb
    for s in (1, 2, 4):
        exp = _atrous_b3_clamped(exp, s)
    np.testing.assert_allclose(out[..., :3], exp, rtol=1e-9, atol=1e-12)


def test_ref_moment_sequence_closed_form():
    """1x1 image: mu1_t = sum_k a(1-a)^(t-k) l_k from zero; out = input; alpha of the init image = sqrt(var+eps)."""
    a = 0.2
    lum = [0.5, 2.0, 1.0, 4.0, 0.25, 3.0, 1.5, 0.75]
    mom = np.zeros((1, 1, 2))
    for t, l in enumerate(lum):
        raw = np.array([[[l, l, l, 1.0]]])
        out, mom = oracle.ref_frame(raw, mom, fp16_store=False, dtype=np.float64)
        m1 = sum(a * (1 - a) ** (t - k) * lum[k] for k in range(t + 1))
        m2 = sum(a * (1 - a) ** (t - k) * lum[k] ** 2 for k in range(t + 1))
        np.testing.assert_allclose(mom[0, 0], [m1, m2], rtol=1e-12)
        np.testing.assert_allclose(out[0, 0, :3], [l, l, l], rtol=1e-12)


def test_ref_small_images_clamp():
    """1x1 and 2x2: every tap clamps inside the image; output is a convex combination of the pixels."""
    rng = np.random.default_rng(3)
    for (h, w) in ((1, 1), (2, 2), (1, 5)):
        raw = np.concatenate([rng.uniform(0, 3, (h, w, 3)), np.ones((h, w, 1))], -1)
        out, _ = oracle.ref_frame(raw, np.zeros((h, w, 2)), fp16_store=False, dtype=np.float64)
        for c in range(3):
            assert out[..., c].min() >= raw[..., c].min() - 1e-12
            assert out[..., c].max() <= raw[..., c].max() + 1e-12


# ------------------------------------------------------------------ FULL KATs

P = oracle.full_params()


def _static_inputs(h, w, rgb, depth=5.0, normal=(0.0, 0.0, -1.0)):
    rad = np.zeros((h, w, 4))
    rad[...] = list(rgb) + [1.0]
    dep = np.full((h, w), depth)
    nrm = np.zeros((h, w, 3))
    nrm[...] = normal
    mot = np.zeros((h, w, 2))
    return rad, dep, nrm, mot


def test_full_constant_image_is_fixed_point():
    h, w = 11, 14
    st = oracle.FullState(h, w)
    for t in range(6):
        rad, dep, nrm, mot = _static_inputs(h, w, (0.4, 0.7, 0.1))
        out, var = oracle.full_frame(P, st, rad, dep, nrm, mot)
        np.testing.assert_allclose(out[..., :3], rad[..., :3], rtol=1e-13)
        assert np.all(st.hist[..., 3] == min(t + 1, 32))
        assert np.all(np.abs(var) < 1e-20)


@pytest.mark.parametrize("levels", [1, 2, 3, 4, 5])
def test_full_constant_image_is_fixed_point_at_every_level_count(levels):
    """A constant image stays itself through any number of a-trous levels, with non-default edge-stop widths."""
    h, w = 9, 13
    p = oracle.full_params(levels=levels, sigma_l=2.5, sigma_n=64.0, sigma_z=0.5)
    st = oracle.FullState(h, w)
    for t in range(4):
        rad, dep, nrm, mot = _static_inputs(h, w, (0.9, 0.3, 0.6))
        out, var = oracle.full_frame(p, st, rad, dep, nrm, mot)
        np.testing.assert_allclose(out[..., :3], rad[..., :3], rtol=1e-13)
        assert np.all(out[..., 3] == 1.0) and np.all(np.abs(var) < 1e-20)


@pytest.mark.parametrize("fallback", [1, 3, 4])
def test_full_fallback_window(fallback):
    """Below `fallback_frames` of history the level-0 variance is the 7x7 spatial estimate, from then on the pixel's
    temporal variance exactly (static camera: the history grows by one each frame).  With no a-trous level the
    oracle returns that level-0 variance itself."""
    h, w = 12, 15
    p = oracle.full_params(fallback_frames=fallback, levels=0)
    st = oracle.FullState(h, w)
    rng = np.random.default_rng(fallback)
    for t in range(6):
        rad, dep, nrm, mot = _static_inputs(h, w, (0.5, 0.5, 0.5))
        rad[..., :3] *= rng.exponential(1.0, (h, w, 1))
        _, var = oracle.full_frame(p, st, rad, dep, nrm, mot)
        assert np.all(st.hist[..., 3] == t + 1)
        if t + 1 >= fallback:
            np.testing.assert_array_equal(var, st.mom[..., 1])
        else:
            assert not np.allclose(var, st.mom[..., 1])
            assert np.all(var >= 0.0) and np.all(np.isfinite(var))


def test_full_history_length_caps_and_disocclusion_resets():
    h, w = 6, 7
    p = oracle.full_params(max_history=5)
    st = oracle.FullState(h, w)
    rad, dep, nrm, mot = _static_inputs(h, w, (1.0, 1.0, 1.0))
    for t in range(8):
        oracle.full_frame(p, st, rad, dep, nrm, mot)
    assert np.all(st.hist[..., 3] == 5)
    # motion pointing far outside the image: no history anywhere
    oracle.full_frame(p, st, rad, dep, nrm, np.full((h, w, 2), -100.0))
    assert np.all(st.hist[..., 3] == 1)
    # a depth jump beyond the tolerance (5% + gradient + 0.1 m) also rejects history
    oracle.full_frame(p, st, rad, dep, nrm, mot)
    oracle.full_frame(p, st, rad, dep * 1.5, nrm, mot)
    assert np.all(st.hist[..., 3] == 1)
    # a normal rotation beyond the 0.9 cosine rejects history
    oracle.full_frame(p, st, rad, dep, nrm, mot)
    n2 = np.zeros_like(nrm)
    n2[...] = [0.0, np.sin(0.6), -np.cos(0.6)]
    oracle.full_frame(p, st, rad, dep, n2, mot)
    assert np.all(st.hist[..., 3] == 1)


def test_full_moments_are_ema_of_l_and_l2():
    """Static 1x1 pixel: the mean-centred state equals the EMA of l and l^2 with alpha_t = max(a, 1/t)."""
    lum = [0.5, 2.0, 1.0, 4.0, 0.25, 3.0, 1.5, 0.75, 2.5, 1.0]
    st = oracle.FullState(1, 1)
    m1 = m2 = 0.0
    for t, l in enumerate(lum):
        rad, dep, nrm, mot = _static_inputs(1, 1, (l, l, l))
        oracle.full_frame(P, st, rad, dep, nrm, mot)
        am = max(0.2, 1.0 / (t + 1))
        m1 = (1 - am) * m1 + am * l
        m2 = (1 - am) * m2 + am * l * l
        np.testing.assert_allclose(st.mom[0, 0, 0], m1, rtol=1e-12)
        np.testing.assert_allclose(st.mom[0, 0, 1], m2 - m1 * m1, rtol=1e-9, atol=1e-12)


def test_full_float32_agrees_with_float64():
    from tron_grid_gb300 import scene

    sc = scene.PlaneScene(scene.pan_with_disocclusion(96, 64, seed=5))
    s32 = oracle.FullState(64, 96, np.float32)
    s64 = oracle.FullState(64, 96, np.float64)
    for t in range(6):
        fr = sc.frame(t)
        args = [fr[k].numpy() for k in ("radiance", "depth", "normal", "motion")]
        a, _ = oracle.full_frame(P, s32, *args)
        b, _ = oracle.full_frame(P, s64, *args)
        assert rel_err(a, b).max() <= 1e-4
        assert rel_l2(a, b) <= 1e-5


def test_full_fp16_store_mask_decomposes():
    """The FP16-storage emulation is a mask of independent stores: rounding only the radiance input equals feeding
    binary16-rounded radiance with no emulation, the empty mask equals no emulation, and True rounds every store."""
    from tron_grid_gb300 import scene

    sc = scene.PlaneScene(scene.pan_with_disocclusion(64, 48, seed=7))
    frames = [[sc.frame(t)[k].numpy() for k in ("radiance", "depth", "normal", "motion")] for t in range(4)]
    states = {k: oracle.FullState(48, 64, np.float32) for k in ("in", "pre", "none", "zero", "all", "true")}
    for rad, dep, nrm, mot in frames:
        rad16 = rad.astype(np.float16).astype(np.float32)
        a, _ = oracle.full_frame(P, states["in"], rad, dep, nrm, mot, fp16_store=oracle.Q_INPUT)
        b, _ = oracle.full_frame(P, states["pre"], rad16, dep, nrm, mot, fp16_store=0)
        np.testing.assert_array_equal(a, b)
        c, _ = oracle.full_frame(P, states["none"], rad, dep, nrm, mot, fp16_store=False)
        d, _ = oracle.full_frame(P, states["zero"], rad, dep, nrm, mot, fp16_store=0)
        np.testing.assert_array_equal(c, d)
        e, _ = oracle.full_frame(P, states["all"], rad, dep, nrm, mot, fp16_store=oracle.Q_ALL)
        f, _ = oracle.full_frame(P, states["true"], rad, dep, nrm, mot, fp16_store=True)
        np.testing.assert_array_equal(e, f)
    # the storage form's mask leaves the records and (for an RGBA32F output) the output unrounded
    assert oracle.fp16_storage_mask(False) & (oracle.Q_RECORD | oracle.Q_OUTPUT) == 0
    assert oracle.fp16_storage_mask(True) & oracle.Q_OUTPUT


def test_full_denoises():
    """On a static noisy scene without emitters the output is much closer to the truth than the input."""
    from tron_grid_gb300 import scene

    spec = scene.SceneSpec(128, 72, seed=2, yaw_deg=0.0, extra={"no_emitters": True})
    sc = scene.PlaneScene(spec)
    st = oracle.FullState(72, 128)
    for t in range(8):
        fr = sc.frame(t)
        out, _ = oracle.full_frame(P, st, *(fr[k].numpy() for k in ("radiance", "depth", "normal", "motion")))
    truth = fr["truth"].numpy()
    noisy = fr["radiance"].numpy()
    assert rel_l2(out, truth) < 0.5 * rel_l2(noisy, truth)


def test_oct16_codec_roundtrip():
    rng = np.random.default_rng(0)
    n = rng.normal(size=(5000, 3))
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    d = oracle.oct16_decode(oracle.oct16_encode(n)).astype(np.float64)
    ang = np.arctan2(np.linalg.norm(np.cross(d, n), axis=1), np.sum(d * n, axis=1))
    assert ang.max() < 1e-4
    np.testing.assert_allclose(np.linalg.norm(d, axis=1), 1.0, atol=1e-6)
