"""The bloom + post-process oracle (a restatement of src/bloom_downsample.slang and src/postprocess.slang,
host order src/main.cpp:306-430), pinned against the reference shaders themselves: their outputs recorded in
tests/golden/post_*.npz and, where the reference checkout is present, the shaders compiled as C++; plus
closed-form known answers."""
import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "post_*.npz")))


def test_golden_fixtures_present():
    assert len(GOLDEN) >= 5


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_restatement_matches_reference_outputs(path):
    """Bit-exact against the reference shaders' display bytes and every bloom mip."""
    z = np.load(path)
    out, mips = oracle.post_frame(z["hdr"].astype(np.float32))
    np.testing.assert_array_equal(np.rint(out * 255.0).astype(np.uint8), z["out_u8"])
    assert len(mips) == len([k for k in z.files if k.startswith("mip")])
    for i, m in enumerate(mips):
        np.testing.assert_array_equal(m, z[f"mip{i}"].astype(np.float32), err_msg=f"mip {i}")


@pytest.mark.skipif(not oracle.post_reference_available(), reason="reference checkout not present")
@pytest.mark.parametrize("wh", [(2, 1), (33, 17), (256, 144)])
def test_restatement_matches_compiled_reference(wh):
    w, h = wh
    rng = np.random.default_rng(w + h)
    hdr = np.concatenate([rng.uniform(0, 3, (h, w, 3)) * rng.choice([1, 6], size=(h, w, 1)), np.ones((h, w, 1))], -1)
    hdr = hdr.astype(np.float16).astype(np.float32)
    a, ma = oracle.post_frame(hdr)
    b, mb = oracle.post_frame_reference(hdr)
    np.testing.assert_array_equal(a, b)
    for x, y in zip(ma, mb):
        np.testing.assert_array_equal(x, y)


@pytest.mark.parametrize("wh,n", [((1, 1), 1), ((2, 2), 1), ((4, 2), 2), ((64, 36), 6), ((3840, 2160), 6),
                                  ((1280, 720), 6), ((7, 1), 2)])
def test_mip_chain_sizes(wh, n):
    sizes = oracle.bloom_mip_sizes(*wh)
    assert len(sizes) == n
    assert sizes[0] == (max(wh[0] // 2, 1), max(wh[1] // 2, 1))


def test_black_frame_is_black_and_dim_frame_does_not_bloom():
    h, w = 20, 30
    black = np.zeros((h, w, 4), np.float32)
    black[..., 3] = 1
    out, mips = oracle.post_frame(black)
    assert (np.rint(out[..., :3] * 255) == 0).all() and (out[..., 3] == 1).all()
    dim = black.copy()
    dim[..., :3] = 0.3  # luminance 0.3 < threshold 1.0
    _, mips = oracle.post_frame(dim)
    assert all((m[..., :3] == 0).all() for m in mips)


def test_float_and_double_agree():
    rng = np.random.default_rng(7)
    h, w = 45, 80
    hdr = np.concatenate([rng.uniform(0, 4, (h, w, 3)), np.ones((h, w, 1))], -1).astype(np.float32)
    a, _ = oracle.post_frame(hdr, fp16_store=False, unorm8=False)
    b, _ = oracle.post_frame(hdr, fp16_store=False, unorm8=False, dtype=np.float64)
    assert np.abs(a - b).max() <= 1e-5


def test_product_defaults_are_the_reference_constants():
    from tron_grid_gb300 import post

    p = post.default_params()
    assert (p.bloom_threshold, p.max_mips) == (1.0, 6)
    assert p.bloom_strength == np.float32(0.095)
