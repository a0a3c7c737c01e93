"""GPU parity of the bloom + post-process chain (tg_post_process) against the reference shaders' outputs and the
oracle.

The kernels evaluate every operation as an IEEE-rounded single-precision operation in the shaders' order; only
the sRGB curve's power (exp2f(log2f(c) / 2.4)) is CUDA's.  Tolerances (written here): bloom mips (rgba16f) identical to the reference;
display bytes within 1 unit, at least 99.9% identical; the float32 output within 1e-5 of the oracle's.
"""
import glob
import os
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
import tron_grid_gb300 as tg  # noqa: E402
from tron_grid_gb300 import _lib as L  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = sorted(glob.glob(os.path.join(ROOT, "tests", "golden", "post_*.npz")))


def check_bytes(got_rgba_u8, want_u8, what=""):
    d = np.abs(got_rgba_u8.astype(np.int32) - want_u8.astype(np.int32))
    assert d.max() <= 1, f"{what}: {d.max()} units apart"
    same = float((d == 0).mean())
    assert same >= 0.999, f"{what}: only {same:.5f} of bytes identical"


def run(hdr_np, dev, order="bgra", hdr_dtype=torch.float16, out_dtype=torch.uint8, pp=None):
    h, w = hdr_np.shape[:2]
    pp = pp or tg.PostProcessor(w, h)
    hdr = torch.from_numpy(hdr_np).to(dev, hdr_dtype)
    out = torch.zeros((h, w, 4), dtype=out_dtype, device=dev)
    pp.process(hdr, out, order=order)
    torch.cuda.synchronize()
    return out.cpu().numpy(), pp


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p) for p in GOLDEN])
def test_matches_reference_outputs(cuda_dev, path):
    z = np.load(path)
    bgra, pp = run(z["hdr"].astype(np.float32), cuda_dev)
    rgba = bgra[..., [2, 1, 0, 3]]
    check_bytes(rgba, z["out_u8"], os.path.basename(path))
    mips = pp.bloom_mips()
    assert len(mips) == len([k for k in z.files if k.startswith("mip")])
    for i, m in enumerate(mips):
        np.testing.assert_array_equal(m, z[f"mip{i}"].astype(np.float32), err_msg=f"mip {i}")
    pp.close()


@pytest.mark.parametrize("wh", [(1, 1), (2, 3), (97, 61), (640, 360)])
def test_against_oracle_rgba_and_float(cuda_dev, wh):
    w, h = wh
    rng = np.random.default_rng(w * 7 + h)
    hdr = np.concatenate([rng.uniform(0, 2, (h, w, 3)) * rng.choice([1.0, 1.0, 9.0], size=(h, w, 1)),
                          np.ones((h, w, 1))], -1).astype(np.float16).astype(np.float32)
    want, _ = oracle.post_frame(hdr)
    got, pp = run(hdr, cuda_dev, order="rgba")
    check_bytes(got, np.rint(want * 255).astype(np.uint8), f"{wh} rgba8")
    want_f, _ = oracle.post_frame(hdr, unorm8=False)
    got_f, _ = run(hdr, cuda_dev, out_dtype=torch.float32, pp=pp)
    assert np.abs(got_f - want_f).max() <= 1e-5
    got32, _ = run(hdr, cuda_dev, order="rgba", hdr_dtype=torch.float32, pp=pp)  # float32 HDR input, same values
    np.testing.assert_array_equal(got32, got)
    pp.close()


def test_resize_and_padded_rows(cuda_dev):
    pp = tg.PostProcessor(64, 36)
    rng = np.random.default_rng(3)
    hdr = np.concatenate([rng.uniform(0, 5, (50, 90, 3)), np.ones((50, 90, 1))], -1).astype(np.float16)
    pp.resize(90, 50)
    assert pp.info()["mip_count"] == len(oracle.bloom_mip_sizes(90, 50))
    big = torch.zeros((50, 100, 4), dtype=torch.float16, device=cuda_dev)
    big[:, :90] = torch.from_numpy(hdr).to(cuda_dev)
    outbig = torch.full((50, 96, 4), 7, dtype=torch.uint8, device=cuda_dev)
    pp.process(big[:, :90], outbig[:, :90])
    torch.cuda.synchronize()
    want, _ = oracle.post_frame(hdr.astype(np.float32))
    check_bytes(outbig[:, :90].cpu().numpy()[..., [2, 1, 0, 3]], np.rint(want * 255).astype(np.uint8), "padded")
    assert (outbig[:, 90:] == 7).all()
    pp.close()


def test_invalid_arguments(cuda_dev):
    pp = tg.PostProcessor(16, 8)
    hdr = torch.zeros((8, 16, 4), dtype=torch.float16, device=cuda_dev)
    with pytest.raises(TypeError):
        pp.process(hdr.to(torch.int16))
    import ctypes as C

    lib = L.load()
    hi = L.Image(hdr.data_ptr(), 0, L.FMT_RGBA16F, 0)
    bad = L.Image(hdr.data_ptr() + 2, 0, L.FMT_BGRA8, 0)  # misaligned output
    assert lib.tg_post_process(pp.handle, C.byref(hi), C.byref(bad), None) == L.ERR_INVALID
    odd = L.Image(hdr.data_ptr(), 0, L.FMT_RG16F, 0)
    assert lib.tg_post_process(pp.handle, C.byref(odd), C.byref(hi), None) == L.ERR_INVALID
    p = L.PostParams(1.0, 0.095, 0, 0)
    h = C.c_void_p()
    assert lib.tg_post_create(16, 8, C.byref(p), 0, C.byref(h)) == L.ERR_INVALID
    pp.close()
