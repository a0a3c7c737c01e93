"""GPU eye-frame readback (tg_eye_*): every byte and depth equal to the numpy packing of the same images, the
ring's two-behind / triple-buffer contract, and a caller-provided host region.  Byte work: the bar is bit-exact."""
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

SIZES = [(8, 8), (32, 32), (7, 5), (64, 64), (1, 1), (256, 256), (13, 3)]


def frames(dev, seed, dtype, sizes=SIZES):
    g = torch.Generator(device="cpu").manual_seed(seed)
    cols, deps = [], []
    for (w, h) in sizes:
        if dtype == torch.uint8:
            c = torch.randint(0, 256, (h, w, 4), generator=g, dtype=torch.uint8)
        else:
            c = (torch.rand((h, w, 4), generator=g) * 1.4 - 0.2).to(dtype)  # includes values outside [0, 1]
        cols.append(c.to(dev))
        deps.append(torch.rand((h, w), generator=g).to(dev))
    return cols, deps


@pytest.mark.parametrize("dtype,order", [(torch.uint8, "bgra"), (torch.uint8, "rgba"), (torch.float16, "bgra"),
                                         (torch.float32, "bgra")])
def test_pack_matches_numpy(cuda_dev, dtype, order):
    er = tg.EyeReadback(SIZES, fovs=[1.0 + 0.1 * i for i in range(len(SIZES))])
    cols, deps = frames(cuda_dev, 1, dtype)
    er.submit(0, cols, deps, order=order)
    got = er.acquire(0)
    for i, ((rgb, dep, fov), c, d) in enumerate(zip(got, cols, deps)):
        want_rgb, want_dep = oracle.eye_pack(c.cpu().numpy(), d.cpu().numpy(), order=order)
        np.testing.assert_array_equal(rgb, want_rgb, err_msg=f"eye {i}")
        np.testing.assert_array_equal(dep, want_dep, err_msg=f"eye {i}")
        assert fov == pytest.approx(1.0 + 0.1 * i)
    er.close()


def test_ring_two_behind(cuda_dev):
    """Frame t's views stay valid until t + ring is submitted; older frames report TG_ERR_STATE."""
    er = tg.EyeReadback(SIZES[:3], ring=3)
    sent = {}
    for t in range(6):
        cols, deps = frames(cuda_dev, 10 + t, torch.uint8, SIZES[:3])
        er.submit(t, cols, deps)
        sent[t] = (cols, deps)
        if t >= 2:
            got = er.acquire(t - 2)  # the reference's reader runs two frames behind
            want = oracle.eye_pack(sent[t - 2][0][0].cpu().numpy(), sent[t - 2][1][0].cpu().numpy())
            np.testing.assert_array_equal(got[0][0], want[0])
    with pytest.raises(L.TgError) as e:
        er.acquire(2)  # slot 2 % 3 now holds frame 5
    assert e.value.status == L.ERR_STATE
    with pytest.raises(L.TgError):
        er.acquire(6)  # never submitted
    with pytest.raises(L.TgError):
        er.submit(9, *frames(cuda_dev, 99, torch.uint8, SIZES[:3]))  # out of order
    er.close()


def test_caller_host_buffer(cuda_dev):
    sizes = [(16, 16), (5, 9)]
    import ctypes as C

    ws = (C.c_uint32 * 2)(*[s[0] for s in sizes])
    hs = (C.c_uint32 * 2)(*[s[1] for s in sizes])
    n = L.load().tg_eye_host_bytes(2, ws, hs, 3)
    raw = np.zeros(n + 4096, np.uint8)
    off = (-raw.ctypes.data) % 4096
    buf = raw[off:off + n]
    er = tg.EyeReadback(sizes, host_buffer=buf)
    g = torch.Generator(device="cpu").manual_seed(3)
    cols = [torch.randint(0, 256, (h, w, 4), generator=g, dtype=torch.uint8).to(cuda_dev) for (w, h) in sizes]
    deps = [torch.rand((h, w), generator=g).to(cuda_dev) for (w, h) in sizes]
    er.submit(0, cols, deps)
    got = er.acquire(0)
    rgb0 = got[0][0]
    assert rgb0.ctypes.data == buf.ctypes.data  # the views point into the caller's region
    np.testing.assert_array_equal(rgb0, oracle.eye_pack(cols[0].cpu().numpy(), deps[0].cpu().numpy())[0])
    er.close()


def test_invalid_arguments(cuda_dev):
    import ctypes as C

    lib = L.load()
    d = L.EyeDesc(0, None, None, None, 3, 0, None, 0)
    h = C.c_void_p()
    assert lib.tg_eye_create(C.byref(d), C.byref(h)) == L.ERR_INVALID
    er = tg.EyeReadback([(4, 4)])
    c = torch.zeros((4, 4, 4), dtype=torch.uint8, device=cuda_dev)
    dep = torch.zeros((4, 4), dtype=torch.float32, device=cuda_dev)
    bad = (L.Image * 1)(L.Image(c.data_ptr(), 0, L.FMT_R32F, 0))
    good_d = (L.Image * 1)(L.Image(dep.data_ptr(), 0, L.FMT_R32F, 0))
    assert lib.tg_eye_submit(er.handle, 0, bad, good_d, None) == L.ERR_INVALID
    er.close()
