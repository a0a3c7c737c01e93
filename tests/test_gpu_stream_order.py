"""Stream order of the chain kernels, which are launched with programmatic
dependent launch: every kernel waits for the previous kernel of its stream to
complete before it reads anything, so a producer kernel that writes the inputs
just before the call and a consumer kernel that reads the output just after it
need no synchronisation.  A sequence run that way on one side stream must
equal, bit for bit, the same sequence run with a device synchronisation around
every call.
"""
import pytest
import torch

import tron_grid_gb300 as tg
from tron_grid_gb300 import scene

pytestmark = pytest.mark.gpu

KEYS = ("radiance", "depth", "normal", "motion")
CASES = [(tg.MODE_FULL, tg.STORAGE_FP32), (tg.MODE_FULL, tg.STORAGE_FP16), (tg.MODE_REF_EXACT, tg.STORAGE_FP16),
         (tg.MODE_REF_EXACT, tg.STORAGE_FP32)]


def _frames(dev, W, H, n, mode, storage):
    sc = scene.PlaneScene(scene.pan_with_disocclusion(W, H, seed=21), device=dev)
    out = []
    for t in range(n):
        fr = sc.frame(t)
        if mode == tg.MODE_REF_EXACT:
            rad = fr["radiance"].half() if storage == tg.STORAGE_FP16 else fr["radiance"]
            out.append({"radiance": rad, "depth": None, "normal": None, "motion": None})
        elif storage == tg.STORAGE_FP16:
            out.append({"radiance": fr["radiance"].half(), "depth": fr["depth"],
                        "normal": scene.oct16_encode(fr["normal"]), "motion": fr["motion"]})
        else:
            out.append({k: fr[k] for k in KEYS})
    return out


@pytest.mark.parametrize("mode,storage", CASES)
def test_producer_chain_consumer_on_one_stream(cuda_dev, mode, storage):
    W, H, n = 640, 360, 6
    frames = _frames(cuda_dev, W, H, n, mode, storage)
    out_dt = torch.float16 if storage == tg.STORAGE_FP16 else torch.float32
    torch.cuda.synchronize()

    den = tg.Denoiser(W, H, mode=mode, storage=storage)
    want = []
    for fr in frames:
        out = torch.empty((H, W, 4), dtype=out_dt, device=cuda_dev)
        torch.cuda.synchronize()
        den.denoise(fr["radiance"], fr["depth"], fr["normal"], fr["motion"], out=out)
        den.synchronize()
        torch.cuda.synchronize()
        want.append(out.clone())
    den.close()

    den = tg.Denoiser(W, H, mode=mode, storage=storage)
    side = torch.cuda.Stream(cuda_dev)
    bufs = {k: (torch.empty_like(v) if v is not None else None) for k, v in frames[0].items()}
    out = torch.empty((H, W, 4), dtype=out_dt, device=cuda_dev)
    got = []
    with torch.cuda.stream(side):
        for fr in frames:
            for k, v in fr.items():
                if v is not None:
                    bufs[k].copy_(v)  # producer kernel, just before the chain on the same stream
            den.denoise(bufs["radiance"], bufs["depth"], bufs["normal"], bufs["motion"], out=out, stream=side)
            got.append(out.clone())  # consumer kernel, just after it
    side.synchronize()
    assert den.info()["device_errors"] == 0
    den.close()
    for t, (a, b) in enumerate(zip(want, got)):
        assert torch.equal(a, b), f"frame {t} differs"
