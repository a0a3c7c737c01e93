"""Shared metrics for the parity tests."""
import numpy as np

Y709 = np.array([0.2126, 0.7152, 0.0722])

# Per-pixel luminance tolerance of the FP32 paths: |a - b| <= REL_TOL * max(|b|, LUM_FLOOR).
REL_TOL = 1e-4
LUM_FLOOR = 1e-3


def luminance(img):
    img = np.asarray(img, np.float64)
    return img[..., :3] @ Y709


def rel_err(a, b, floor=LUM_FLOOR):
    """Per-pixel relative luminance error of a against b."""
    la, lb = luminance(a), luminance(b)
    return np.abs(la - lb) / np.maximum(np.abs(lb), floor)


def rel_l2(a, b):
    la, lb = luminance(a), luminance(b)
    return float(np.sqrt(np.sum((la - lb) ** 2) / max(np.sum(lb ** 2), 1e-300)))


def psnr(a, b):
    """PSNR (dB) of a against b on luminance, with the peak of b."""
    la, lb = luminance(a), luminance(b)
    mse = float(np.mean((la - lb) ** 2))
    peak = float(np.max(np.abs(lb)))
    return float("inf") if mse == 0 else 10.0 * np.log10(peak * peak / mse)


def report(a, b):
    r = rel_err(a, b)
    return dict(max_abs=float(np.max(np.abs(luminance(a) - luminance(b)))), max_rel=float(np.max(r)),
                rel_l2=rel_l2(a, b), psnr=psnr(a, b))
