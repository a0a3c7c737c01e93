"""Generates tests/golden/ref_exact_*.npz from the reference shader itself.

The reference shader `src/svgf_denoise.slang` is compiled as C++ by
oracle/build.py (three Slang-only tokens removed, everything else unchanged)
and run here on seeded inputs; its outputs are the golden vectors that pin the
oracle's restatement on machines without the reference checkout.

Usage: python tests/golden/make_golden.py   (needs the reference checkout)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

CASES = [(33, 17, 5, 0), (8, 8, 3, 1), (1, 1, 4, 2), (2, 3, 4, 3), (64, 36, 4, 4)]


def inputs(w, h, frames, seed):
    rng = np.random.default_rng(seed)
    raw = []
    for _ in range(frames):
        base = rng.uniform(0.05, 0.9, size=(h, w, 3)) * rng.choice([1.0, 1.0, 1.0, 12.0], size=(h, w, 1))
        noisy = base * rng.exponential(1.0, size=(h, w, 3))
        img = np.concatenate([noisy, np.ones((h, w, 1))], -1)
        raw.append(img.astype(np.float16).astype(np.float32))
    return np.stack(raw)


def main():
    if not oracle.reference_available():
        print("reference shader translation unavailable; nothing generated")
        return 1
    for (w, h, frames, seed) in CASES:
        raw = inputs(w, h, frames, seed)
        rec = {"raw": raw}
        for f16 in (True, False):
            mom = np.zeros((h, w, 2), np.float32)
            outs, moms = [], []
            for t in range(frames):
                o, mom = oracle.ref_frame_reference(raw[t], mom, fp16_store=f16)
                outs.append(o)
                moms.append(mom)
            tag = "f16" if f16 else "f32"
            rec[f"out_{tag}"] = np.stack(outs)
            rec[f"mom_{tag}"] = np.stack(moms)
        path = os.path.join(HERE, f"ref_exact_{w}x{h}_s{seed}.npz")
        np.savez_compressed(path, **rec)
        print(path, os.path.getsize(path))
    return 0


if __name__ == "__main__":
    sys.exit(main())
