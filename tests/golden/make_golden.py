"""Generates tests/golden/ref_exact_*.npz, tests/golden/fog_*.npz and
tests/golden/post_*.npz from the reference shaders themselves.

The reference shaders `src/svgf_denoise.slang`, `src/volumetric_filter.slang`,
`src/bloom_downsample.slang` and `src/postprocess.slang` are compiled as C++ by
oracle/build.py (the Slang-only tokens removed, floating literals of the
later three suffixed as float, everything else unchanged) and run here on
seeded inputs; their outputs are the golden vectors that pin the oracle's
restatements on machines without the reference checkout.

Usage: python tests/golden/make_golden.py   (needs the reference checkout)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402

CASES = [(33, 17, 5, 0), (8, 8, 3, 1), (1, 1, 4, 2), (2, 3, 4, 3), (64, 36, 4, 4)]

# froxel-filter sequences: (w, h, d, frames, seed, yaw deg/frame, translation m/frame); frame 0 has no history.
# The second case's camera turns 90 deg per frame (most froxels fall outside the previous grid or behind the
# previous camera); the third moves 150 m per frame along its view axis (previous depth beyond far).
FOG_CASES = [(24, 14, 8, 4, 0, 3.0, (0.2, 0.0, -0.5)), (9, 5, 3, 3, 1, 90.0, (0.0, 0.0, 0.0)),
             (16, 9, 6, 3, 2, 0.0, (0.0, 0.0, -150.0)), (1, 1, 1, 2, 3, 1.0, (0.0, 0.0, -0.1))]


def fog_sequence(w, h, d, frames, seed, yaw, trans):
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "tron-grid_gb300"))
    import fog_scene  # noqa: E402

    sc = fog_scene.FogScene(fog_scene.FogSpec(width=w, height=h, depth=d, yaw_deg=yaw, translation=trans,
                                              seed=seed, frames=frames))
    rng = np.random.default_rng(100 + seed)
    blocks, raws = [], []
    for t in range(frames):
        blocks.append(np.frombuffer(oracle.fog_param_block(**sc.param_args(t)), np.uint8))
        raw = rng.uniform(0.0, 2.0, size=(d, h, w, 4)) * rng.exponential(1.0, size=(d, h, w, 1))
        raws.append(raw.astype(np.float16).astype(np.float32))
    return np.stack(blocks), np.stack(raws)


# bloom + post-process frames: (w, h, seed); HDR with sparse bright pixels above the bloom threshold
POST_CASES = [(1, 1, 0), (3, 5, 1), (64, 36, 2), (97, 61, 3), (160, 90, 4)]


def post_hdr(w, h, seed):
    rng = np.random.default_rng(200 + seed)
    base = rng.uniform(0.0, 1.2, size=(h, w, 3)) * rng.choice([1.0, 1.0, 1.0, 10.0], size=(h, w, 1))
    return np.concatenate([base, np.ones((h, w, 1))], -1).astype(np.float16)


def make_post():
    for (w, h, seed) in POST_CASES:
        hdr = post_hdr(w, h, seed)
        out, mips = oracle.post_frame_reference(hdr.astype(np.float32))
        rec = {"hdr": hdr, "out_u8": np.rint(out * 255.0).astype(np.uint8)}
        for i, m in enumerate(mips):
            rec[f"mip{i}"] = m.astype(np.float16)
        path = os.path.join(HERE, f"post_{w}x{h}_s{seed}.npz")
        np.savez_compressed(path, **rec)
        print(path, os.path.getsize(path))


def make_fog():
    for (w, h, d, frames, seed, yaw, trans) in FOG_CASES:
        blocks, raw = fog_sequence(w, h, d, frames, seed, yaw, trans)
        rec = {"params": blocks, "raw": raw}
        for f16 in (True, False):
            hist = np.zeros((d, h, w, 4), np.float32)
            outs = []
            for t in range(frames):
                hist = oracle.fog_filter_reference(blocks[t].tobytes(), raw[t], hist, fp16_store=f16)
                outs.append(hist)
            rec[f"out_{'f16' if f16 else 'f32'}"] = np.stack(outs)
        path = os.path.join(HERE, f"fog_{w}x{h}x{d}_s{seed}.npz")
        np.savez_compressed(path, **rec)
        print(path, os.path.getsize(path))


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
    if not (oracle.reference_available() and oracle.fog_reference_available() and oracle.post_reference_available()):
        print("reference shader translation unavailable; nothing generated")
        return 1
    make_post()
    make_fog()
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
