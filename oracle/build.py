"""Build recipe for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Produces
  oracle/_build/liborc.so    - the C++ restatements (oracle/svgf_oracle.cpp,
                               oracle/fog_oracle.cpp);
  oracle/_ref/libsvgf_ref.so - the reference shader `src/svgf_denoise.slang`
                               compiled as C++ (when its translation exists);
  oracle/_ref/libfog_ref.so  - the reference shader `src/volumetric_filter.slang`
                               compiled as C++ (when its translation exists);
  oracle/_ref/libpost_ref.so - the reference shaders `src/bloom_downsample.slang`
                               and `src/postprocess.slang` compiled as C++.

The translations of the shaders are made here from the reference checkout, with
textual edits that remove Slang-only syntax:
  * the `[shader("compute")]` attribute line,
  * the `[numthreads(8, 8, 1)]` attribute line,
  * the `: SV_DispatchThreadID` parameter semantic,
and, for the froxel filter and the bloom / post-process shaders, an `f` suffix
on every unsuffixed floating literal (Slang floating literals are 32-bit; the
denoiser's arithmetic is unaffected by this and its translation does not need
it).  Everything else compiles unchanged against oracle/slang_prelude.hpp,
oracle/slang_prelude_fog.hpp or oracle/slang_prelude_post.hpp.  The
translations are written to oracle/_ref/ (git-ignored, never committed) so that
a machine without the reference checkout can still compile them.

Usage: python oracle/build.py [--reference-root DIR]
"""
from __future__ import annotations

import argparse
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORC_LIB = os.path.join(BUILD_DIR, "liborc.so")
REF_LIB = os.path.join(REF_DIR, "libsvgf_ref.so")
REF_GEN = os.path.join(REF_DIR, "svgf_denoise_gen.cpp")
FOG_REF_LIB = os.path.join(REF_DIR, "libfog_ref.so")
FOG_REF_GEN = os.path.join(REF_DIR, "volumetric_filter_gen.cpp")
POST_REF_LIB = os.path.join(REF_DIR, "libpost_ref.so")
BLOOM_REF_GEN = os.path.join(REF_DIR, "bloom_downsample_gen.cpp")
PP_REF_GEN = os.path.join(REF_DIR, "postprocess_gen.cpp")


def default_reference_root() -> str:
    """The reference checkout to translate: $TG_REFERENCE_ROOT, else a directory named `reference` beside this
    repository's own directory.  Where neither exists the translations are skipped."""
    env = os.environ.get("TG_REFERENCE_ROOT")
    if env:
        return env
    return os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off"]
# The timed CPU baseline is built for speed, not for bit-agreement with the GPU's discrete decisions: fused
# multiply-adds allowed, no errno from the math library, unrolled loops.  Host code must build the same way on
# x86-64 and aarch64 hosts, so no -march=native: both targets' baselines already have fused multiply-add
# (aarch64) or SSE2 vectors (x86-64), and the restatement is a per-pixel loop over rows that OpenMP spreads over
# every host core.
TIMING_CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=fast", "-fno-math-errno",
                   "-funroll-loops"]
ORC_TIMING_LIB = os.path.join(BUILD_DIR, "liborc_timing.so")


def _newer(target: str, *sources: str) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def _oracle_sources():
    return [os.path.join(HERE, "svgf_oracle.cpp"), os.path.join(HERE, "fog_oracle.cpp"),
            os.path.join(HERE, "post_oracle.cpp")]


def build_oracle(force: bool = False) -> str:
    """The checker build (liborc.so): no contraction, so that its discrete decisions match the GPU's."""
    srcs = _oracle_sources()
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not _newer(ORC_LIB, *srcs, __file__):
        tmp = ORC_LIB + ".tmp"
        subprocess.check_call(["g++", *CXXFLAGS, *srcs, "-o", tmp])
        os.replace(tmp, ORC_LIB)
    return ORC_LIB


def build_oracle_timing(force: bool = False) -> str:
    """The timed CPU baseline's build (liborc_timing.so) of the same sources, with TIMING_CXXFLAGS."""
    srcs = _oracle_sources()
    os.makedirs(BUILD_DIR, exist_ok=True)
    if force or not _newer(ORC_TIMING_LIB, *srcs, __file__):
        tmp = ORC_TIMING_LIB + ".tmp"
        subprocess.check_call(["g++", *TIMING_CXXFLAGS, *srcs, "-o", tmp])
        os.replace(tmp, ORC_TIMING_LIB)
    return ORC_TIMING_LIB


_FLOAT_LITERAL = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eE][+-]?\d+)?|\.\d+(?:[eE][+-]?\d+)?|\d+[eE][+-]?\d+)(?![\w.])")


def _strip_slang(text: str, shader: str, entries: int = 1) -> str:
    out_lines = []
    removed = 0
    for line in text.splitlines():
        s = line.strip()
        if s == '[shader("compute")]' or re.fullmatch(r"\[numthreads\(\s*8\s*,\s*8\s*,\s*1\s*\)\]", s):
            removed += 1
            continue
        out_lines.append(line)
    body = "\n".join(out_lines) + "\n"
    body, nsem = re.subn(r"\s*:\s*SV_DispatchThreadID", "", body)
    if removed != 2 * entries or nsem != entries:
        raise RuntimeError(f"unexpected layout of {shader} (attributes removed={removed}, semantics={nsem})")
    return body


def _write_if_changed(path: str, text: str) -> None:
    os.makedirs(os.path.dirname(path), exist_ok=True)
    if not os.path.exists(path) or open(path, encoding="utf-8").read() != text:
        with open(path, "w", encoding="utf-8") as f:
            f.write(text)


def translate_fog_reference(reference_root: str | None = None) -> str | None:
    """Write oracle/_ref/volumetric_filter_gen.cpp from the reference shader, if present."""
    reference_root = reference_root or default_reference_root()
    shader = os.path.join(reference_root, "src", "volumetric_filter.slang")
    if not os.path.isfile(shader):
        return None
    with open(shader, encoding="utf-8") as f:
        body = _strip_slang(f.read(), shader)
    body = _FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", body)
    _write_if_changed(FOG_REF_GEN, f"// Generated by oracle/build.py from {shader}; not committed.\n" + body)
    return FOG_REF_GEN


def translate_post_reference(reference_root: str | None = None) -> bool:
    """Write oracle/_ref/{bloom_downsample,postprocess}_gen.cpp from the reference shaders, if present."""
    reference_root = reference_root or default_reference_root()
    for name, gen, entries in (("bloom_downsample.slang", BLOOM_REF_GEN, 3), ("postprocess.slang", PP_REF_GEN, 1)):
        shader = os.path.join(reference_root, "src", name)
        if not os.path.isfile(shader):
            return False
        with open(shader, encoding="utf-8") as f:
            body = _strip_slang(f.read(), shader, entries)
        body = _FLOAT_LITERAL.sub(lambda m: m.group(1) + "f", body)
        _write_if_changed(gen, f"// Generated by oracle/build.py from {shader}; not committed.\n" + body)
    return True


def build_post_reference(force: bool = False, reference_root: str | None = None) -> str | None:
    """Compile the translated bloom / post-process shaders; None when no translation exists."""
    translate_post_reference(reference_root)
    if not (os.path.isfile(BLOOM_REF_GEN) and os.path.isfile(PP_REF_GEN)):
        return None
    drv = os.path.join(HERE, "post_ref_driver.cpp")
    pre = os.path.join(HERE, "slang_prelude_post.hpp")
    if force or not _newer(POST_REF_LIB, BLOOM_REF_GEN, PP_REF_GEN, drv, pre):
        tmp = POST_REF_LIB + ".tmp"
        subprocess.check_call(["g++", *CXXFLAGS, "-std=c++20", "-Wno-attributes", "-I", HERE, "-I", REF_DIR, drv, "-o", tmp])
        os.replace(tmp, POST_REF_LIB)
    return POST_REF_LIB


def build_fog_reference(force: bool = False, reference_root: str | None = None) -> str | None:
    """Compile the translated froxel-filter shader; None when no translation exists."""
    translate_fog_reference(reference_root)
    if not os.path.isfile(FOG_REF_GEN):
        return None
    drv = os.path.join(HERE, "fog_ref_driver.cpp")
    pre = os.path.join(HERE, "slang_prelude_fog.hpp")
    if force or not _newer(FOG_REF_LIB, FOG_REF_GEN, drv, pre):
        tmp = FOG_REF_LIB + ".tmp"
        subprocess.check_call(["g++", *CXXFLAGS, "-std=c++20", "-Wno-attributes", "-I", HERE, "-I", REF_DIR, drv, "-o", tmp])
        os.replace(tmp, FOG_REF_LIB)
    return FOG_REF_LIB


def translate_reference(reference_root: str | None = None) -> str | None:
    """Write oracle/_ref/svgf_denoise_gen.cpp from the reference shader, if present."""
    reference_root = reference_root or default_reference_root()
    shader = os.path.join(reference_root, "src", "svgf_denoise.slang")
    if not os.path.isfile(shader):
        return None
    with open(shader, encoding="utf-8") as f:
        text = f.read()
    out_lines = []
    removed = 0
    for line in text.splitlines():
        s = line.strip()
        if s == '[shader("compute")]' or re.fullmatch(r"\[numthreads\(\s*8\s*,\s*8\s*,\s*1\s*\)\]", s):
            removed += 1
            continue
        out_lines.append(line)
    body = "\n".join(out_lines) + "\n"
    body, nsem = re.subn(r"\s*:\s*SV_DispatchThreadID", "", body)
    if removed != 2 or nsem != 1:
        raise RuntimeError(f"unexpected shader layout (attributes removed={removed}, semantics={nsem})")
    os.makedirs(REF_DIR, exist_ok=True)
    header = f"// Generated by oracle/build.py from {shader}; not committed.\n"
    new = header + body
    if not os.path.exists(REF_GEN) or open(REF_GEN, encoding="utf-8").read() != new:
        with open(REF_GEN, "w", encoding="utf-8") as f:
            f.write(new)
    return REF_GEN


def build_reference(force: bool = False, reference_root: str | None = None) -> str | None:
    """Compile the translated reference shader; None when no translation exists."""
    translate_reference(reference_root)
    if not os.path.isfile(REF_GEN):
        return None
    drv = os.path.join(HERE, "ref_driver.cpp")
    pre = os.path.join(HERE, "slang_prelude.hpp")
    if force or not _newer(REF_LIB, REF_GEN, drv, pre):
        tmp = REF_LIB + ".tmp"
        subprocess.check_call(["g++", *CXXFLAGS, "-std=c++20", "-Wno-attributes", "-I", HERE, "-I", REF_DIR, drv, "-o", tmp])
        os.replace(tmp, REF_LIB)
    return REF_LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference-root", default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build_oracle(a.force))
    print(build_oracle_timing(a.force))
    r = build_reference(a.force, a.reference_root)
    print(r if r else "reference shader translation absent: oracle/_ref not built")
    r = build_fog_reference(a.force, a.reference_root)
    print(r if r else "reference froxel-filter translation absent: oracle/_ref/libfog_ref.so not built")
    r = build_post_reference(a.force, a.reference_root)
    print(r if r else "reference bloom / post-process translation absent: oracle/_ref/libpost_ref.so not built")
    return 0


if __name__ == "__main__":
    sys.exit(main())
