"""The no-alloc entry point's per-context address cache, tested on the host.

The device address of the entry point's scratch array belongs to a CUDA
context.  Calling the entry point in a second context with the first
context's address would make its kernels write through an address that is not
mapped there, so the check that the lookup repeats when the context changes is
made here without a GPU: tests/native/noalloc_ctx_cache_test.cpp drives the
cache of tron-grid_gb300/csrc/noalloc_ctx_cache.h with a fake context source.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_context_change_repeats_the_lookup(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "noalloc_ctx_cache_test"
    src = os.path.join(ROOT, "tests", "native", "noalloc_ctx_cache_test.cpp")
    inc = os.path.join(ROOT, "tron-grid_gb300", "csrc")
    subprocess.run([cxx, "-std=c++17", "-O1", "-Wall", "-Werror", "-I", inc, src, "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
