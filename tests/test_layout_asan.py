"""Host-side layout builders under AddressSanitizer / UndefinedBehaviorSanitizer.

compute-sanitizer is not available for the GPU runs, so the memory-safety
check of this project's own host code runs here: `tests/layout_check.cpp`
decodes the sliced and batched layouts exactly as the kernels read them and
compares the decoded product with the CSR product (exact integer arithmetic)
for random matrices and builder parameters, compiled with -fsanitize=address,
undefined together with the builder sources.
"""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

from conftest import ROOT

CSRC = os.path.join(ROOT, "vnec_gb300", "csrc")


def _cuda_include() -> str:
    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    return os.path.join(home, "include")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_layout_builders_under_asan(tmp_path):
    exe = tmp_path / "layout_check"
    cmd = ["g++", "-std=c++17", "-O1", "-g", "-fopenmp", "-fsanitize=address,undefined", "-fno-omit-frame-pointer",
           "-fno-sanitize-recover=undefined", "-I", os.path.join(ROOT, "include"), "-I", CSRC, "-I", _cuda_include(),
           os.path.join(ROOT, "tests", "layout_check.cpp"), os.path.join(CSRC, "sliced_build.cpp"),
           os.path.join(CSRC, "batch_build.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    env = dict(os.environ, ASAN_OPTIONS="detect_leaks=1:abort_on_error=1", OMP_NUM_THREADS="4")
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    assert "0 failures" in r.stdout
