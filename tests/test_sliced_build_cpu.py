"""Host-only checks of the sliced builder (no GPU): tests/sliced_build_check.cpp
is compiled with g++ against vnec_gb300/csrc/sliced_build.cpp and run on a
27-point stencil, a constant-offset band and random rows.  It checks that the
builder flags a delta task as a shared-pattern task exactly when every row has
the task's length and the first row's column gaps, and that the stored pattern
and the host view's counts match."""
from __future__ import annotations

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_shared_pattern_tasks(tmp_path):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not found")
    from vnec_gb300.build import cuda_home

    exe = tmp_path / "sliced_build_check"
    csrc = os.path.join(ROOT, "vnec_gb300", "csrc")
    cmd = [gxx, "-O1", "-std=c++17", "-fopenmp", "-I", csrc, "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(cuda_home(), "include"), os.path.join(ROOT, "tests", "sliced_build_check.cpp"),
           os.path.join(csrc, "sliced_build.cpp"), "-o", str(exe)]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = r.stdout.strip().splitlines()
    assert len(lines) == 6
    assert all("mismatches 0, missed 0" in line for line in lines), r.stdout
