"""A C program written against the reference's API (tests/c_harness.c),
compiled with gcc and linked to libvnec_gb300.so, follows the reference
harness's flow — IRD_VNEC dispatch (VNEC-L at >= 3e6 rows), Build_VNEC_*,
SpMV_VNEC_* on host vectors, handle release — then SpB_mxv with a NULL handle,
pipelined host calls and the known-answer pattern, each checked against its own
serial loop."""
from __future__ import annotations

import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(built, tmp_path_factory):
    lib = os.path.join(ROOT, "vnec_gb300", "_lib")
    exe = str(tmp_path_factory.mktemp("c") / "c_harness")
    subprocess.run(["gcc", "-std=c99", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c_harness.c"), "-L", lib, "-lvnec_gb300", "-lm",
                    f"-Wl,-rpath,{lib}", "-o", exe], check=True, capture_output=True)
    return exe


@pytest.mark.parametrize("n,k,seed", [(100_000, 16, 1), (65_536, 4, 3), (3_000_000, 4, 2)],
                         ids=["sliced_or_dense", "small", "merge_path"])
def test_c_program_drives_the_library(harness, n, k, seed):
    r = subprocess.run([harness, str(n), str(k), str(seed)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout
    assert r.stdout.count("ok  ") == 7  # dispatch, SpB_mxv, 4 pipelined calls, known answer
