"""The drop-in proof: the reference's OWN core library builds the objects.

tests/core_harness.c is compiled against the reference's headers and linked
with the reference's core sources (src/core/src, compiled from the
reference's own files: SpB_Matrix_new, SpB_Matrix_build_FP64's COO -> CSR,
SpB_Vector_new / setElement / extractElement, SpB_Matrix_free ...) and with
libvnec_gb300.so in place of the reference's operation module.  It runs the
reference harness's flow (src/operation/test/test_spmv_vnec.cpp:140-275):
IRD_VNEC dispatch below 3,000,000 rows, VNEC-L above, the handles released
the way the harness releases them, the harness's 1e-8 per-row check and a
bit-exact known answer.

The reference's sources reach the GPU host as the oracle's staged archive
(oracle/Makefile, ``ref-stage``; unpacked by ``make ref``); without it the
test is skipped.
"""
from __future__ import annotations

import glob
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def harness(built, tmp_path_factory):
    from oracle import oracle as O

    tree = O.reference_tree()
    if tree is None:
        pytest.skip("the reference's sources are not staged on this host (oracle/_ref/src-tree)")
    lib = os.path.join(ROOT, "vnec_gb300", "_lib")
    out = tmp_path_factory.mktemp("core")
    inc = ["-I", os.path.join(tree, "include"), "-I", os.path.join(tree, "src", "core", "include")]
    objs = []
    # The reference's core library, compiled from its own sources (no SIMD
    # code; its CMake builds it with OpenMP).
    for src in sorted(glob.glob(os.path.join(tree, "src", "core", "src", "*.c"))):
        obj = str(out / (os.path.basename(src) + ".o"))
        subprocess.run(["gcc", "-std=gnu11", "-O2", "-fPIC", "-fopenmp", "-DWITH_OMP", "-w", *inc, "-c", src,
                        "-o", obj], check=True, capture_output=True)
        objs.append(obj)
    exe = str(out / "core_harness")
    r = subprocess.run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror", *inc, "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "core_harness.c"), *objs, "-fopenmp", "-L", lib,
                        "-lvnec_gb300", "-lm", f"-Wl,-rpath,{lib}", "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


@pytest.mark.parametrize("n,deg,seed", [(200_000, 8, 1), (65_536, 16, 4), (3_100_000, 4, 2)],
                         ids=["ird_dispatch", "uniform_k16", "merge_path"])
def test_reference_core_objects_through_the_library(harness, n, deg, seed):
    r = subprocess.run([harness, str(n), str(deg), str(seed)], capture_output=True, text=True, timeout=900)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "FAIL" not in r.stdout
    assert r.stdout.count("ok  ") == 7
    assert ("L: Build_VNEC_L" in r.stdout) == (n >= 3_000_000)
