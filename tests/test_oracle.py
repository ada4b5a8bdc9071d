"""The CPU oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by the reference library compiled from its own
sources (tests/golden/make_golden.py); the oracle restates that library in C.
Bit-for-bit agreement pins the restatement, so the GPU parity tests can use it
at sizes and on machines where the reference itself cannot run.
"""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, golden_cases, golden_csr, golden_manifest, load_golden

CASES = golden_cases()


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    a = np.ascontiguousarray(a)
    b = np.ascontiguousarray(b)
    return a.shape == b.shape and a.tobytes() == b.tobytes()


def racy_rows(m, nparts: int = 36) -> np.ndarray:
    """Rows receiving carries from two or more partitions.  The reference's
    carry fix-up (spmv_vnec_L_for_mxv.c:159-164, spmv_vnec_D_for_mxv.c:479-484)
    is a parallel `y[row] += carry` without atomics, so for these rows the
    reference's own last bits change from run to run."""
    from oracle import oracle as O

    sx, sy, ex, ey = (np.zeros(nparts, dtype=np.int64) for _ in range(4))
    O.lib().orc_partition(nparts, m.n_rows, m.nnz, m.row_ptr.ctypes.data, sx.ctypes.data, sy.ctypes.data,
                          ex.ctypes.data, ey.ctypes.data)
    rows, counts = np.unique(ex[:-1], return_counts=True)
    return rows[(counts >= 2) & (rows < m.n_rows)]


def carry_equal(y, y_ref, m, x, nparts: int = 36) -> bool:
    """Bit-equal outside racy rows, within 1e-12 * sum|a x| on them."""
    from oracle import oracle as O

    racy = racy_rows(m, nparts)
    keep = np.ones(m.n_rows, dtype=bool)
    keep[racy] = False
    if not bits_equal(y[keep], y_ref[keep]):
        return False
    if racy.size:
        _, cond = O.spmv_neumaier(m, x.astype(np.float64))
        tol = 1e-12 if y.dtype == np.float64 else 1e-5
        return bool(np.all(np.abs(y[racy].astype(np.float64) - y_ref[racy]) <= tol * cond[racy]))
    return True


ARM_DIR = os.path.join(GOLDEN, "arm")
ARM_CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(ARM_DIR, "*.npz")))


def test_arm_manifest_matches_arm_build_constants():
    """The ARM fixtures come from the reference's ARM_NEON build (NUM_THREADS 48,
    nLanes 2/4; src/operation/include/SpB_mxv.h:18-24)."""
    import json

    from oracle import oracle as O

    with open(os.path.join(ARM_DIR, "manifest.json")) as f:
        rb = json.load(f)["reference_build"]
    assert (rb["NUM_THREADS"], rb["nLanes_f64"], rb["nLanes_f32"]) == (
        O.ARM["nparts"], O.ARM["nlanes_f64"], O.ARM["nlanes_f32"])
    assert set(ARM_CASES) == set(CASES)


@pytest.mark.parametrize("case", ARM_CASES)
@pytest.mark.parametrize("tag,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_oracle_arm_parameterisation_reproduces_arm_build(built, case, tag, dtype):
    """The restatement with the ARM build's constants and arithmetic (48
    partitions, 2/4 lanes, unfused vmlaq lane updates, fused scalar loops)
    reproduces the reference's ARM_NEON build bit for bit on the golden inputs
    (rows fed by two or more partitions' carries within 1e-12, as on x86)."""
    from oracle import oracle as O

    g = load_golden(case)
    with np.load(os.path.join(ARM_DIR, f"{case}.npz")) as z:
        a = {k: z[k] for k in z.files}
    m = golden_csr(g)
    x = g["x"]
    nparts = O.ARM["nparts"]
    assert bits_equal(O.spmv_serial(m, x, dtype=dtype, build=O.ARM), a[f"y_serial_{tag}"])
    assert carry_equal(O.spmv_vnec("L", m, x, dtype=dtype, build=O.ARM), a[f"y_L_{tag}"], m, x, nparts)
    if bool(a["vnec_ds_defined"]):
        assert carry_equal(O.spmv_vnec("D", m, x, dtype=dtype, build=O.ARM), a[f"y_D_{tag}"], m, x, nparts)
        assert bits_equal(O.spmv_vnec("S", m, x, dtype=dtype, build=O.ARM), a[f"y_S_{tag}"])
        choice, ratio = O.ird(m, fp64=(tag == "f64"), build=O.ARM)
        assert abs(ratio - float(a[f"ird_{tag}"])) <= 5.01e-7
        assert {0: 1, 1: 2}[choice] == int(a[f"auto_variant_{tag}"])


def test_manifest_matches_reference_build_constants():
    from oracle import oracle as O

    rb = golden_manifest()["reference_build"]
    assert rb["NUM_THREADS"] == O.X86["nparts"]
    assert rb["nLanes_f64"] == O.X86["nlanes_f64"]
    assert rb["nLanes_f32"] == O.X86["nlanes_f32"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("tag,dtype", [("f64", np.float64), ("f32", np.float32)])
def test_oracle_reproduces_reference_bit_for_bit(built, case, tag, dtype):
    from oracle import oracle as O

    g = load_golden(case)
    m = golden_csr(g)
    x = g["x"]
    assert bits_equal(O.spmv_serial(m, x, dtype=dtype), g[f"y_serial_{tag}"])
    assert carry_equal(O.spmv_vnec("L", m, x, dtype=dtype), g[f"y_L_{tag}"], m, x)
    if bool(g["vnec_ds_defined"]):
        assert carry_equal(O.spmv_vnec("D", m, x, dtype=dtype), g[f"y_D_{tag}"], m, x)
        assert bits_equal(O.spmv_vnec("S", m, x, dtype=dtype), g[f"y_S_{tag}"])
        choice, ratio = O.ird(m, fp64=(tag == "f64"))
        # the reference prints the ratio with "%f" (6 decimals): that is all the fixture holds
        assert abs(ratio - float(g[f"ird_{tag}"])) <= 5.01e-7
        assert {0: 1, 1: 2}[choice] == int(g[f"auto_variant_{tag}"])


@pytest.mark.parametrize("case", [c for c in CASES if c.startswith("kat_")])
def test_known_answer_pattern_is_exact(built, case):
    """A_ij = i, x_j = j: y_i = i * sum(cols of row i), exact in FP64 (every variant)."""
    g = load_golden(case)
    rp, col = g["row_ptr"], g["col"].astype(np.int64)
    n = int(g["n_rows"])
    rows = np.repeat(np.arange(n), np.diff(rp))
    exact = np.arange(n, dtype=np.float64) * np.bincount(rows, weights=col.astype(np.float64), minlength=n)
    for v in ("serial", "L", "D", "S", "auto"):
        assert bits_equal(g[f"y_{v}_f64"], exact), v


def test_hub_row_exposes_reference_D_carry_defect(built):
    """A row longer than a partition: the reference's D kernel restarts its
    tail carry at the row start (spmv_vnec_D_for_mxv.c:471) and double counts;
    the restatement reproduces that, the serial and L results do not."""
    g = load_golden("hub_row")
    assert not np.allclose(g["y_D_f64"][3], g["y_serial_f64"][3])
    assert np.allclose(g["y_L_f64"], g["y_serial_f64"], rtol=1e-12, atol=1e-12)


def test_neumaier_oracle_is_more_accurate_than_serial(built):
    from oracle import oracle as O
    from vnec_gb300 import generators as G

    m = G.lognormal(4000, sigma=2.0, seed=5)
    x = G.vector(m.n_cols, seed=6)
    y_c, cond = O.spmv_neumaier(m, x)
    # exact reference via float128-free pairwise: use numpy longdouble where available
    rows = np.repeat(np.arange(m.n_rows), np.diff(m.row_ptr))
    prod = m.val.astype(np.longdouble) * x[m.col].astype(np.longdouble)
    exact = np.zeros(m.n_rows, dtype=np.longdouble)
    np.add.at(exact, rows, prod)
    err_c = np.abs(y_c - exact.astype(np.float64)) / np.maximum(cond, 1e-300)
    err_s = np.abs(O.spmv_serial(m, x) - exact.astype(np.float64)) / np.maximum(cond, 1e-300)
    assert err_c.max() <= err_s.max()
    assert err_c.max() < 1e-15


@pytest.mark.skipif("not __import__('oracle.oracle', fromlist=['x']).ref_available()")
def test_oracle_matches_live_reference_on_fresh_matrices(built):
    """Where a reference build exists (its X86_SIMD build on an AVX-512 x86
    host, its ARM_NEON build on aarch64), the restatement with that build's
    constants matches it on fresh seeds."""
    from oracle import oracle as O
    from vnec_gb300 import generators as G

    b = O.ref_build()
    for m in (G.uniform_k(3000, 12, seed=21), G.rmat(12, 40000, seed=22), G.banded(2500, 17, seed=23),
              G.lognormal(2500, sigma=2.2, cap=600, seed=24)):
        x = G.vector(m.n_cols, seed=25)
        for dt in (np.float64, np.float32):
            for var, code in (("D", 1), ("S", 2), ("L", 3)):
                y_ref, _, _ = O.ref_spmv(code, m, x, dtype=dt)
                assert carry_equal(O.spmv_vnec(var, m, x, dtype=dt, build=b), y_ref, m, x, b["nparts"]), (var, dt)


def test_timed_cpu_baseline_loops(built):
    """The timed loops behind the CPU baseline (VNEC-L and VNEC-S FP64, format
    built once, `reps` calls) compute the same y as the untimed restatement and
    return a positive time per call."""
    from oracle import oracle as O
    from vnec_gb300 import generators as G

    m = G.uniform_k(4096, 16, seed=0)
    x = G.vector(m.n_cols, seed=1)
    for build in (O.X86, O.ARM):
        assert O.time_S_f64(m, x, build=build, warm=1, reps=3) > 0.0
        assert O.time_L_f64(m, x, build["nparts"], warm=1, reps=3) > 0.0
    y_ref, cond = O.spmv_neumaier(m, x)
    y = O.spmv_vnec("S", m, x, build=O.ARM)
    assert np.all(np.abs(y - y_ref) <= 1e-12 * cond)
