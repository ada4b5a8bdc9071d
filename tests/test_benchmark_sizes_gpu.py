"""Parity at the benchmarked sizes, through the C ABI.

Each benchmark workload is checked at its full size, so a regression that
only shows at scale cannot pass:

* uniform 65,536 x 16 (exactly 16 distinct sorted uniform columns per row,
  values and x U(-1, 1), seed 0) — the reference's CPU-sized case — through
  the reference harness's own call sequence (IRD_VNEC, then Build_VNEC_S_FP64
  + SpMV_VNEC_S_FP64, src/operation/test/test_spmv_vnec.cpp:197-256), through
  the forced D and L builds, and through SpB_mxv with a NULL handle; plus the
  harness's known-answer pattern (A_ij = i, x_j = j, :169,185) bit for bit;
* the 27-point stencil on 256^3 (16.7M rows, 449,455,096 nonzeros) in plain
  FP64 and in the FP32, BF16-with-row-scale and FP32 hi+lo forms, on the
  default (shared-pattern) layout;
* the 512-matrix batch (rows log-uniform in [1e3, 2e5], lognormal(ln 8, 1.5)
  row lengths capped at 4,096, seed 0) at k = 1, 4, 8, 16, 32 right-hand
  sides in the FP64, FP32 and DF32 forms, with autotuned layouts, sampled
  rows of every matrix against the compensated oracle.

Criteria (row-wise, against the compensated FP64 oracle, cond = sum_j
|a_ij x_j|): FP64 and DF32 1e-12, FP32 1e-6, BF16 1e-2 (the reference's
per-row check, test_spmv_vnec.cpp:261-269, with a conditioning-aware
denominator).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "fp32": 1e-6, "bf16": 1e-2, "df32": 1e-12}


def _check(y, y_ref, cond, tol, what):
    err = np.abs(np.asarray(y, dtype=np.float64) - y_ref)
    bad = ~(err <= tol * cond + 1e-300)
    assert not bad.any(), (f"{what}: {bad.sum()} rows exceed {tol:g}*cond; worst "
                           f"{np.max(err / np.maximum(cond, 1e-300)):.3g}")


@pytest.fixture(scope="module")
def uniform64k():
    from vnec_gb300 import generators as G

    m = G.uniform_k(65536, 16, seed=0)
    assert m.n_rows == 65536 and m.nnz == 16 * 65536
    return m, G.vector(m.n_cols, seed=0)


def test_uniform64k_reference_flow(built, uniform64k):
    """IRD_VNEC picks S here (as the reference's x86 build does, IRD 0.125);
    S, D and L builds and SpB_mxv(…, NULL) all meet 1e-12 row-wise."""
    from oracle import oracle as O
    from vnec_gb300 import api

    m, xv = uniform64k
    y_ref, cond = O.spmv_neumaier(m, xv)
    A = api.Matrix.from_csr(m)
    x = api.Vector(xv)
    assert api.IRD_VNEC(A, api.SpB_FP64) == api.SpB_VNEC_S
    flows = {"S": (api.Build_VNEC_S_FP64, api.SpMV_VNEC_S_FP64, api.VNEC_S_free_fp64),
             "D": (api.Build_VNEC_D_FP64, api.SpMV_VNEC_D_FP64, api.VNEC_D_free_fp64),
             "L": (api.Build_VNEC_L, api.SpMV_VNEC_L_FP64, api.VNEC_L_free)}
    for name, (build, spmv, free) in flows.items():
        h = build(A)
        try:
            for _ in range(2):
                y = api.Vector(n=m.n_rows)
                spmv(y, A, x, h)
                _check(y.values, y_ref, cond, TOL["fp64"], f"VNEC-{name}")
        finally:
            free(h)
    y = api.Vector(n=m.n_rows)
    api.SpB_mxv(y, A, x)
    _check(y.values, y_ref, cond, TOL["fp64"], "SpB_mxv")
    api.lib().SpB_VNEC_forget_ext(A.handle)


def test_uniform64k_known_answer(built, uniform64k):
    """A_ij = i, x_j = j on the same structure: every build returns the exact
    integers bit for bit."""
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    m, _ = uniform64k
    kat, xk = G.kat_values(m)
    rows = np.repeat(np.arange(m.n_rows, dtype=np.int64), np.diff(m.row_ptr))
    exact = np.arange(m.n_rows, dtype=np.float64) * np.bincount(rows, weights=m.col[: m.nnz].astype(np.float64),
                                                                minlength=m.n_rows)
    assert exact.max() < 2.0 ** 53
    A = api.Matrix.from_csr(kat)
    x = api.Vector(xk)
    for build, spmv, free in ((api.Build_VNEC_S_FP64, api.SpMV_VNEC_S_FP64, api.VNEC_S_free_fp64),
                              (api.Build_VNEC_D_FP64, api.SpMV_VNEC_D_FP64, api.VNEC_D_free_fp64),
                              (api.Build_VNEC_L, api.SpMV_VNEC_L_FP64, api.VNEC_L_free)):
        h = build(A)
        try:
            y = api.Vector(n=m.n_rows)
            spmv(y, A, x, h)
            assert y.values.tobytes() == exact.tobytes(), build.__name__
        finally:
            free(h)
    y = api.Vector(n=m.n_rows)
    api.SpB_mxv(y, A, x)
    assert y.values.tobytes() == exact.tobytes()
    api.lib().SpB_VNEC_forget_ext(A.handle)


def test_stencil256_all_forms(built):
    """27-point stencil on 256^3 in every form, default layout (shared column
    patterns for the precision forms), two calls each (identical bits)."""
    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    m = G.stencil27(256, seed=0)
    assert m.n_rows == 256 ** 3 and m.nnz == 766 ** 3
    xv = G.vector(m.n_cols, seed=0)
    y_ref, cond = O.spmv_neumaier(m, xv)
    forms = {"fp64": api.PREC_FP64, "fp32": api.PREC_FP32, "bf16": api.PREC_BF16, "df32": api.PREC_DF32}
    for name, prec in forms.items():
        p = api.Plan(m, kernel=api.KERNEL_S, precision=prec)
        try:
            assert p.info().precision == prec
            y = p.mxv_host(xv)
            _check(y, y_ref, cond, TOL[name], f"stencil256 {name}")
            assert p.mxv_host(xv).tobytes() == y.tobytes()
        finally:
            p.free()
    # The learned selection (the default for SpB_mxv) on the same matrix.
    p = api.Plan(m, kernel=api.KERNEL_LEARNED)
    try:
        _check(p.mxv_host(xv), y_ref, cond, TOL["fp64"], "stencil256 learned")
    finally:
        p.free()


@pytest.fixture(scope="module")
def batch512():
    from vnec_gb300 import generators as G

    mats = G.batch_lognormal(512, seed=0)
    yield mats
    for m in mats:
        m.free()


def _sampled_rows(mats, rng, per_mat=24):
    """Per matrix: up to per_mat sampled row indices and the sub-CSR of those rows."""
    from conftest import Csr

    out = []
    for m in mats:
        rows = np.sort(rng.choice(m.n_rows, size=min(per_mat, m.n_rows), replace=False))
        lens = np.diff(m.row_ptr)[rows]
        rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        idx = np.concatenate([np.arange(m.row_ptr[r], m.row_ptr[r + 1]) for r in rows]).astype(np.int64)
        out.append((rows, Csr(len(rows), m.n_cols, rp, m.col[idx], m.val[idx])))
    return out


@pytest.mark.parametrize("k", [1, 4, 8, 16, 32])
def test_batch512_all_forms(built, batch512, k):
    from oracle import oracle as O
    from vnec_gb300 import api

    mats = batch512
    assert len(mats) == 512
    rng = np.random.default_rng(100 + k)
    samples = _sampled_rows(mats, rng)
    for name, prec in (("fp64", api.PREC_FP64), ("fp32", api.PREC_FP32), ("df32", api.PREC_DF32)):
        p = api.BatchPlan(mats, k, precision=prec, autotune=True)
        try:
            ro, co = p.offsets()
            X = np.random.default_rng(k).uniform(-1, 1, int(co[-1]) * k)
            Y = p.mxv_host(X).reshape(-1)
            for i, (rows, sub) in enumerate(samples):
                Xi = X[co[i] * k:co[i + 1] * k].reshape(mats[i].n_cols, k)
                y_ref, cond = O.spmm_neumaier(sub, Xi)
                Yi = Y[ro[i] * k:ro[i + 1] * k].reshape(mats[i].n_rows, k)[rows]
                _check(Yi, y_ref, cond, TOL[name], f"batch512 k={k} {name} matrix {i}")
        finally:
            p.free()


def test_rmat24_reference_flow_through_build_vnec_l(built):
    """The reference harness's call sequence on the 2^24-row power-law matrix
    (>= 3e6 rows: Build_VNEC_L + SpMV_VNEC_L_FP64 on host vectors): from 2^26
    nonzeros on Build_VNEC_L hands back the automatic selection's plan; y must
    meet 1e-12 row-wise on two calls, and the handle must be released both ways
    the library allows."""
    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    m = G.rmat(24, 1 << 28, seed=1)
    xv = G.vector(m.n_cols, seed=1)
    y_ref, cond = O.spmv_neumaier(m, xv)
    A = api.Matrix.from_csr(m)
    x = api.Vector(xv)
    h = api.Build_VNEC_L(A)
    try:
        inf = api.Info()
        assert api.lib().SpB_VNEC_plan_info_ext(h, api.C.byref(inf)) == api.SpB_SUCCESS
        assert inf.kernel != api.KERNEL_L  # the selected plan, not the merge path
        for _ in range(2):
            y = api.Vector(n=m.n_rows)
            api.SpMV_VNEC_L_FP64(y, A, x, h)
            _check(y.values, y_ref, cond, TOL["fp64"], "Build_VNEC_L R-MAT 2^24")
    finally:
        api.VNEC_L_free(h)
