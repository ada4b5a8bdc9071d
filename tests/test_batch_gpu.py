"""GPU parity of the batched multi-right-hand-side path, through the C ABI.

Y_m = A_m X_m for a batch of uneven CSR matrices and k right-hand sides, one
call for the whole batch.  Criteria (per matrix, row and right-hand side,
against the compensated FP64 oracle, conditioning sum_j |a_ij x_j|):
  FP64 form: |Y - Yhat| <= 1e-12 * cond
  FP32 form: |Y - Yhat| <= 1e-6  * cond
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import Csr

pytestmark = pytest.mark.gpu

TOL = {0: 1e-12, 1: 1e-6, 3: 1e-12}
KS = [1, 2, 4, 8, 16, 32]


def lanes_for(k):
    return [L for L in (1, 2, 4, 8, 16, 32) if 32 % L == 0 and k % L == 0 and k // L in (1, 2, 4, 8)]


def edge_mats(seed=5):
    """Shapes the layout must handle: all-empty rows, 1x1, rectangular, one
    long dense row (chunked), rows longer than every group, a 0-column matrix."""
    rng = np.random.default_rng(seed)
    mats = [Csr(5, 7, np.zeros(6, np.int64), np.zeros(0, np.int32), np.zeros(0))]
    mats.append(Csr(1, 1, [0, 1], [0], [rng.uniform(-1, 1)]))
    # rectangular 40 x 300, ragged rows with some empty
    rp, ci = [0], []
    for r in range(40):
        n = int(rng.integers(0, 30)) if r % 5 else 0
        ci += sorted(rng.choice(300, size=n, replace=False).tolist())
        rp.append(len(ci))
    mats.append(Csr(40, 300, rp, ci, rng.uniform(-1, 1, len(ci))))
    # 3 rows: a dense row of 5000 columns between two short rows
    ci = [7] + list(range(5000)) + [1, 4999]
    mats.append(Csr(3, 5000, [0, 1, 5001, 5003], ci, rng.uniform(-1, 1, len(ci))))
    mats.append(Csr(4, 0, np.zeros(5, np.int64), np.zeros(0, np.int32), np.zeros(0)))
    return mats


def small_batch(seed=0, n=10):
    from vnec_gb300 import generators as gen

    mats = gen.batch_lognormal(n, rows_lo=30, rows_hi=3000, sigma=1.5, cap=2048, seed=seed)
    return mats + edge_mats(seed)


def oracle_batch(mats, X, k, co, ro):
    from oracle import oracle as O

    ys, conds = [], []
    for i, m in enumerate(mats):
        Xi = X[co[i] * k:co[i + 1] * k].reshape(m.n_cols, k)
        if m.n_rows == 0:
            continue
        if m.n_cols == 0:
            ys.append(np.zeros((m.n_rows, k)))
            conds.append(np.zeros((m.n_rows, k)))
            continue
        y, c = O.spmm_neumaier(m, Xi)
        ys.append(y)
        conds.append(c)
    return np.concatenate(ys), np.concatenate(conds)


def check(Y, Yref, cond, tol):
    Y = Y.reshape(Yref.shape)
    err = np.abs(Y - Yref)
    bad = ~(err <= tol * cond)
    assert not bad.any(), f"{bad.sum()} entries exceed {tol}*cond; worst {np.max(err / np.maximum(cond, 1e-300))}"


@pytest.fixture(scope="module")
def batch():
    mats = small_batch()
    return mats


def _x(plan, k, seed=1):
    _, co = plan.offsets()
    return np.random.default_rng(seed).uniform(-1, 1, int(co[-1]) * k)


@pytest.mark.parametrize("k", KS)
@pytest.mark.parametrize("precision", [0, 1, 3], ids=["fp64", "fp32", "df32"])
def test_batch_all_lanes(built, batch, k, precision):
    """Every supported lanes-per-row layout, with a small long-row limit so that
    chunked rows (and the in-kernel long-row completion) are exercised."""
    from vnec_gb300 import api

    for L, unroll in [(L, u) for L in lanes_for(k) for u in (1, 2, 3)]:
        p = api.BatchPlan(batch, k, lanes=L, long_row_len=64, precision=precision, max_steps=4, unroll=unroll,
                          k1_layout=-1)
        try:
            ro, co = p.offsets()
            X = _x(p, k)
            Yref, cond = oracle_batch(batch, X, k, co, ro)
            inf = p.info()
            assert inf.kernel == api.KERNEL_BATCH and inf.lanes == L and inf.rhs == k
            for _ in range(3):  # repeated calls: the arrival counters must come back to 0
                Y = p.mxv_host(X)
                check(Y, Yref, cond, TOL[precision])
        finally:
            p.free()


@pytest.mark.parametrize("k", [1, 4, 8, 32])
@pytest.mark.parametrize("precision", [0, 1, 3], ids=["fp64", "fp32", "df32"])
def test_batch_staged_entries_bit_identical(built, batch, k, precision):
    """Kernel mode 3 (each task's columns and values read in bulk and passed to
    the slots by shuffles) sums the same steps in the same order as mode 1:
    identical Y for every lanes layout, with long rows spanning several bulk
    rounds."""
    from vnec_gb300 import api

    for L in lanes_for(k):
        ys = []
        for unroll in (1, 3):
            p = api.BatchPlan(batch, k, lanes=L, long_row_len=2048, precision=precision, unroll=unroll,
                              k1_layout=-1)
            try:
                ys.append(p.mxv_host(_x(p, k)))
            finally:
                p.free()
        assert ys[0].tobytes() == ys[1].tobytes(), L


@pytest.mark.parametrize("k", [1, 8, 32])
def test_batch_default_layout_and_graph_off(built, batch, k):
    from vnec_gb300 import api

    outs = []
    for graph in (True, False):
        p = api.BatchPlan(batch, k, graph=graph)
        try:
            ro, co = p.offsets()
            X = _x(p, k, seed=3)
            Yref, cond = oracle_batch(batch, X, k, co, ro)
            Y = p.mxv_host(X)
            check(Y, Yref, cond, TOL[0])
            outs.append(Y)
        finally:
            p.free()
    assert outs[0].tobytes() == outs[1].tobytes()


@pytest.mark.parametrize("k", [1, 4, 32])
def test_batch_df32_guard_for_out_of_range_x(built, batch, k):
    """X values outside the double-float split range switch the same launch to
    FP64; the next in-range X runs double-float again."""
    from vnec_gb300 import api

    p = api.BatchPlan(batch, k, precision=api.PREC_DF32, long_row_len=64)
    try:
        ro, co = p.offsets()
        for bad in (1e30, 3e-20, 5e-324, None):
            X = _x(p, k, seed=6)
            if bad is not None:
                X[::13] = bad
            Yref, cond = oracle_batch(batch, X, k, co, ro)
            check(p.mxv_host(X), Yref, cond, TOL[3])
    finally:
        p.free()


def test_batch_df32_rejects_out_of_range_values(built, batch):
    from vnec_gb300 import api

    bad = Csr(2, 2, [0, 1, 2], [0, 1], [1e-30, 2.0])
    with pytest.raises(api.VnecError, match="DF32"):
        api.BatchPlan([batch[0], bad], 4, precision=api.PREC_DF32)


@pytest.mark.parametrize("precision", [0, 1, 3], ids=["fp64", "fp32", "df32"])
def test_batch_host_calls_in_parts(built, precision):
    """Host-vector calls copy X in, compute and copy Y out part by part (groups
    of row windows, each with the X rows of its matrices): bit-identical to the
    device-pointer call for any number of parts, including windows that split a
    matrix and matrices without rows."""
    import torch

    from vnec_gb300 import api

    mats = small_batch(seed=9, n=24)
    k = 4
    outs = []
    for parts in (1, 3, 8, 64):
        p = api.BatchPlan(mats, k, precision=precision, window_rows=500, host_parts=parts, long_row_len=128)
        try:
            ro, co = p.offsets()
            X = _x(p, k, seed=4)
            Y = p.mxv_host(X)
            x = torch.from_numpy(X).cuda()
            y = torch.full((int(ro[-1]) * k,), float("nan"), dtype=torch.float64, device="cuda")
            p.mxv_device(x.data_ptr(), y.data_ptr())
            torch.cuda.synchronize()
            assert y.cpu().numpy().tobytes() == Y.reshape(-1).tobytes(), parts
            outs.append(Y)
        finally:
            p.free()
    Yref, cond = oracle_batch(mats, X, k, co, ro)
    check(outs[-1], Yref, cond, TOL[precision])


def test_batch_graph_pointer_changes(built, batch):
    """The captured graph follows the (x, y) pair of each call."""
    import torch

    from vnec_gb300 import api

    k = 8
    p = api.BatchPlan(batch, k, long_row_len=128)
    try:
        ro, co = p.offsets()
        xs = [_x(p, k, seed=s) for s in (10, 11)]
        refs = [oracle_batch(batch, X, k, co, ro) for X in xs]
        dx = [torch.from_numpy(X).cuda() for X in xs]
        dy = [torch.full((int(ro[-1]) * k,), float("nan"), dtype=torch.float64, device="cuda") for _ in xs]
        s = torch.cuda.Stream()
        for order in ([0, 1, 0], [1, 1, 0]):
            for i in order:
                dy[i].fill_(float("nan"))
                with torch.cuda.stream(s):
                    p.mxv_device(dx[i].data_ptr(), dy[i].data_ptr(), s.cuda_stream)
                s.synchronize()
                check(dy[i].cpu().numpy(), refs[i][0], refs[i][1], TOL[0])
    finally:
        p.free()


def test_batch_reference_matrices(built):
    """Plans from reference-layout SpB_Matrix objects (64-bit offsets/columns)."""
    from vnec_gb300 import api

    mats = small_batch(seed=4, n=4)
    As = [api.Matrix.from_csr(m) for m in mats]
    p = api.BatchPlan(As, 4)
    try:
        ro, co = p.offsets()
        X = _x(p, 4)
        Yref, cond = oracle_batch(mats, X, 4, co, ro)
        check(p.mxv_host(X), Yref, cond, TOL[0])
    finally:
        p.free()


@pytest.mark.parametrize("precision", [0, 1])
def test_batch_autotune(built, batch, precision):
    """The autotuner times every candidate layout on the batch and keeps the
    fastest; the plan built with its choice is correct."""
    from vnec_gb300 import api

    k = 16
    p = api.BatchPlan(batch, k, autotune=True, precision=precision)
    try:
        cand, ms, best = p.tuning()
        assert len(cand) == len(lanes_for(k)) * 3 * 2 * 3  # lanes x long-row limit x warps x kernel mode
        assert 0 <= best < len(cand) and all(t > 0 for t in ms)
        assert ms[best] == min(ms)
        inf = p.info()
        assert (inf.lanes, inf.long_row_len, inf.threads_per_block // 32) == cand[best][:3]
        ro, co = p.offsets()
        X = _x(p, k)
        Yref, cond = oracle_batch(batch, X, k, co, ro)
        check(p.mxv_host(X), Yref, cond, TOL[precision])
    finally:
        p.free()


def test_batch_invalid(built, batch):
    import torch

    from vnec_gb300 import api

    for kw in (dict(k=3), dict(k=64), dict(k=8, lanes=3), dict(k=32, lanes=2), dict(k=4, warps_per_block=5),
               dict(k=4, precision=2)):
        k = kw.pop("k")
        with pytest.raises(api.VnecError):
            api.BatchPlan(batch, k, **kw)
    bad = Csr(2, 2, [0, 1, 2], [0, 5], [1.0, 2.0])  # column out of range
    with pytest.raises(api.VnecError, match="matrix 1"):
        api.BatchPlan([batch[0], bad], 2)
    # misaligned device pointers are rejected on the host for k / lanes >= 2
    p = api.BatchPlan(batch, 4, lanes=2)
    try:
        ro, co = p.offsets()
        x = torch.zeros(int(co[-1]) * 4 + 1, dtype=torch.float64, device="cuda")
        y = torch.zeros(int(ro[-1]) * 4 + 1, dtype=torch.float64, device="cuda")
        with pytest.raises(api.VnecError, match="aligned"):
            p.mxv_device(x.data_ptr() + 8, y.data_ptr(), 0)
    finally:
        p.free()


def test_batch_config_scale_sample(built):
    """The batched workload's distribution (rows log-uniform in [1e3, 2e5],
    lognormal(ln 8, 1.5) lengths capped at 4096) on 24 matrices, k = 32."""
    from vnec_gb300 import api
    from vnec_gb300 import generators as gen

    mats = gen.batch_lognormal(24, seed=7)
    k = 32
    p = api.BatchPlan(mats, k)
    try:
        ro, co = p.offsets()
        X = _x(p, k, seed=2)
        Yref, cond = oracle_batch(mats, X, k, co, ro)
        check(p.mxv_host(X), Yref, cond, TOL[0])
    finally:
        p.free()


@pytest.mark.parametrize("k", [1, 8, 32])
@pytest.mark.parametrize("precision", [0, 1, 3], ids=["fp64", "fp32", "df32"])
def test_batch_dispatch_modes_bit_identical(built, batch, k, precision):
    """One warp per task (blocks dispatched in task order) and persistent warps
    striding the task list run every task the same way: identical Y, also
    through the host path split into parts and with the autotuner choosing."""
    from vnec_gb300 import api

    outs = []
    for dispatch in (1, 2):
        p = api.BatchPlan(batch, k, precision=precision, long_row_len=64, dispatch=dispatch, k1_layout=-1)
        try:
            X = _x(p, k)
            outs.append(p.mxv_host(X))
            assert p.mxv_host(X).tobytes() == outs[-1].tobytes()
        finally:
            p.free()
    assert outs[0].tobytes() == outs[1].tobytes()
    p = api.BatchPlan(batch, k, precision=precision, autotune=True)
    try:
        ro, co = p.offsets()
        X = _x(p, k)
        Yref, cond = oracle_batch(batch, X, k, co, ro)
        check(p.mxv_host(X), Yref, cond, TOL[precision])
    finally:
        p.free()


@pytest.mark.parametrize("precision", [0, 1, 3], ids=["fp64", "fp32", "df32"])
def test_batch_k1_runs_as_one_sliced_plan(built, batch, precision):
    """At k = 1 the batch runs as one sliced plan of its block-diagonal
    concatenation (the default, reported as lanes = 0).  It and the batch
    kernel (k1_layout = -1) both meet the form's tolerance against the oracle;
    the device call with and without a graph, the host call in parts and
    pipelined host calls give the same bits; the DF32 guard covers
    out-of-range X."""
    import torch

    from vnec_gb300 import api

    ref = api.BatchPlan(batch, 1, precision=precision, k1_layout=-1)
    try:
        ro, co = ref.offsets()
        X = _x(ref, 1, seed=5)
        Yref, cond = oracle_batch(batch, X, 1, co, ro)
        Yk = ref.mxv_host(X)
        assert ref.info().lanes >= 1
    finally:
        ref.free()
    check(Yk, Yref, cond, TOL[precision])
    outs = []
    for graph in (True, False):
        p = api.BatchPlan(batch, 1, precision=precision, graph=graph, host_parts=3, window_rows=500)
        try:
            inf = p.info()
            assert inf.kernel == api.KERNEL_BATCH and inf.lanes == 0 and inf.rhs == 1
            assert inf.items_per_thread in (4, 8, 12, 16) and inf.precision == precision
            assert np.array_equal(p.offsets()[0], ro) and np.array_equal(p.offsets()[1], co)
            Y = p.mxv_host(X)
            check(Y, Yref, cond, TOL[precision])
            x = torch.from_numpy(X).cuda()
            y = torch.full((int(ro[-1]),), float("nan"), dtype=torch.float64, device="cuda")
            for _ in range(2):
                p.mxv_device(x.data_ptr(), y.data_ptr())
            torch.cuda.synchronize()
            assert y.cpu().numpy().tobytes() == Y.reshape(-1).tobytes()
            hx = torch.from_numpy(X).pin_memory()
            hys = [torch.empty(int(ro[-1]), dtype=torch.float64).pin_memory() for _ in range(3)]
            for hy in hys:
                p.mxv_host_async(hx.numpy(), hy.numpy())
            p.host_wait()
            for hy in hys:
                assert hy.numpy().tobytes() == Y.reshape(-1).tobytes()
            if precision == api.PREC_DF32:
                Xb = X.copy()
                Xb[::13] = 1e30
                Yb, condb = oracle_batch(batch, Xb, 1, co, ro)
                check(p.mxv_host(Xb), Yb, condb, TOL[precision])
            outs.append(Y)
        finally:
            p.free()
    assert outs[0].tobytes() == outs[1].tobytes()


def test_batch_k1_layout_option_checked(built, batch):
    from vnec_gb300 import api

    for bad in (1, -2):
        with pytest.raises(api.VnecError, match="k1_layout"):
            api.BatchPlan(batch, 1, k1_layout=bad)
