"""The allocation-free entry point, SpB_mxv_csr_noalloc_ext.

It exists for callers that cannot let the library allocate device memory
(a host whose device memory belongs to its own pool allocator, or a
latency-critical loop that must not pay for cudaMalloc/cudaFree).  Its
output is checked against the compensated FP64 oracle directly, within the
FP64 tolerance the other parity tests use (|y_i - y*_i| <= 1e-12 * sum_j
|a_ij x_j|), and against the plan-based entry point (SpB_mxv_device_ext on a
merge-path plan), on two calls in a row — the second call reuses the same
fixed scratch array as the first.  Edge cases: no rows, no nonzeros, only
empty rows, and one row that spans many merge-path tiles (its partial sums
travel through the scratch's carry slots).  This file is collected last so
that a run stopping at the first failure has already run every other test;
it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12
ITEMS_PER_TILE = 256 * 7  # the entry point's merge-path tile


def _bind():
    from vnec_gb300 import api

    lib = api.lib()
    f = lib.SpB_mxv_csr_noalloc_ext
    f.argtypes = [C.c_int64, C.c_int64, C.c_int64] + [C.c_void_p] * 6
    f.restype = C.c_int
    return api, f


def _oracle(m, x):
    from oracle import oracle as O

    return O.spmv_neumaier(m, x)


def _long_row_matrix():
    """2,000 short rows around one row of 20,000 nonzeros (more than 11
    tiles of 1,792 merge items), plus empty rows at both ends."""
    from conftest import Csr

    rng = np.random.default_rng(11)
    n = 2000
    lens = rng.integers(0, 9, n)
    lens[:3] = 0
    lens[-3:] = 0
    lens[977] = 20000
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    col = np.concatenate([np.sort(rng.choice(n if L < n else 50000, L, replace=False)) for L in lens]).astype(np.int32)
    n_cols = 50000
    val = rng.uniform(-1, 1, int(rp[-1]))
    return Csr(n, n_cols, rp, col, val)


def _matrix(name):
    from conftest import Csr
    from vnec_gb300 import generators as G

    if name == "rmat18":
        return G.rmat(18, 16 << 18, seed=5)
    if name == "hub_rows":
        return G.rmat(14, 1 << 20, a=0.7, b=0.1, c=0.1, seed=6)
    if name == "lognormal":
        return G.lognormal(50000, sigma=2.0, seed=7)
    if name == "long_row":
        return _long_row_matrix()
    if name == "empty_rows":
        return Csr(5000, 300, np.zeros(5001, dtype=np.int64), np.zeros(0, np.int32), np.zeros(0))
    raise ValueError(name)


def _call(noalloc, api, m, x_dev, stream):
    import torch

    rp = torch.from_numpy(np.ascontiguousarray(m.row_ptr, dtype=np.int32)).cuda()
    nnz = m.nnz
    ci = torch.from_numpy(np.ascontiguousarray(m.col[:nnz], dtype=np.int32)).cuda() if nnz else None
    vv = torch.from_numpy(np.ascontiguousarray(m.val[:nnz], dtype=np.float64)).cuda() if nnz else None
    outs = []
    for _ in range(2):
        y = torch.full((max(m.n_rows, 1),), float("nan"), dtype=torch.float64, device="cuda")
        rc = noalloc(m.n_rows, m.n_cols, nnz, rp.data_ptr(), ci.data_ptr() if ci is not None else None,
                     vv.data_ptr() if vv is not None else None, x_dev.data_ptr() if x_dev is not None else None,
                     y.data_ptr(), stream)
        assert rc == api.SpB_SUCCESS, api.last_error()
        torch.cuda.synchronize()
        outs.append(y.cpu().numpy()[: m.n_rows])
    return outs


@pytest.mark.parametrize("name", ["rmat18", "hub_rows", "lognormal", "long_row"])
def test_noalloc_matches_oracle_and_plan_on_two_calls(built, name):
    import torch

    from vnec_gb300 import generators as G

    api, noalloc = _bind()
    m = _matrix(name)
    if name == "long_row":
        assert int(np.max(np.diff(m.row_ptr))) > 3 * ITEMS_PER_TILE
    xv = G.vector(m.n_cols, seed=8)
    y_star, cond = _oracle(m, xv)

    # Existing entry point: merge-path plan (same tile shape), device pointers.
    plan = api.Plan(m, kernel=api.KERNEL_L, pipeline_stages=1, threads_per_block=256, items_per_thread=7)
    x = torch.from_numpy(xv).cuda()
    y_plan = torch.empty(m.n_rows, dtype=torch.float64, device="cuda")
    plan.mxv_device(x.data_ptr(), y_plan.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    y_ref = y_plan.cpu().numpy()
    plan.free()

    for call, y in enumerate(_call(noalloc, api, m, x, torch.cuda.current_stream().cuda_stream)):
        assert np.all(np.isfinite(y)), f"call {call}: rows left unwritten"
        assert np.all(np.abs(y - y_star) <= TOL_F64 * cond + 1e-300), f"call {call} vs oracle"
        assert np.all(np.abs(y - y_ref) <= TOL_F64 * cond + 1e-300), f"call {call} vs plan entry point"


def test_noalloc_rows_without_nonzeros(built):
    """nnz = 0 (only empty rows): every y entry is written as zero, with no
    column, value or x array passed; n_rows = 0 is a successful no-op."""
    import torch

    api, noalloc = _bind()
    m = _matrix("empty_rows")
    for call, y in enumerate(_call(noalloc, api, m, None, torch.cuda.current_stream().cuda_stream)):
        assert np.array_equal(y, np.zeros(m.n_rows)), f"call {call}"
    y = torch.full((4,), 7.0, dtype=torch.float64, device="cuda")
    rp = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert noalloc(0, 0, 0, rp.data_ptr(), None, None, None, y.data_ptr(), None) == api.SpB_SUCCESS
    torch.cuda.synchronize()
    assert y.cpu().tolist() == [7.0] * 4


def test_noalloc_rejects_inputs_beyond_its_scratch(built):
    api, noalloc = _bind()
    rc = noalloc(300_000_000, 1000, 200_000_000, 1, 1, 1, 1, 1, None)
    assert rc == api.SpB_FAILURE
    assert "allocation-free limit" in api.last_error()
    # Sizes whose sum would overflow a signed 64-bit integer are rejected
    # one by one before the sum is formed.
    big = (1 << 63) - 10
    for n_rows, nnz in ((big, 5), (5, big), (big, big)):
        assert noalloc(n_rows, 1000, nnz, 1, 1, 1, 1, 1, None) == api.SpB_FAILURE
        assert "allocation-free limit" in api.last_error()
    assert noalloc(-1, 10, 10, 1, 1, 1, 1, 1, None) == api.SpB_FAILURE
    assert noalloc(10, 1 << 40, 10, 1, 1, 1, 1, 1, None) == api.SpB_FAILURE
