"""The allocation-free entry point, SpB_mxv_csr_noalloc_ext.

It exists for callers that cannot let the library allocate device memory
(a host whose device memory belongs to its own pool allocator, or a
latency-critical loop that must not pay for cudaMalloc/cudaFree).  Its output
must agree with the plan-based entry point (SpB_mxv_device_ext on a merge-path
plan) within the FP64 tolerance the other parity tests use, on two calls in a
row — the second call reuses the same fixed scratch array as the first.  This
file is collected last so that a run stopping at the first failure has
already run every other test; it also passes on its own in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_F64 = 1e-12


def _bind():
    from vnec_gb300 import api

    lib = api.lib()
    f = lib.SpB_mxv_csr_noalloc_ext
    f.argtypes = [C.c_int64, C.c_int64, C.c_int64] + [C.c_void_p] * 6
    f.restype = C.c_int
    return api, f


def _within_tolerance(y, y_ref, m, x):
    from oracle import oracle as O

    _, cond = O.spmv_neumaier(m, x)
    return bool(np.all(np.abs(y - y_ref) <= TOL_F64 * cond + 1e-300))


@pytest.mark.parametrize("name", ["rmat18", "hub_rows", "lognormal"])
def test_noalloc_matches_plan_entry_point_on_two_calls(built, name):
    import torch

    from vnec_gb300 import generators as G

    api, noalloc = _bind()
    if name == "rmat18":
        m = G.rmat(18, 16 << 18, seed=5)
    elif name == "hub_rows":
        m = G.rmat(14, 1 << 20, a=0.7, b=0.1, c=0.1, seed=6)
    else:
        m = G.lognormal(50000, sigma=2.0, seed=7)
    xv = G.vector(m.n_cols, seed=8)

    # Existing entry point: merge-path plan (same tile shape), device pointers.
    plan = api.Plan(m, kernel=api.KERNEL_L, pipeline_stages=1, threads_per_block=256, items_per_thread=7)
    x = torch.from_numpy(xv).cuda()
    y_plan = torch.empty(m.n_rows, dtype=torch.float64, device="cuda")
    plan.mxv_device(x.data_ptr(), y_plan.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    y_ref = y_plan.cpu().numpy()
    plan.free()

    # New entry point: the caller owns every device array.
    rp = torch.from_numpy(np.ascontiguousarray(m.row_ptr, dtype=np.int32)).cuda()
    ci = torch.from_numpy(np.ascontiguousarray(m.col[: m.nnz], dtype=np.int32)).cuda()
    vv = torch.from_numpy(np.ascontiguousarray(m.val[: m.nnz], dtype=np.float64)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        y = torch.full((m.n_rows,), float("nan"), dtype=torch.float64, device="cuda")
        rc = noalloc(m.n_rows, m.n_cols, m.nnz, rp.data_ptr(), ci.data_ptr(), vv.data_ptr(), x.data_ptr(),
                     y.data_ptr(), stream)
        assert rc == api.SpB_SUCCESS, api.last_error()
        torch.cuda.synchronize()
        assert _within_tolerance(y.cpu().numpy(), y_ref, m, xv), f"call {call}"


def test_noalloc_rejects_inputs_beyond_its_scratch(built):
    api, noalloc = _bind()
    rc = noalloc(300_000_000, 1000, 200_000_000, 1, 1, 1, 1, 1, None)
    assert rc == api.SpB_FAILURE
    assert "allocation-free limit" in api.last_error()
