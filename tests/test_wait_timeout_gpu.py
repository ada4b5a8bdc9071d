"""Bounded device waits: the timeout path of the pipelined merge-path kernel.

Every mbarrier wait of that kernel gives up after a poll limit, raises the
plan's device error flag, finishes the bulk copies it still has in flight and
exits.  Setting the limit to zero polls makes every CTA give up at its first
wait — the wait runs out without any fault — so the test can check that the
status call reports the timeout, that the report clears, and that the next
call with the default limit is correct.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("arith", ["fp64", "df32"])
def test_pipeline_wait_timeout_is_reported_then_cleared(built, arith):
    import torch

    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    m = G.rmat(16, 16 << 16, seed=7)
    xv = G.vector(m.n_cols, seed=9)
    y_star, cond = O.spmv_neumaier(m, xv)
    ar = api.ARITH_FP64 if arith == "fp64" else api.ARITH_DF32
    p = api.Plan(m, kernel=api.KERNEL_L, pipeline_stages=2, arithmetic=ar)
    assert p.info().pipeline_stages == 2
    stream = torch.cuda.current_stream().cuda_stream
    x = torch.from_numpy(xv).cuda()
    y = torch.zeros(m.n_rows, dtype=torch.float64, device="cuda")

    p.set_wait_polls(0)
    p.mxv_device(x.data_ptr(), y.data_ptr(), stream)
    with pytest.raises(api.VnecError, match="timed out"):
        p.device_status(stream)
    p.device_status(stream)  # the report was cleared

    p.set_wait_polls(-1)
    for _ in range(2):
        y.fill_(float("nan"))
        p.mxv_device(x.data_ptr(), y.data_ptr(), stream)
        p.device_status(stream)
        yh = y.cpu().numpy()
        assert np.all(np.abs(yh - y_star) <= 1e-12 * cond + 1e-300)
    p.free()


def test_wait_polls_accepted_by_plans_without_waits(built):
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    m = G.rmat(12, 16 << 12, seed=3)
    xv = G.vector(m.n_cols, seed=4)
    for kernel in (api.KERNEL_S, api.KERNEL_D):
        p = api.Plan(m, kernel=kernel)
        p.set_wait_polls(0)
        y = p.mxv_host(xv)
        p.device_status()
        assert np.all(np.isfinite(y))
        p.free()
