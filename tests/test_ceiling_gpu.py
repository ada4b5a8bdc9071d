"""The measurement kernel behind bench.py's gather-ceiling leg
(SpB_VNEC_stream_gather_ext): its partial sums add up to sum_i val[i] *
x[col[i]], for item counts that do and do not fill whole rounds of loads."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [0, 1, 1000, 1 << 20, (1 << 22) + 12345])
def test_stream_gather_sum(built, n):
    import torch

    from vnec_gb300 import api

    rng = np.random.default_rng(n)
    n_x = 50_000
    xv = rng.uniform(-1, 1, n_x)
    col = rng.integers(0, n_x, n).astype(np.int32)
    val = rng.uniform(-1, 1, n)
    x, c, v = (torch.from_numpy(a).cuda() for a in (xv, col, val))
    out = torch.full((api.STREAM_GATHER_BLOCKS,), float("nan"), dtype=torch.float64, device="cuda")
    if n == 0:
        api.stream_gather(x.data_ptr(), n_x, 0, 0, 0, out.data_ptr())
        torch.cuda.synchronize()
        assert torch.isnan(out).all()  # nothing launched
        return
    api.stream_gather(x.data_ptr(), n_x, c.data_ptr(), v.data_ptr(), n, out.data_ptr())
    torch.cuda.synchronize()
    prod = val * xv[col]
    assert abs(float(out.sum().item()) - float(prod.sum())) <= 1e-12 * float(np.abs(prod).sum()) + 1e-300
