"""Device-resident power iteration on the mxv path (PageRank).

The reference's test data path is a PageRank workload
(``src/operation/test/test_spmv_vnec.hpp:27``); here the same computation
runs as a chain of SpMV calls whose vectors never leave the GPU:

    r_{t+1} = d * P r_t + ((1 - d) + d * sum_{i dangling} r_t[i]) / n

with P the column-stochastic transition matrix of the graph (P[j, i] =
1 / outdeg(i) for an edge i -> j).  P r is planned as the transpose of the
row-scaled adjacency (``transpose=True``).  Every iteration runs only the
library's kernels: a device dot product of r with the dangling mask
(``SpB_VNEC_dot_ext``) writes the dangling mass to a device scalar, and the
SpMV folds d, the teleport term and that scalar into its stores
(``SpB_mxv_axpbyg_ext``).  Every ``check_every`` iterations a device L1
distance (``SpB_VNEC_dot_ext``, mode 1) is read back for the convergence
test: the only host round trip.
"""
from __future__ import annotations

import numpy as np

from . import api


class _Csr:
    def __init__(self, n_rows, n_cols, row_ptr, col, val):
        self.n_rows, self.n_cols = int(n_rows), int(n_cols)
        self.row_ptr = np.asarray(row_ptr, dtype=np.int64)
        self.col = np.asarray(col, dtype=np.int32)
        self.val = np.asarray(val, dtype=np.float64)


def transition(adj) -> tuple[_Csr, np.ndarray]:
    """Row-scaled adjacency (edge i -> j carries 1 / outdeg(i)) and the dangling mask."""
    deg = np.diff(np.asarray(adj.row_ptr, dtype=np.int64))
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1), 0.0)
    return _Csr(adj.n_rows, adj.n_cols, adj.row_ptr, adj.col, np.repeat(inv, deg)), deg == 0


def pagerank(adj, d: float = 0.85, tol: float = 1e-12, max_iter: int = 200, kernel: int = api.KERNEL_S,
             check_every: int = 4):
    """Ranks (numpy, sum 1), iterations run and the final L1 change."""
    import torch

    if adj.n_rows != adj.n_cols:
        raise ValueError("PageRank needs a square adjacency matrix")
    n = adj.n_rows
    P, dangling = transition(adj)
    plan = api.Plan(P, kernel=kernel, transpose=True)
    dev = torch.device("cuda", torch.cuda.current_device())
    dmask = torch.from_numpy(dangling.astype(np.float64)).to(dev)
    r = torch.full((n,), 1.0 / n, dtype=torch.float64, device=dev)
    y = torch.empty_like(r)
    scal = torch.zeros(2, dtype=torch.float64, device=dev)  # [dangling mass, L1 distance]
    part = torch.empty(api.DOT_BLOCKS, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    delta = float("inf")
    it = 0
    try:
        for it in range(1, max_iter + 1):
            api.dot(n, r.data_ptr(), dmask.data_ptr(), 0, part.data_ptr(), scal.data_ptr(), stream)
            plan.mxv_axpbyg(r.data_ptr(), y.data_ptr(), alpha=d, gamma=(1.0 - d) / n, d_g=scal.data_ptr(),
                            g_scale=d / n, stream=stream)
            if it % check_every == 0 or it == max_iter:
                api.dot(n, y.data_ptr(), r.data_ptr(), 1, part.data_ptr(), scal.data_ptr() + 8, stream)
                delta = float(scal[1].item())
                r, y = y, r
                if delta < tol:
                    break
            else:
                r, y = y, r
        plan.device_status(stream)
    finally:
        plan.free()
    return r.cpu().numpy(), it, delta
