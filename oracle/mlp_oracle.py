"""NumPy restatement of the learned kernel selection — TEST INFRASTRUCTURE ONLY.

The checker for the library's GPU feature kernel (``features.cu``) and its
MLP forward / backward kernels (``mlp.cu``): the same 16 features and the
same 16 -> 64 -> 64 -> C ReLU network with masked mean-squared-error loss,
computed in float64.  Only the tests use this module.
"""
from __future__ import annotations

import numpy as np

F, H = 16, 64


def features(n_rows: int, n_cols: int, row_ptr, col) -> np.ndarray:
    """The 16 features of tuner.h from CSR arrays (see matrix_features_device)."""
    rp = np.asarray(row_ptr, dtype=np.int64)
    ci = np.asarray(col, dtype=np.int64)
    nnz = int(rp[-1])
    lens = np.diff(rp)
    nr = max(n_rows, 1)
    mean = nnz / nr
    var = max(0.0, float(np.sum(lens.astype(np.float64) ** 2)) / nr - mean * mean)
    cv = np.sqrt(var) / mean if mean > 0 else 0.0
    f = np.zeros(F)
    f[0] = np.log2(n_rows + 1.0) / 24
    f[1] = np.log2(n_cols + 1.0) / 24
    f[2] = np.log2(nnz + 1.0) / 32
    f[3] = np.log2(mean + 1.0) / 12
    f[4] = min(cv, 8.0) / 8
    f[5] = np.log2((lens.max() if n_rows else 0) + 1.0) / 16
    bins = [(0, 1), (1, 4), (4, 16), (16, 64), (64, 1024), (1024, 1 << 62)]
    for i, (lo, hi) in enumerate(bins):
        f[6 + i] = np.sum((lens >= lo) & (lens < hi)) / nr
    ne = lens > 0
    n_ne = max(int(ne.sum()), 1)
    if nnz:
        starts = rp[:-1][ne]
        ends = rp[1:][ne]
        mn = np.minimum.reduceat(ci, starts)
        mx = np.maximum.reduceat(ci, starts)
        f[12] = min(1.0, float(np.sum((mx - mn + 1) / n_cols)) / n_ne)
        row_of = np.repeat(np.arange(n_rows), lens)
        first = np.zeros(nnz, dtype=bool)
        first[rp[:-1][ne]] = True
        newblk = first.copy()
        newblk[1:] |= (ci[1:] >> 2) != (ci[:-1] >> 2)
        blocks_per_row = np.bincount(row_of[newblk], minlength=n_rows)
        total_blocks = int(blocks_per_row.sum())
        f[13] = min(1.0, nnz / (4.0 * total_blocks)) if total_blocks else 0.0
        dense = ne & (lens >= 2 * blocks_per_row)
        f[14] = min(1.0, dense.sum() / n_ne)
        cnt = np.bincount(ci, minlength=n_cols)
        thr = max(1.0, np.ceil(8.0 * nnz / n_cols))
        f[15] = min(1.0, cnt[cnt >= thr].sum() / nnz)
    return f.astype(np.float32)


def unpack(p: np.ndarray, c: int):
    p = np.asarray(p, dtype=np.float64)
    i = 0
    out = []
    for shape in ((H, F), (H,), (H, H), (H,), (c, H), (c,)):
        n = int(np.prod(shape))
        out.append(p[i:i + n].reshape(shape))
        i += n
    assert i == p.size
    return out


def forward(p: np.ndarray, X: np.ndarray, c: int):
    W1, b1, W2, b2, W3, b3 = unpack(p, c)
    X = np.asarray(X, dtype=np.float64)
    H1 = np.maximum(X @ W1.T + b1, 0.0)
    H2 = np.maximum(H1 @ W2.T + b2, 0.0)
    return H1, H2, H2 @ W3.T + b3


def loss_grad(p: np.ndarray, X, T, M, c: int) -> tuple[float, np.ndarray]:
    """Masked MSE sum(M (O - T)^2) / sum(M) and its gradient w.r.t. the flat parameters."""
    W1, b1, W2, b2, W3, b3 = unpack(p, c)
    X = np.asarray(X, dtype=np.float64)
    T = np.asarray(T, dtype=np.float64)
    M = np.asarray(M, dtype=np.float64)
    H1, H2, O = forward(p, X, c)
    ms = max(M.sum(), 1.0)
    d = (O - T) * M
    loss = float(np.sum(d * d) / ms)
    dO = 2.0 * d / ms
    gW3, gb3 = dO.T @ H2, dO.sum(0)
    dH2 = (dO @ W3) * (H2 > 0)
    gW2, gb2 = dH2.T @ H1, dH2.sum(0)
    dH1 = (dH2 @ W2) * (H1 > 0)
    gW1, gb1 = dH1.T @ X, dH1.sum(0)
    return loss, np.concatenate([g.ravel() for g in (gW1, gb1, gW2, gb2, gW3, gb3)])
