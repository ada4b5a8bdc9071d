"""Device-resident chains on the mxv path: the fused output transform
y := alpha A x + beta z + gamma (SpB_mxv_axpby_ext) for every kernel, with z
absent, separate and aliasing y, and a PageRank power iteration against a
NumPy power iteration on the same graph."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kernel", ["L", "S", "D", "HYBRID", "S_FP32FORM", "PUSH"])
def test_axpby_epilogue(built, kernel):
    import torch

    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    if kernel == "S_FP32FORM":
        kw = dict(kernel=api.KERNEL_S, precision=api.PREC_FP32)
    else:
        kw = dict(kernel=getattr(api, "KERNEL_" + kernel))
    tol = 1e-6 if kernel == "S_FP32FORM" else 1e-12
    rng = np.random.default_rng(3)
    for m in (G.rmat(14, 8 << 14, seed=4), G.lognormal(7000, sigma=2.2, cap=3000, seed=2)):
        p = api.Plan(m, long_row_len=64, **kw)
        xv = rng.uniform(-1, 1, m.n_cols)
        zv = rng.uniform(-1, 1, m.n_rows)
        ax, cond = O.spmv_neumaier(m, xv)
        x = torch.from_numpy(xv).cuda()
        for alpha, beta, gamma, mode in ((0.85, 0.0, 0.3, "none"), (-2.0, 0.5, 0.0, "sep"), (1.5, -1.0, 0.25, "alias")):
            y = torch.from_numpy(zv.copy()).cuda() if mode == "alias" else torch.full((m.n_rows,), np.nan,
                                                                                       dtype=torch.float64,
                                                                                       device="cuda")
            z = torch.from_numpy(zv).cuda()
            d_z = {"none": 0, "sep": z.data_ptr(), "alias": y.data_ptr()}[mode]
            p.mxv_axpby(x.data_ptr(), y.data_ptr(), alpha, beta, d_z, gamma)
            torch.cuda.synchronize()
            want = alpha * ax + (beta * zv if mode != "none" else 0.0) + gamma
            err = np.abs(y.cpu().numpy() - want)
            bound = tol * (abs(alpha) * cond + abs(beta) * np.abs(zv) + abs(gamma)) + 1e-15
            assert np.all(err <= bound), (kernel, mode, float(np.max(err / bound)))
        p.free()


def _pagerank_reference(adj, d=0.85, iters=200):
    """Plain NumPy power iteration (float64) on the same graph."""
    n = adj.n_rows
    rp = np.asarray(adj.row_ptr)
    col = np.asarray(adj.col)
    deg = np.diff(rp)
    src = np.repeat(np.arange(n), deg)
    dangling = deg == 0
    r = np.full(n, 1.0 / n)
    for _ in range(iters):
        contrib = r[src] / deg[src]
        y = np.bincount(col, weights=contrib, minlength=n)
        y = d * y + ((1 - d) + d * r[dangling].sum()) / n
        if np.abs(y - r).sum() < 1e-14:
            r = y
            break
        r = y
    return r


@pytest.mark.parametrize("kernel", ["S", "L"])
def test_pagerank_chain(built, kernel):
    from vnec_gb300 import api
    from vnec_gb300 import generators as G
    from vnec_gb300.pagerank import pagerank

    adj = G.rmat(15, 10 << 15, seed=6)
    ranks, iters, delta = pagerank(adj, tol=1e-13, kernel=getattr(api, "KERNEL_" + kernel))
    ref = _pagerank_reference(adj)
    assert delta < 1e-13 and iters < 200
    assert abs(ranks.sum() - 1.0) < 1e-12
    assert np.abs(ranks - ref).sum() < 1e-11


@pytest.mark.parametrize("n", [0, 1, 777, 1 << 20, (1 << 21) + 5])
def test_device_dot_and_l1_distance(built, n):
    """SpB_VNEC_dot_ext: sum a*b and sum |a - b| in a fixed order (identical
    bits on repeated calls), within 1e-12 of the sums' magnitudes."""
    import torch

    from vnec_gb300 import api

    rng = np.random.default_rng(n)
    a, b = rng.uniform(-1, 1, n), rng.uniform(-1, 1, n)
    da, db = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    part = torch.empty(api.DOT_BLOCKS, dtype=torch.float64, device="cuda")
    out = torch.full((2,), float("nan"), dtype=torch.float64, device="cuda")
    for mode, want, scale in ((0, float(np.dot(a, b)), float(np.abs(a * b).sum())),
                              (1, float(np.abs(a - b).sum()), float(np.abs(a - b).sum()))):
        got = []
        for _ in range(2):
            api.dot(n, da.data_ptr(), db.data_ptr(), mode, part.data_ptr(), out.data_ptr() + 8 * mode)
            torch.cuda.synchronize()
            got.append(float(out[mode].item()))
        assert got[0] == got[1]
        assert abs(got[0] - want) <= 1e-12 * scale + 1e-300


@pytest.mark.parametrize("kernel", ["L", "S", "S_FP32FORM", "HYBRID"])
def test_axpby_with_device_scalar(built, kernel):
    """SpB_mxv_axpbyg_ext: y = alpha A x + beta z + gamma + s * (*d_g), the
    scalar read on the device, fused or as the elementwise pass."""
    import torch

    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    kw = dict(kernel=api.KERNEL_S, precision=api.PREC_FP32) if kernel == "S_FP32FORM" else dict(
        kernel=getattr(api, "KERNEL_" + kernel))
    tol = 1e-6 if kernel == "S_FP32FORM" else 1e-12
    m = G.rmat(14, 8 << 14, seed=4)
    rng = np.random.default_rng(5)
    xv, zv = rng.uniform(-1, 1, m.n_cols), rng.uniform(-1, 1, m.n_rows)
    ax, cond = O.spmv_neumaier(m, xv)
    p = api.Plan(m, long_row_len=64, **kw)
    try:
        x, z = torch.from_numpy(xv).cuda(), torch.from_numpy(zv).cuda()
        g = torch.tensor([0.375], dtype=torch.float64, device="cuda")
        y = torch.full((m.n_rows,), float("nan"), dtype=torch.float64, device="cuda")
        p.mxv_axpbyg(x.data_ptr(), y.data_ptr(), 0.85, -0.5, z.data_ptr(), 0.1, g.data_ptr(), 2.0)
        torch.cuda.synchronize()
        want = 0.85 * ax - 0.5 * zv + 0.1 + 2.0 * 0.375
        bound = tol * (0.85 * cond + 0.5 * np.abs(zv) + 0.85) + 1e-15
        assert np.all(np.abs(y.cpu().numpy() - want) <= bound)
    finally:
        p.free()
