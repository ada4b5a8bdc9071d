"""Synthetic matrix generators and real-matrix readers (host only)."""
from __future__ import annotations

import os

import numpy as np
import pytest


def check_csr(m, sorted_unique=True):
    rp = m.row_ptr
    assert rp[0] == 0 and np.all(np.diff(rp) >= 0) and rp[-1] == m.nnz
    assert m.col.shape[0] >= m.nnz
    if m.nnz:
        assert m.col[: m.nnz].min() >= 0 and m.col[: m.nnz].max() < m.n_cols
    if sorted_unique and m.nnz:
        rows = np.repeat(np.arange(m.n_rows), np.diff(rp))
        same = rows[1:] == rows[:-1]
        assert np.all(np.diff(m.col[: m.nnz].astype(np.int64))[same] > 0)


def test_uniform_k(built):
    from vnec_gb300 import generators as G

    m = G.uniform_k(5000, 16, seed=0)
    check_csr(m)
    assert m.nnz == 5000 * 16 and np.all(np.diff(m.row_ptr) == 16)
    assert -1.0 <= m.val.min() and m.val.max() < 1.0
    m2 = G.uniform_k(5000, 16, seed=0)
    assert np.array_equal(m.col, m2.col) and np.array_equal(m.val, m2.val)
    m3 = G.uniform_k(5000, 16, seed=1)
    assert not np.array_equal(m.col, m3.col)


def test_rmat_dedup_and_skew(built):
    from vnec_gb300 import generators as G

    m = G.rmat(14, 16 << 14, seed=1)
    check_csr(m)
    assert m.n_rows == 1 << 14 and m.nnz <= 16 << 14 and m.nnz > 12 << 14
    lens = np.diff(m.row_ptr)
    assert lens[:64].mean() > 10 * lens.mean()  # low ids are hubs (no relabelling)
    assert np.all((m.val >= 0) & (m.val < 1))


def test_stencil27(built):
    from vnec_gb300 import generators as G

    g = 9
    m = G.stencil27(g, seed=0)
    check_csr(m)
    assert m.nnz == (3 * g - 2) ** 3
    d = m.to_dense()
    assert np.allclose(np.diag(d), 1.0 + np.abs(d - np.diag(np.diag(d))).sum(axis=1))
    off = d - np.diag(np.diag(d))
    assert off.max() <= 0.0 and off.min() > -1.0


def test_lognormal_banded_blockdiag(built):
    from vnec_gb300 import generators as G

    m = G.lognormal(20000, seed=3)
    check_csr(m)
    lens = np.diff(m.row_ptr)
    assert lens.max() <= 4096 and 15 < lens.mean() < 35
    b = G.banded(1000, 9, seed=4)
    check_csr(b)
    assert b.nnz == 1000 * 9 - 2 * (4 + 3 + 2 + 1)
    k = G.blockdiag(100, 16, seed=5)
    check_csr(k)
    assert k.nnz == 6 * 16 * 16 + 4 * 4


def test_vector_and_kat(built):
    from vnec_gb300 import generators as G

    x = G.vector(1000, seed=2)
    assert x.shape == (1000,) and -1 <= x.min() and x.max() < 1
    assert np.array_equal(x, G.vector(1000, seed=2))
    m = G.uniform_k(100, 4, seed=1)
    kat, xk = G.kat_values(m)
    assert np.array_equal(xk, np.arange(100.0))
    assert np.all(kat.val == np.repeat(np.arange(100.0), 4))


def test_mtx_and_sg_round_trip(built, tmp_path):
    from vnec_gb300 import generators as G
    from vnec_gb300 import mtxio

    p = tmp_path / "a.mtx"
    p.write_text("%%MatrixMarket matrix coordinate real symmetric\n% c\n4 4 4\n1 1 2.0\n3 1 -1.5\n4 2 3.0\n4 4 1.0\n")
    m = mtxio.read_mtx(str(p))
    d = m.to_dense()
    want = np.zeros((4, 4))
    want[0, 0], want[2, 0], want[0, 2], want[3, 1], want[1, 3], want[3, 3] = 2.0, -1.5, -1.5, 3.0, 3.0, 1.0
    assert np.array_equal(d, want)
    g = G.rmat(8, 2000, seed=3).copy()
    sg = tmp_path / "g.sg"
    mtxio.write_sg(str(sg), g, directed=True)
    r = mtxio.read_sg(str(sg))
    assert np.array_equal(r.row_ptr, g.row_ptr) and np.array_equal(r.col, g.col)
    assert np.array_equal(r.val, np.repeat(np.arange(g.n_rows, dtype=np.float64), np.diff(g.row_ptr)))
