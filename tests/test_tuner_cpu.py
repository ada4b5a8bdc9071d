"""CPU checks of the learned kernel selection: the NumPy oracle of the MLP
against finite differences, the feature oracle on hand-computed matrices,
the training-target / regret arithmetic and the committed timing dataset."""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import ROOT

C = 15


def test_mlp_oracle_gradient_matches_finite_differences():
    from oracle import mlp_oracle as MO

    rng = np.random.default_rng(0)
    n_params = 64 * 16 + 64 + 64 * 64 + 64 + C * 64 + C
    p = rng.normal(0, 0.3, n_params)
    X = rng.uniform(0, 1, (7, 16))
    T = rng.uniform(0, 3, (7, C))
    M = (rng.uniform(0, 1, (7, C)) > 0.2).astype(float)
    loss, g = MO.loss_grad(p, X, T, M, C)
    idx = rng.choice(n_params, 60, replace=False)
    eps = 1e-6
    for i in idx:
        q = p.copy()
        q[i] += eps
        lp, _ = MO.loss_grad(q, X, T, M, C)
        q[i] -= 2 * eps
        lm, _ = MO.loss_grad(q, X, T, M, C)
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-5 * max(1.0, abs(fd)), (i, fd, g[i])


def test_feature_oracle_on_hand_matrix():
    from oracle import mlp_oracle as MO

    # 4 x 8: row0 cols 0,1,2,3 (one aligned block), row1 empty, row2 cols 1,5 (two blocks), row3 col 7.
    rp = [0, 4, 4, 6, 7]
    col = [0, 1, 2, 3, 1, 5, 7]
    f = MO.features(4, 8, rp, col)
    lens = np.array([4, 0, 2, 1])
    assert f[0] == pytest.approx(np.log2(5) / 24)
    assert f[2] == pytest.approx(np.log2(8) / 32)
    assert f[3] == pytest.approx(np.log2(7 / 4 + 1) / 12)
    cv = np.sqrt(np.mean(lens ** 2) - (7 / 4) ** 2) / (7 / 4)
    assert f[4] == pytest.approx(cv / 8, rel=1e-6)
    assert f[5] == pytest.approx(np.log2(5) / 16)
    assert f[6:12] == pytest.approx([0.25, 0.5, 0.25, 0, 0, 0])
    assert f[12] == pytest.approx(((4 / 8) + (5 / 8) + (1 / 8)) / 3, rel=1e-6)
    assert f[13] == pytest.approx(7 / (4 * 4))                # blocks: 1 + 2 + 1
    assert f[14] == pytest.approx(1 / 3)                      # only row 0 has len >= 2 * blocks
    # mean column count 7/8 -> threshold 7 uses: no column used 7 times
    assert f[15] == 0.0


def test_targets_choice_and_regret():
    from vnec_gb300.tuner import train as TR

    ms = np.array([[2.0, 1.0, np.inf, 4.0], [1.0, 1.5, 3.0, 200.0]])
    T, M = TR.targets(ms)
    assert M.tolist() == [[1, 1, 0, 1], [1, 1, 1, 1]]
    assert T[0].tolist() == pytest.approx([1.0, 0.0, 0.0, 2.0])
    assert T[1, 3] == TR.T_CAP
    pred = np.array([[0.0, 1.0, -5.0, 3.0], [0.2, 0.1, 0.3, 0.4]])
    ch = TR.choose(pred, ms)
    assert ch.tolist() == [0, 1]        # the unavailable config 2 is never chosen
    assert TR.regret(ch, ms).tolist() == pytest.approx([1.0, 0.5])


def _shards():
    return sorted(glob.glob(os.path.join(ROOT, "vnec_gb300", "tuner", "data", "*.npz")))


@pytest.mark.skipif(not _shards(), reason="no timing dataset committed")
def test_committed_dataset_is_consistent():
    from vnec_gb300.tuner import dataset as DS

    d = DS.load(_shards())
    n = len(d["seed"])
    assert n >= 2200 and len(np.unique(d["seed"])) == n
    assert d["features"].shape == (n, 16) and d["ms"].shape == (n, C)
    assert np.all(np.isfinite(d["features"]))
    fin = np.isfinite(d["ms"])
    assert fin.any(axis=1).all()
    best = np.argmin(np.where(fin, d["ms"], np.inf), axis=1)
    assert np.array_equal(best, d["best"])
    small = d["seed"] < DS.LARGE_FIRST
    assert set(np.unique(d["family"][small])) == set(range(5))
    assert d["n_rows"][small].min() >= 1e4 and d["n_rows"][small].max() <= 4.2e6
    if (~small).any():  # large records: 4e6 - 1.7e7 rows
        assert d["n_rows"][~small].min() >= 3.9e6 and d["n_rows"][~small].max() <= 1.7e7
