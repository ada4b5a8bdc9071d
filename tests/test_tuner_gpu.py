"""GPU checks of the learned kernel selection, through the C ABI.

- the feature kernel against the NumPy feature oracle;
- the MLP forward pass and gradient against the NumPy oracle (float64);
- training with the library's kernels: loss decreases, runs are reproducible;
- the exhaustive autotuner, and plans built by kernel SEARCH / RULE / LEARNED
  against the FP64 oracle;
- on the committed timing dataset: a network trained here by the library's
  kernels has held-out regret <= 10 % against the exhaustive search, and beats
  the reference's rule-based choice (the method without the learned part).
"""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import ROOT, Csr

pytestmark = pytest.mark.gpu

C = 15


def _mats():
    from vnec_gb300 import generators as G

    return [G.rmat(15, 12 << 15, seed=3), G.uniform_k(20000, 9, seed=1), G.banded(30000, 17, seed=2),
            G.blockdiag(20000, 16, seed=4), G.lognormal(15000, sigma=2.5, cap=4096, seed=5)]


def test_features_kernel_matches_oracle(built):
    from oracle import mlp_oracle as MO
    from vnec_gb300 import api

    mats = _mats()
    # unsorted columns and a rectangular shape
    rng = np.random.default_rng(3)
    rp = np.concatenate([[0], np.cumsum(rng.integers(0, 40, 500))])
    col = rng.integers(0, 3000, rp[-1]).astype(np.int32)
    mats.append(Csr(500, 3000, rp, col, rng.uniform(-1, 1, rp[-1])))
    for m in mats:
        f = api.features(m)
        ref = MO.features(m.n_rows, m.n_cols, m.row_ptr, m.col)
        assert np.allclose(f, ref, atol=2e-6, rtol=1e-5), (f, ref)


def _batch(seed, n=37):
    rng = np.random.default_rng(seed)
    X = rng.uniform(0, 1, (n, 16)).astype(np.float32)
    T = rng.uniform(0, 4, (n, C)).astype(np.float32)
    M = (rng.uniform(0, 1, (n, C)) > 0.15).astype(np.float32)
    return X, T, M


def test_mlp_forward_and_gradient_match_oracle(built):
    from oracle import mlp_oracle as MO
    from vnec_gb300 import api

    net = api.Mlp(seed=11)
    try:
        p = net.params
        X, T, M = _batch(1)
        _, _, O = MO.forward(p, X, C)
        assert np.allclose(net.predict(X), O, rtol=1e-5, atol=1e-5)
        loss, g = net.loss_grad(X, T, M)
        loss_ref, g_ref = MO.loss_grad(p, X, T, M, C)
        assert loss == pytest.approx(loss_ref, rel=1e-5)
        scale = np.abs(g_ref).max()
        assert np.allclose(g, g_ref, rtol=1e-4, atol=1e-5 * scale)
        # parameters round-trip
        q = np.random.default_rng(2).normal(0, 0.1, p.size).astype(np.float32)
        net.params = q
        assert np.array_equal(net.params, q)
    finally:
        net.free()


def test_mlp_training_reduces_loss_and_is_reproducible(built):
    from vnec_gb300 import api

    rng = np.random.default_rng(5)
    X = rng.uniform(0, 1, (300, 16)).astype(np.float32)
    # a learnable target: each output a fixed random function of the features
    W = rng.normal(0, 1, (16, C))
    T = np.maximum(X @ W, 0).astype(np.float32)
    M = np.ones_like(T)
    runs = []
    for _ in range(2):
        net = api.Mlp(seed=3)
        curve = net.train(X, T, M, epochs=60, batch=32, lr=3e-3, seed=9)
        runs.append((curve, net.params))
        net.free()
    curve = runs[0][0]
    assert curve[-1] < 0.1 * curve[0]
    assert np.array_equal(runs[0][1], runs[1][1]) and np.array_equal(runs[0][0], runs[1][0])


def test_autotune_times_every_configuration(built):
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    cfg = api.tune_configs()
    assert len(cfg) == C
    m = G.banded(40000, 9, seed=2)
    ms, best = api.autotune(m, reps=3)
    assert np.all(np.isfinite(ms)) and best == int(np.argmin(ms))
    # unsorted columns: only the merge-path and the pure sliced configurations exist
    rng = np.random.default_rng(1)
    rp = np.arange(0, 4 * 5001, 4)
    col = rng.integers(0, 5000, rp[-1]).astype(np.int32)
    u = Csr(5000, 5000, rp, col, rng.uniform(-1, 1, rp[-1]))
    ms, best = api.autotune(u, reps=2)
    for i, (k, chunk, permille) in enumerate(cfg):
        assert np.isfinite(ms[i]) == (k == api.KERNEL_L or permille > 1000), (i, cfg[i])


@pytest.mark.parametrize("kernel", ["SEARCH", "RULE", "LEARNED"])
def test_tuned_plans_are_correct(built, kernel):
    from oracle import oracle as O
    from vnec_gb300 import api
    from vnec_gb300 import generators as G

    k = getattr(api, "KERNEL_" + kernel)
    for m in _mats()[:3]:
        xv = G.vector(m.n_cols, seed=4)
        p = api.Plan(m, kernel=k)
        cfg, how = api.plan_choice(p)
        assert 0 <= cfg < C
        if kernel == "SEARCH":
            assert how == api.CHOSEN_SEARCH
        elif kernel == "RULE":
            assert how == api.CHOSEN_RULE and cfg == api.rule_choice(m)
        else:
            assert how in (api.CHOSEN_LEARNED, api.CHOSEN_FALLBACK)
            if api.builtin_model() is None:
                assert how == api.CHOSEN_FALLBACK
        y = p.mxv_host(xv)
        y_ref, cond = O.spmv_neumaier(m, xv)
        assert np.all(np.abs(y - y_ref) <= 1e-12 * cond)
        p.free()


def _shards():
    return sorted(glob.glob(os.path.join(ROOT, "vnec_gb300", "tuner", "data", "*.npz")))


@pytest.mark.skipif(not _shards(), reason="no timing dataset committed")
def test_learned_selection_regret_and_gain(built):
    """Train on the committed GB300 timings with the library's kernels; held-out
    regret against the exhaustive autotune <= 10 %; the learned choice beats
    the reference's rule-based choice (and the best single fixed
    configuration) on the held-out matrices."""
    from vnec_gb300.tuner import dataset as DS
    from vnec_gb300.tuner import train as TR

    d = DS.load(_shards())
    tr, ho = TR.split(d)
    T, M = TR.targets(tr["ms"])
    net, curve = TR.train_model(tr["features"], T, M)
    try:
        assert curve[-1] < curve[0]
        rep = TR.evaluate(net, ho)
    finally:
        net.free()
    assert rep["n"] >= 200
    assert rep["learned"]["mean_regret"] <= 0.10, rep
    assert rep["learned"]["mean_regret"] < rep["rule"]["mean_regret"], rep
    assert rep["geomean_speedup_learned_over_rule"] > 1.0, rep
    fixed = TR.summary(np.full(len(ho["seed"]), TR.best_fixed_config(tr)), ho["ms"], ho["bytes"])
    assert rep["learned"]["mean_regret"] < fixed["mean_regret"], (rep, fixed)


@pytest.mark.skipif(not _shards(), reason="no timing dataset committed")
def test_builtin_model_regret(built):
    """The model compiled into the library chooses with <= 10 % mean held-out regret."""
    from vnec_gb300 import api
    from vnec_gb300.tuner import dataset as DS
    from vnec_gb300.tuner import train as TR

    bm = api.builtin_model()
    if bm is None:
        pytest.skip("library built without a trained model")
    params, _ = bm
    d = DS.load(_shards())
    _, ho = TR.split(d)
    net = api.Mlp()
    try:
        net.params = params
        rep = TR.evaluate(net, ho)
    finally:
        net.free()
    assert rep["learned"]["mean_regret"] <= 0.10, rep
