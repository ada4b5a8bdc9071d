"""Training of the learned kernel selection with the library's GPU kernels.

The targets are the exhaustive autotuner's timings: for matrix i and
configuration c, T[i, c] = log2(ms[i, c] / min_c ms[i, c]) (clipped at
T_CAP; configurations that cannot be built are masked out).  The MLP
(16 -> 64 -> 64 -> C, FP32) is trained with Adam on masked squared error by
the library's forward/backward/update kernels; its choice for a matrix is
the configuration with the lowest predicted cost.  Records with seed < 2000
and three of every four large records train; seeds 2000-2199 and the other
large records are held out; regret = ms[choice] / ms[best] - 1.

    python -m vnec_gb300.tuner.train --data shard*.npz --weights tuner_weights.inc --report report.json
"""
from __future__ import annotations

import argparse
import glob
import json

import numpy as np

from .. import api
from . import dataset

N_TRAIN = 2000
T_CAP = 6.0
TRAIN_DEFAULTS = dict(epochs=400, batch=64, lr=2e-3, weight_decay=1e-4, seed=1)


def targets(ms: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    M = np.isfinite(ms)
    best = np.where(M, ms, np.inf).min(axis=1, keepdims=True)
    T = np.where(M, np.log2(np.where(M, ms, 1.0) / best), 0.0)
    return np.minimum(T, T_CAP).astype(np.float32), M.astype(np.float32)


def choose(pred: np.ndarray, ms: np.ndarray) -> np.ndarray:
    p = np.where(np.isfinite(ms), pred, np.inf)
    return np.argmin(p, axis=1)


def regret(choice: np.ndarray, ms: np.ndarray) -> np.ndarray:
    best = np.where(np.isfinite(ms), ms, np.inf).min(axis=1)
    return ms[np.arange(len(ms)), choice] / best - 1.0


def summary(choice: np.ndarray, ms: np.ndarray, nbytes: np.ndarray) -> dict:
    r = regret(choice, ms)
    t = ms[np.arange(len(ms)), choice]
    return {"mean_regret": float(r.mean()), "median_regret": float(np.median(r)),
            "p90_regret": float(np.quantile(r, 0.9)), "max_regret": float(r.max()),
            "optimal_fraction": float(np.mean(r <= 1e-9)),
            "aggregate_gbs": float(nbytes.sum() / (t.sum() / 1e3) / 1e9),
            "mean_gbs": float(np.mean(nbytes / (t / 1e3) / 1e9))}


def split(d: dict):
    """(training, held-out) records: seeds below N_TRAIN and three of every four
    large records train."""
    s = d["seed"]
    large = s >= dataset.LARGE_FIRST
    tr = (s < N_TRAIN) | (large & ((s - dataset.LARGE_FIRST) % 4 != 3))
    return {k: v[tr] for k, v in d.items()}, {k: v[~tr] for k, v in d.items()}


def train_model(X, T, M, **kw) -> tuple[api.Mlp, np.ndarray]:
    p = dict(TRAIN_DEFAULTS)
    p.update(kw)
    model = api.Mlp(seed=p.pop("seed"))
    curve = model.train(X, T, M, seed=7, **p)
    return model, curve


def evaluate(model: api.Mlp, d: dict) -> dict:
    pred = model.predict(d["features"])
    learned = choose(pred, d["ms"])
    out = {"learned": summary(learned, d["ms"], d["bytes"]),
           "rule": summary(d["rule"].astype(np.int64), d["ms"], d["bytes"]),
           "exhaustive": summary(choose(d["ms"], d["ms"]), d["ms"], d["bytes"])}
    rt = d["ms"][np.arange(len(learned)), d["rule"].astype(np.int64)]
    lt = d["ms"][np.arange(len(learned)), learned]
    out["geomean_speedup_learned_over_rule"] = float(np.exp(np.mean(np.log(rt / lt))))
    out["n"] = int(len(learned))
    return out


def best_fixed_config(d: dict) -> int:
    """The single configuration with the lowest total time over `d` (a learned-free baseline)."""
    ms = np.where(np.isfinite(d["ms"]), d["ms"], 1e9)
    return int(np.argmin(ms.sum(axis=0)))


def write_weights(path: str, params: np.ndarray, frange: np.ndarray, note: str) -> None:
    def arr(a):
        vals = ", ".join(f"{float(v):.9e}f" for v in np.asarray(a, dtype=np.float32).ravel())
        return "{" + vals + "}"

    with open(path, "w") as f:
        f.write("// Generated by vnec_gb300/tuner/train.py: parameters of the built-in kernel\n")
        f.write("// selection model and the feature range (min, max per feature) of its\n")
        f.write(f"// training set.  {note}\n")
        f.write("static const int kHaveModel = 1;\n")
        f.write(f"static const float kModelParams[{params.size}] = {arr(params)};\n")
        f.write(f"static const float kFeatureRange[{frange.size}] = {arr(frange)};\n")


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--data", nargs="+", required=True)
    ap.add_argument("--weights", default=None, help="write the trained model as a C include file")
    ap.add_argument("--report", default=None)
    ap.add_argument("--epochs", type=int, default=TRAIN_DEFAULTS["epochs"])
    a = ap.parse_args()
    paths = sorted(p for pat in a.data for p in glob.glob(pat))
    d = dataset.load(paths)
    tr, ho = split(d)
    T, M = targets(tr["ms"])
    model, curve = train_model(tr["features"], T, M, epochs=a.epochs)
    frange = np.stack([tr["features"].min(axis=0), tr["features"].max(axis=0)], axis=1)
    fixed = best_fixed_config(tr)
    rep = {"train": evaluate(model, tr), "held_out": evaluate(model, ho),
           "best_fixed_config": fixed,
           "held_out_best_fixed": summary(np.full(len(ho["seed"]), fixed), ho["ms"], ho["bytes"]),
           "loss_first_last": [float(curve[0]), float(curve[-1])], "n_train": int(len(tr["seed"])),
           "n_held_out": int(len(ho["seed"])), "configs": api.tune_configs()}
    print(json.dumps(rep, indent=1))
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    if a.weights:
        h = rep["held_out"]
        write_weights(a.weights, model.params, frange,
                      f"Held-out mean regret {h['learned']['mean_regret']:.4f} over {h['n']} matrices.")


if __name__ == "__main__":
    main()
