"""Training data of the learned kernel selection.

Seeded synthetic FP64 matrices from a generator mix — uniform random, R-MAT
(a in [0.45, 0.65]), banded (bandwidth 3-257), block-diagonal with dense
8x8-64x64 blocks and lognormal row lengths (sigma in [0.5, 3]) — with row
counts log-uniform in [1e4, 4e6] (reduced where a matrix would exceed
MAX_NNZ nonzeros), and large records (seeds from LARGE_FIRST: 4e6 - 1.7e7
rows, R-MAT up to scale 24, 27-point stencils up to 256^3).  Each record
holds the 16 features (GPU feature kernel),
the exhaustive autotuner's median time of every configuration on this GPU,
the reference rule's choice and the algorithmic bytes of one SpMV.

    python -m vnec_gb300.tuner.dataset --first 0 --count 800 --out shard0.npz
"""
from __future__ import annotations

import argparse
import math
import time

import numpy as np

from .. import api
from .. import generators as G

FAMILIES = ("uniform", "rmat", "banded", "blockdiag", "lognormal", "stencil")
MAX_NNZ = 60_000_000
ROWS_LO, ROWS_HI = 1e4, 4e6
# Records with seed >= LARGE_FIRST: large matrices (4e6 - 1.7e7 rows, up to
# LARGE_MAX_NNZ nonzeros: R-MAT scale 22-24, 27-point stencils, uniform,
# banded, lognormal), so that workloads of the headline size lie inside the
# trained feature range.
LARGE_FIRST = 3000
LARGE_MAX_NNZ = 300_000_000
LARGE_ROWS_LO, LARGE_ROWS_HI = 4e6, 1.7e7


def _loguni(rng, lo, hi):
    return math.exp(rng.uniform(math.log(lo), math.log(hi)))


def sample_large(seed: int):
    rng = np.random.default_rng([seed, 0x1A26E])
    fam = ("rmat", "stencil", "uniform", "banded", "lognormal")[seed % 5]
    n = int(_loguni(rng, LARGE_ROWS_LO, LARGE_ROWS_HI))
    gseed = 1000 + seed
    if fam == "rmat":
        a = rng.uniform(0.5, 0.6)
        b = c = (0.95 - a) / 2
        scale = 22 + (seed // 5) % 3  # 22, 23, 24 in turn
        deg = rng.uniform(8, 17)
        m = G.rmat(scale, int(min(LARGE_MAX_NNZ, deg * (1 << scale))), a, b, c, lo=0.0, hi=1.0, seed=gseed)
        desc = f"rmat scale={scale} a={a:.3f} deg={deg:.1f}"
    elif fam == "stencil":
        g = int(round(n ** (1.0 / 3.0)))
        m = G.stencil27(g, seed=gseed)
        desc = f"stencil27 g={g}"
    elif fam == "uniform":
        k = int(rng.integers(4, 25))
        m = G.uniform_k(min(n, LARGE_MAX_NNZ // k), k, seed=gseed)
        desc = f"uniform k={k}"
    elif fam == "banded":
        bw = int(round(_loguni(rng, 3, 63))) | 1
        m = G.banded(min(n, LARGE_MAX_NNZ // bw), bw, seed=gseed)
        desc = f"banded bw={bw}"
    else:
        sigma = rng.uniform(0.5, 1.5)
        mean_len = 8.0 * math.exp(sigma * sigma / 2)
        m = G.lognormal(int(min(n, LARGE_MAX_NNZ / mean_len)), sigma=sigma, cap=4096, seed=gseed)
        desc = f"lognormal sigma={sigma:.2f}"
    return m, fam, desc


def sample(seed: int):
    """The matrix of record `seed` and a short description."""
    if seed >= LARGE_FIRST:
        return sample_large(seed)
    rng = np.random.default_rng([seed, 0x7E57])
    fam = FAMILIES[seed % 5]
    n = int(_loguni(rng, ROWS_LO, ROWS_HI))
    gseed = 1000 + seed
    if fam == "uniform":
        k = max(2, int(round(_loguni(rng, 2, 48))))
        n = min(n, MAX_NNZ // k)
        m = G.uniform_k(n, k, seed=gseed)
        desc = f"uniform k={k}"
    elif fam == "rmat":
        a = rng.uniform(0.45, 0.65)
        b = c = (0.95 - a) / 2
        scale = int(min(22, max(14, round(math.log2(n)))))
        deg = rng.uniform(4, 24)
        edges = int(min(MAX_NNZ, deg * (1 << scale)))
        m = G.rmat(scale, edges, a, b, c, lo=-1.0, hi=1.0, seed=gseed)
        desc = f"rmat scale={scale} a={a:.3f} deg={deg:.1f}"
    elif fam == "banded":
        bw = int(round(_loguni(rng, 3, 257))) | 1
        n = min(n, MAX_NNZ // bw)
        m = G.banded(n, bw, seed=gseed)
        desc = f"banded bw={bw}"
    elif fam == "blockdiag":
        bs = int(round(_loguni(rng, 8, 64)))
        n = min(n, MAX_NNZ // bs)
        m = G.blockdiag(n, bs, seed=gseed)
        desc = f"blockdiag bs={bs}"
    else:
        sigma = rng.uniform(0.5, 3.0)
        mean_len = min(4096.0, 8.0 * math.exp(sigma * sigma / 2))
        n = int(min(n, MAX_NNZ / mean_len))
        n = max(n, int(ROWS_LO))
        m = G.lognormal(n, sigma=sigma, cap=4096, seed=gseed)
        desc = f"lognormal sigma={sigma:.2f}"
    return m, fam, desc


def algorithmic_bytes(m) -> int:
    return m.nnz * 12 + (m.n_rows + 1) * 4 + m.n_cols * 8 + m.n_rows * 8


def record(seed: int, reps: int = 5) -> dict:
    m, fam, desc = sample(seed)
    f = api.features(m)
    ms, best = api.autotune(m, reps=reps)
    rule = api.rule_choice(m)
    r = dict(seed=seed, family=FAMILIES.index(fam), n_rows=m.n_rows, nnz=m.nnz, features=f, ms=ms, best=best,
             rule=rule, bytes=algorithmic_bytes(m), desc=desc)
    m.free()
    return r


def build_shard(first: int, count: int, out: str, reps: int = 5, budget_s: float | None = None) -> int:
    recs = []
    t0 = time.time()
    for s in range(first, first + count):
        recs.append(record(s, reps))
        if budget_s is not None and time.time() - t0 > budget_s:
            break
    np.savez_compressed(
        out, seed=np.array([r["seed"] for r in recs], dtype=np.int64),
        family=np.array([r["family"] for r in recs], dtype=np.int8),
        n_rows=np.array([r["n_rows"] for r in recs], dtype=np.int64),
        nnz=np.array([r["nnz"] for r in recs], dtype=np.int64),
        features=np.stack([r["features"] for r in recs]).astype(np.float32),
        ms=np.stack([r["ms"] for r in recs]).astype(np.float64),
        best=np.array([r["best"] for r in recs], dtype=np.int16),
        rule=np.array([r["rule"] for r in recs], dtype=np.int16),
        bytes=np.array([r["bytes"] for r in recs], dtype=np.int64),
        desc=np.array([r["desc"] for r in recs]))
    return len(recs)


def load(paths) -> dict:
    """Concatenation of shards, ordered by seed."""
    parts = [dict(np.load(p)) for p in paths]
    d = {k: np.concatenate([p[k] for p in parts]) for k in parts[0]}
    order = np.argsort(d["seed"], kind="stable")
    return {k: v[order] for k, v in d.items()}


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--first", type=int, default=0)
    ap.add_argument("--count", type=int, default=100)
    ap.add_argument("--out", required=True)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--budget-s", type=float, default=None, help="stop early after this many seconds")
    a = ap.parse_args()
    t0 = time.time()
    n = build_shard(a.first, a.count, a.out, a.reps, a.budget_s)
    print(f"{n} records in {time.time() - t0:.1f} s -> {a.out}", flush=True)


if __name__ == "__main__":
    main()
