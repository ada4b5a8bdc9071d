"""Re-times stored configurations of the tuner's data after a kernel change.

The data shards hold, per matrix, the exhaustive autotuner's time of every
configuration.  When a kernel changes, only the configurations that run it
need new timings: this regenerates each record's matrix from its seed (the
generators are deterministic), times the listed configurations on this GPU
with the autotuner's own protocol (SpB_VNEC_time_configs_ext) and writes the
shard back with those columns, the best index and nothing else replaced.

    python -m vnec_gb300.tuner.refresh --configs 0 --data vnec_gb300/tuner/data/shard*.npz
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from .. import api
from . import dataset


def refresh_shard(path: str, configs: list[int], reps: int = 5, out: str | None = None) -> int:
    d = dict(np.load(path))
    ms = d["ms"].copy()
    t0 = time.time()
    for i, seed in enumerate(d["seed"]):
        m, _, _ = dataset.sample(int(seed))
        assert m.nnz == int(d["nnz"][i]) and m.n_rows == int(d["n_rows"][i]), f"record {seed} changed"
        ms[i, configs] = api.time_configs(m, configs, reps=reps)
        m.free()
    d["ms"] = ms
    d["best"] = np.where(np.isfinite(ms), ms, np.inf).argmin(axis=1).astype(np.int16)
    np.savez_compressed(out or path, **d)
    print(f"{path}: {len(d['seed'])} records re-timed for configurations {configs} in {time.time() - t0:.1f} s",
          flush=True)
    return len(d["seed"])


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--configs", required=True, help="comma-separated configuration indices")
    ap.add_argument("--data", nargs="+", required=True)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out-dir", default=None, help="write the refreshed shards here instead of in place")
    a = ap.parse_args()
    import os

    cfgs = [int(c) for c in a.configs.split(",")]
    for p in a.data:
        out = os.path.join(a.out_dir, os.path.basename(p)) if a.out_dir else None
        if a.out_dir:
            os.makedirs(a.out_dir, exist_ok=True)
        refresh_shard(p, cfgs, a.reps, out)


if __name__ == "__main__":
    main()
