"""Outputs of the reference's ARM_NEON build on the golden inputs.

Run on an aarch64 host (the GPU host) after ``oracle/Makefile`` has built
``oracle/_ref/libvnec_ref.so`` from the reference's own sources with the
reference's ARM flags (``-DARM_NEON``, NUM_THREADS 48, nLanes 2/4):

    python tests/golden/make_golden_arm.py --out tests/golden/arm

For every fixture ``tests/golden/<case>.npz`` (the inputs written by
make_golden.py on x86) it runs the ARM build's VNEC FP64 and FP32 paths — D, S
and L forced, the harness's own dispatch (IRD_VNEC) and the serial CSR loop of
its test — and stores only the outputs in ``<out>/<case>.npz``, plus
``<out>/manifest.json`` with the build constants.  tests/test_oracle.py pins
the oracle's ARM parameterisation against these files bit for bit.
"""
from __future__ import annotations

import argparse
import glob
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from conftest import golden_csr  # noqa: E402
from oracle import oracle as O  # noqa: E402


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "arm"))
    args = ap.parse_args()
    O.build()
    if not O.ref_available() or O.ref_build() is not O.ARM:
        raise SystemExit("needs the reference's ARM_NEON build (oracle/_ref/libvnec_ref.so on an aarch64 host)")
    R = O.ref()
    os.makedirs(args.out, exist_ok=True)
    nparts = R.ref_num_threads()
    manifest = {"reference_build": {"NUM_THREADS": nparts, "nLanes_f64": R.ref_nlanes_f64(),
                                    "nLanes_f32": R.ref_nlanes_f32(), "flags": "ARM_NEON"}, "cases": {}}
    for path in sorted(glob.glob(os.path.join(HERE, "*.npz"))):
        name = os.path.splitext(os.path.basename(path))[0]
        with np.load(path) as z:
            g = {k: z[k] for k in z.files}
        m = golden_csr(g)
        x = g["x"]
        # D and S are only defined when every partition starts before the end
        # of the merge path (see make_golden.py).
        items = m.n_rows + m.nnz
        sane = ((items + nparts - 1) // nparts) * (nparts - 1) < items and m.nnz > 0
        out = {"vnec_ds_defined": np.bool_(sane)}
        meta = {"vnec_ds_defined": bool(sane)}
        for dt, tag in ((np.float64, "f64"), (np.float32, "f32")):
            for var, vname in ((1, "D"), (2, "S"), (3, "L"), (4, "serial")):
                if vname in ("D", "S") and not sane:
                    continue
                y, _, _ = O.ref_spmv(var, m, x, dtype=dt)
                out[f"y_{vname}_{tag}"] = y
            if not sane:
                continue
            y, used, irdv = O.ref_spmv(0, m, x, dtype=dt)
            out[f"y_auto_{tag}"] = y
            out[f"auto_variant_{tag}"] = np.int32(used)
            out[f"ird_{tag}"] = np.float32(irdv)
            meta[f"auto_{tag}"] = {1: "D", 2: "S", 3: "L"}[used]
            meta[f"ird_{tag}"] = irdv
        np.savez_compressed(os.path.join(args.out, f"{name}.npz"), **out)
        manifest["cases"][name] = meta
        print(name, meta)
    with open(os.path.join(args.out, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
