"""Generates the golden fixtures in this directory from the reference itself.

Run in a container where the reference sources exist (default
/root/reference) on an x86-64 host with AVX-512:

    python tests/golden/make_golden.py [--ref /root/reference]

It builds ``oracle/_ref/libvnec_ref.so`` from the reference's own sources
(oracle/Makefile, target ``ref``), then, for each case below, runs the
reference's VNEC FP64 and FP32 paths (D, S and L forced, the harness's own
dispatch, and the serial CSR loop of its test) and stores inputs and outputs
in ``<case>.npz``.  Cases: the two Matrix Market fixtures the reference ships
(data/graph/pdf_test, data/graph/grb_ppt), seeded synthetic matrices of the
benchmark families at small sizes, the harness's known-answer pattern
(A_ij = i, x_j = j, test_spmv_vnec.cpp:169,185), and edge cases (empty
rows, a row longer than a partition, an empty matrix).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from vnec_gb300 import generators as G  # noqa: E402
from vnec_gb300 import mtxio  # noqa: E402


def hub_matrix(seed: int = 7) -> G.HostCSR:
    """100 x 5000, short rows plus one 4000-entry row spanning many partitions."""
    rng = np.random.default_rng(seed)
    rows = []
    for r in range(100):
        k = 4000 if r == 3 else int(rng.integers(0, 9))
        rows.append(np.sort(rng.choice(5000, size=k, replace=False)))
    row_ptr = np.zeros(101, dtype=np.int64)
    row_ptr[1:] = np.cumsum([len(c) for c in rows])
    col = np.concatenate(rows).astype(np.int32)
    val = rng.uniform(-1.0, 1.0, size=col.size)
    return G.from_arrays(100, 5000, row_ptr, col, val)


def empty_rows_matrix(seed: int = 8) -> G.HostCSR:
    """300 x 300 with 70% empty rows including a run of trailing empty rows."""
    rng = np.random.default_rng(seed)
    lens = np.where(rng.random(300) < 0.3, rng.integers(1, 40, size=300), 0)
    lens[-25:] = 0
    rows = [np.sort(rng.choice(300, size=int(k), replace=False)) for k in lens]
    row_ptr = np.zeros(301, dtype=np.int64)
    row_ptr[1:] = np.cumsum(lens)
    col = np.concatenate(rows).astype(np.int32)
    return G.from_arrays(300, 300, row_ptr, col, rng.uniform(-1, 1, size=col.size))


def cases(ref_root: str):
    yield "pdf_test", mtxio.read_mtx(os.path.join(ref_root, "data/graph/pdf_test/pdf_test.mtx")), None
    yield "grb_ppt", mtxio.read_mtx(os.path.join(ref_root, "data/graph/grb_ppt/grb_ppt.mtx")), None
    yield "uniform_k16", G.uniform_k(2048, 16, seed=0).copy(), None
    yield "rmat_s11", G.rmat(11, 16 * 2048, seed=1).copy(), None
    yield "stencil_g8", G.stencil27(8, seed=2).copy(), None
    yield "lognormal_1500", G.lognormal(1500, seed=3).copy(), None
    yield "banded_bw9", G.banded(1200, 9, seed=4).copy(), None
    yield "blockdiag_16", G.blockdiag(640, 16, seed=5).copy(), None
    yield "hub_row", hub_matrix(), None
    yield "empty_rows", empty_rows_matrix(), None
    yield "empty_matrix", G.from_arrays(5, 5, np.zeros(6, dtype=np.int64), np.zeros(0, np.int32), np.zeros(0)), None
    for name, m in (("kat_uniform_k16", G.uniform_k(2048, 16, seed=0)), ("kat_rmat_s11", G.rmat(11, 16 * 2048, seed=1))):
        kat, x = G.kat_values(m)
        yield name, kat, x


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={args.ref}"], check=True)
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={args.ref}", "ref"], check=True)
    if not O.ref_available():
        raise SystemExit("reference library not built (needs the reference sources and an AVX-512 x86 host)")
    R = O.ref()
    manifest = {"reference_build": {"NUM_THREADS": R.ref_num_threads(), "nLanes_f64": R.ref_nlanes_f64(),
                                    "nLanes_f32": R.ref_nlanes_f32()}, "cases": {}}
    for name, m, x in cases(args.ref):
        if x is None:
            x = G.vector(m.n_cols, seed=11)
        out = {"n_rows": m.n_rows, "n_cols": m.n_cols, "row_ptr": m.row_ptr.astype(np.int64),
               "col": m.col[: m.nnz].astype(np.int32), "val": m.val[: m.nnz].astype(np.float64), "x": x}
        # The reference's D and S builders are only defined when every one of
        # its NUM_THREADS partitions starts before the end of the merge path:
        # otherwise the row-rounded partitions of Build_VNEC_S read past ptr
        # (spmv_vnec_S_for_mxv.c:362-370) and one such call never returned.
        nparts = R.ref_num_threads()
        items = m.n_rows + m.nnz
        sane = ((items + nparts - 1) // nparts) * (nparts - 1) < items and m.nnz > 0
        meta = {"n_rows": m.n_rows, "n_cols": m.n_cols, "nnz": m.nnz, "vnec_ds_defined": bool(sane)}
        out["vnec_ds_defined"] = np.bool_(sane)
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
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
        manifest["cases"][name] = meta
        print(name, meta)
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump(manifest, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
