"""Generates the ingest fixtures in tests/golden/ingest/ from the reference's
own graph reader and converter.

Run where the reference's sources exist (default /root/reference):

    python tests/golden/make_ingest_golden.py [--ref /root/reference]

It compiles, with g++ and into oracle/_ref/ingest/, the reference's .mtx ->
.sg converter (data/converter.cpp, with utilities/builder.hpp, reader.hpp,
writer.hpp) and tests/golden/ingest_dump.cpp (the reference's Builder /
Reader loading a .mtx or .sg and printing the CSR they yield).  For each
Matrix Market input — the two the reference ships (data/graph/pdf_test,
data/graph/grb_ppt) and small files this script writes to exercise the
reader's rules (duplicates, self-loops, symmetric mirroring, pattern and
integer fields, comments, unsorted entries) — it stores:

  <name>.mtx  the input (only for the inputs written here)
  <name>.sg   the converter's serialized graph
  <name>.npz  the CSR the reference's reader builds from the .mtx and from
              the .sg (offsets and destinations, uint64)

tests/test_ingest_cpu.py checks vnec_gb300.mtxio against these files.
"""
from __future__ import annotations

import argparse
import os
import shutil
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "ingest")
BUILD = os.path.join(ROOT, "oracle", "_ref", "ingest")


def written_inputs() -> dict[str, str]:
    """Small Matrix Market files covering the reader's rules."""
    rng = np.random.default_rng(17)
    files = {}
    # general, real: duplicates, self-loops, unsorted entries, comments
    lines = ["%%MatrixMarket matrix coordinate real general", "% comment line", "%another", "9 9 0"]
    ent = [(1, 2), (3, 3), (9, 1), (1, 2), (5, 7), (2, 9), (4, 4), (7, 5), (5, 7), (6, 1), (8, 8), (1, 9)]
    ent += [(int(a), int(b)) for a, b in rng.integers(1, 10, size=(20, 2))]
    lines[3] = f"9 9 {len(ent)}"
    lines += [f"{a} {b} {rng.uniform(-1, 1):.6f}" for a, b in ent]
    files["general_dups"] = "\n".join(lines) + "\n"
    # symmetric, real: lower triangle with diagonal entries
    ent = [(2, 1), (3, 1), (3, 3), (5, 2), (6, 6), (7, 4), (8, 1), (8, 7), (4, 4), (6, 5)]
    lines = ["%%MatrixMarket matrix coordinate real symmetric", f"8 8 {len(ent)}"]
    lines += [f"{a} {b} {rng.uniform(-1, 1):.4f}" for a, b in ent]
    files["symmetric_diag"] = "\n".join(lines) + "\n"
    # pattern, general, with trailing blank line
    ent = [(int(a), int(b)) for a, b in rng.integers(1, 13, size=(30, 2))]
    lines = ["%%MatrixMarket matrix coordinate pattern general", f"12 12 {len(ent)}"]
    lines += [f"{a} {b}" for a, b in ent]
    files["pattern"] = "\n".join(lines) + "\n\n"
    # integer field, skew-symmetric (read as general by the reference)
    ent = [(2, 1), (4, 1), (5, 3), (6, 2), (6, 5), (3, 2)]
    lines = ["%%MatrixMarket matrix coordinate integer skew-symmetric", f"6 6 {len(ent)}"]
    lines += [f"{a} {b} {int(rng.integers(-9, 10))}" for a, b in ent]
    files["integer_skew"] = "\n".join(lines) + "\n"
    return files


def build_tools(ref: str) -> tuple[str, str]:
    os.makedirs(BUILD, exist_ok=True)
    flags = ["g++", "-O2", "-std=c++17", "-fopenmp", "-w", "-include", "cstdint", "-I", f"{ref}/include",
             "-I", f"{ref}/src/core/include", "-I", f"{ref}/data"]
    conv = os.path.join(BUILD, "converter")
    dump = os.path.join(BUILD, "ingest_dump")
    subprocess.run(flags + ["-o", conv, f"{ref}/data/converter.cpp"], check=True)
    subprocess.run(flags + ["-o", dump, os.path.join(HERE, "ingest_dump.cpp")], check=True)
    return conv, dump


def read_dump(path: str) -> tuple[np.ndarray, np.ndarray]:
    a = np.fromfile(path, dtype=np.uint64)
    n, m = int(a[0]), int(a[1])
    return a[2:3 + n].copy(), a[3 + n:3 + n + m].copy()


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    args = ap.parse_args()
    conv, dump = build_tools(args.ref)
    os.makedirs(OUT, exist_ok=True)
    work = os.path.join(BUILD, "work")
    os.makedirs(work, exist_ok=True)
    inputs = {name: os.path.join(args.ref, "data", "graph", name, f"{name}.mtx") for name in ("pdf_test", "grb_ppt")}
    for name, text in written_inputs().items():
        p = os.path.join(OUT, f"{name}.mtx")
        with open(p, "w") as f:
            f.write(text)
        inputs[name] = p
    for name, mtx in inputs.items():
        src = os.path.join(work, f"{name}.mtx")
        shutil.copyfile(mtx, src)
        sg = os.path.join(OUT, f"{name}.sg")
        subprocess.run([conv, "-f", src, "-o", sg], check=True, capture_output=True)
        subprocess.run([dump, src, os.path.join(work, "m.bin")], check=True, capture_output=True)
        subprocess.run([dump, sg, os.path.join(work, "s.bin")], check=True, capture_output=True)
        mo, md = read_dump(os.path.join(work, "m.bin"))
        so, sd = read_dump(os.path.join(work, "s.bin"))
        np.savez_compressed(os.path.join(OUT, f"{name}.npz"), mtx_offsets=mo, mtx_dests=md, sg_offsets=so,
                            sg_dests=sd)
        print(name, "nodes", len(mo) - 1, "edges", len(md))


if __name__ == "__main__":
    main()
