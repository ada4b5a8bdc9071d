"""Ingest pinned to the reference's own graph reader and converter.

The fixtures in tests/golden/ingest/ were made by the reference's code
(tests/golden/make_ingest_golden.py): its .mtx -> .sg converter
(data/converter.cpp) and its Builder / Reader loading the .mtx and the .sg
(utilities/builder.hpp:165-185,319-344, utilities/reader.hpp:37-240).  The
library's readers must yield the same CSR, and its .sg writer the same bytes.
"""
from __future__ import annotations

import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

INGEST = os.path.join(GOLDEN, "ingest")
NAMES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(INGEST, "*.npz")))


@pytest.mark.parametrize("name", NAMES)
def test_read_sg_matches_reference_reader(name):
    from vnec_gb300 import mtxio

    z = np.load(os.path.join(INGEST, f"{name}.npz"))
    g = mtxio.read_sg(os.path.join(INGEST, f"{name}.sg"))
    assert np.array_equal(g.row_ptr, z["sg_offsets"].astype(np.int64))
    assert np.array_equal(g.col[: g.nnz], z["sg_dests"].astype(np.int32))
    # the harness's values: A_ij = i (test_spmv_vnec.cpp:169)
    assert np.array_equal(g.val[: g.nnz], np.repeat(np.arange(g.n_rows, dtype=np.float64), np.diff(g.row_ptr)))
    # the reference reads the same graph from the .mtx and from its .sg
    assert np.array_equal(z["mtx_offsets"], z["sg_offsets"]) and np.array_equal(z["mtx_dests"], z["sg_dests"])


@pytest.mark.parametrize("name", [n for n in NAMES if os.path.exists(os.path.join(INGEST, f"{n}.mtx"))])
def test_read_mtx_graph_matches_reference_reader(name):
    from vnec_gb300 import mtxio

    z = np.load(os.path.join(INGEST, f"{name}.npz"))
    g = mtxio.read_mtx_graph(os.path.join(INGEST, f"{name}.mtx"))
    assert np.array_equal(g.row_ptr, z["mtx_offsets"].astype(np.int64))
    assert np.array_equal(g.col[: g.nnz], z["mtx_dests"].astype(np.int32))


@pytest.mark.parametrize("name", NAMES)
def test_write_sg_matches_reference_converter(name, tmp_path):
    from vnec_gb300 import mtxio

    sg = os.path.join(INGEST, f"{name}.sg")
    with open(sg, "rb") as f:
        want = f.read()
    g = mtxio.read_sg(sg)
    out = tmp_path / "g.sg"
    mtxio.write_sg(str(out), g, directed=bool(want[0]))
    assert out.read_bytes() == want


def test_read_mtx_graph_rejects_what_the_reference_rejects(tmp_path):
    from vnec_gb300 import mtxio

    bad = {"rect": "%%MatrixMarket matrix coordinate real general\n3 4 1\n1 2 1.0\n",
           "complex": "%%MatrixMarket matrix coordinate complex general\n2 2 1\n1 2 1 0\n",
           "array": "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n",
           "hermitian": "%%MatrixMarket matrix coordinate real hermitian\n2 2 1\n2 1 1.0\n",
           "noheader": "3 3 1\n1 2 1.0\n"}
    for name, text in bad.items():
        p = tmp_path / f"{name}.mtx"
        p.write_text(text)
        with pytest.raises(ValueError):
            mtxio.read_mtx_graph(str(p))
