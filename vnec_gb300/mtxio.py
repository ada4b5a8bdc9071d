"""Real-matrix ingest: Matrix Market (.mtx) and GAP serialized graphs (.sg).

* ``read_mtx`` follows the coordinate Matrix Market format the reference's
  reader accepts (``utilities/reader.hpp:37-150``): 1-based (row, col[, value])
  triples after a size line; ``symmetric`` files are mirrored; ``pattern``
  files get value 1.
* ``read_mtx_graph`` reads a .mtx file the way the reference's graph reader
  does before its test harness assigns values (``utilities/reader.hpp:37-163``
  then ``utilities/builder.hpp:165-185``): the pattern only, 0-based,
  ``symmetric`` files mirrored, edges sorted, duplicate edges and self-loops
  removed; values are the harness's (row index).
* ``read_sg`` / ``write_sg`` follow the serialized CSR the reference's test
  harness loads (``utilities/reader.hpp:189-240``): bool directed, uint64
  num_edges, uint64 num_nodes, uint64 offsets[num_nodes + 1], uint64
  destinations[num_edges] (and the inverse graph when directed).

Both return a :class:`vnec_gb300.generators.HostCSR` with sorted rows; for
``.sg`` graphs the values are those the reference harness assigns (row index,
``test_spmv_vnec.cpp:169``) unless a value array is supplied.
"""
from __future__ import annotations

import numpy as np

from .generators import HostCSR, from_arrays


def _coo_to_csr(n_rows: int, n_cols: int, r: np.ndarray, c: np.ndarray, v: np.ndarray,
                merge_duplicates: bool = True) -> HostCSR:
    order = np.lexsort((c, r))
    r, c, v = r[order], c[order], v[order]
    if merge_duplicates and r.size:
        key = r.astype(np.int64) * max(n_cols, 1) + c
        first = np.concatenate(([True], key[1:] != key[:-1]))
        idx = np.cumsum(first) - 1
        v = np.bincount(idx, weights=v, minlength=int(first.sum())).astype(np.float64)
        r, c = r[first], c[first]
    counts = np.bincount(r, minlength=n_rows)
    row_ptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    return from_arrays(n_rows, n_cols, row_ptr, c, v)


def read_mtx(path: str) -> HostCSR:
    with open(path) as f:
        header = f.readline().strip().lower().split()
        if len(header) < 4 or header[0] != "%%matrixmarket" or header[2] != "coordinate":
            raise ValueError(f"{path}: only coordinate Matrix Market files are supported")
        field = header[3]
        symmetry = header[4] if len(header) > 4 else "general"
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        n_rows, n_cols, nnz = (int(t) for t in line.split()[:3])
        data = np.loadtxt(f, ndmin=2, max_rows=nnz) if nnz else np.zeros((0, 3))
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = data[:, 2].astype(np.float64) if field != "pattern" and data.shape[1] > 2 else np.ones(len(r))
    if symmetry in ("symmetric", "skew-symmetric", "hermitian"):
        off = r != c
        sign = -1.0 if symmetry == "skew-symmetric" else 1.0
        r, c, v = np.concatenate((r, c[off])), np.concatenate((c, r[off])), np.concatenate((v, sign * v[off]))
    return _coo_to_csr(n_rows, n_cols, r, c, v)


def read_mtx_graph(path: str, values: np.ndarray | None = None) -> HostCSR:
    """The graph the reference's Builder makes from a Matrix Market file (the
    CSR its .mtx -> .sg converter writes): square coordinate matrices only,
    field pattern / real / double / integer, symmetry general, skew-symmetric
    (read as general) or symmetric (each entry also read transposed); then
    sorted, duplicate edges merged into one, self-loops dropped."""
    with open(path) as f:
        head = f.readline().split()
        if len(head) < 5 or head[0] not in ("%%MatrixMarket", "%MatrixMarket"):
            raise ValueError(f"{path}: .mtx file did not start with %%MatrixMarket or %MatrixMarket")
        obj, fmt, field, symmetry = head[1], head[2], head[3], head[4]
        if obj != "matrix" or fmt != "coordinate":
            raise ValueError(f"{path}: only matrix coordinate format is read")
        if field not in ("pattern", "real", "double", "integer"):
            raise ValueError(f"{path}: unsupported field {field!r}")
        if symmetry not in ("general", "skew-symmetric", "symmetric"):
            raise ValueError(f"{path}: unsupported symmetry {symmetry!r}")
        line = f.readline()
        while line.startswith("%"):
            line = f.readline()
        n_rows, n_cols = (int(t) for t in line.split()[:2])
        if n_rows != n_cols:
            raise ValueError(f"{path}: matrix must be square")
        pairs = [tuple(int(t) for t in ln.split()[:2]) for ln in f if ln.strip()]
    e = np.asarray(pairs, dtype=np.int64).reshape(-1, 2) - 1
    if symmetry == "symmetric":
        e = np.concatenate((e, e[:, ::-1]))
    e = e[e[:, 0] != e[:, 1]]
    e = np.unique(e, axis=0)  # sorted by (row, column), duplicates merged
    counts = np.bincount(e[:, 0], minlength=n_rows)
    row_ptr = np.zeros(n_rows + 1, dtype=np.int64)
    np.cumsum(counts, out=row_ptr[1:])
    if values is None:
        values = np.repeat(np.arange(n_rows, dtype=np.float64), counts)
    return from_arrays(n_rows, n_cols, row_ptr, e[:, 1], np.asarray(values, dtype=np.float64))


def read_sg(path: str, values: np.ndarray | None = None) -> HostCSR:
    with open(path, "rb") as f:
        directed = bool(np.frombuffer(f.read(1), dtype=np.uint8)[0])
        num_edges = int(np.frombuffer(f.read(8), dtype=np.uint64)[0])
        num_nodes = int(np.frombuffer(f.read(8), dtype=np.uint64)[0])
        offsets = np.frombuffer(f.read(8 * (num_nodes + 1)), dtype=np.uint64).astype(np.int64)
        dests = np.frombuffer(f.read(8 * num_edges), dtype=np.uint64).astype(np.int64)
    del directed  # the inverse graph, when present, is not needed for y = A x
    if values is None:
        values = np.repeat(np.arange(num_nodes, dtype=np.float64), np.diff(offsets))
    # Rows of a .sg file are not guaranteed sorted: sort within rows.
    rows = np.repeat(np.arange(num_nodes, dtype=np.int64), np.diff(offsets))
    return _coo_to_csr(num_nodes, num_nodes, rows, dests, np.asarray(values, dtype=np.float64),
                       merge_duplicates=False)


def write_sg(path: str, m: HostCSR, directed: bool = False) -> None:
    """Writes the pattern of a square matrix; a directed graph also gets its
    inverse (transposed) adjacency, as the reference reader expects."""
    with open(path, "wb") as f:
        f.write(np.uint8(1 if directed else 0).tobytes())
        f.write(np.uint64(m.nnz).tobytes())
        f.write(np.uint64(m.n_rows).tobytes())
        f.write(np.ascontiguousarray(m.row_ptr, dtype=np.uint64).tobytes())
        f.write(np.ascontiguousarray(m.col[: m.nnz], dtype=np.uint64).tobytes())
        if directed:
            rows = np.repeat(np.arange(m.n_rows, dtype=np.int64), np.diff(m.row_ptr))
            t = _coo_to_csr(m.n_cols, m.n_rows, np.asarray(m.col[: m.nnz], dtype=np.int64), rows,
                            np.ones(m.nnz), merge_duplicates=False)
            f.write(np.ascontiguousarray(t.row_ptr, dtype=np.uint64).tobytes())
            f.write(np.ascontiguousarray(t.col, dtype=np.uint64).tobytes())
