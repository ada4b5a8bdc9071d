"""Seeded synthetic sparse matrices for tests, benchmarks and tuner data.

Thin ctypes layer over ``libvnec_gen.so`` (``csrc/generators.cpp``).  Each
generator returns a :class:`HostCSR` whose numpy arrays view memory owned by
the C++ side (no copy, so 2^28-edge R-MAT matrices stay cheap); the memory is
released when the object is garbage collected or :meth:`HostCSR.free` runs.

The shapes follow the workloads the reference is measured on: exactly-k
uniform rows, R-MAT power-law graphs, a 27-point stencil, lognormal row
lengths, dense bands and dense diagonal blocks.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _loader

_i64, _i32, _u64, _f64 = C.c_int64, C.c_int32, C.c_uint64, C.c_double


_library_path: str | None = None


def use_library(path: str) -> None:
    """Load the generators from another build of ``csrc/generators.cpp`` (the
    same seeded algorithms, e.g. the oracle's copy, so that a CPU-only run maps
    no product library).  Must be called before the first generator call."""
    global _library_path
    _library_path = path


def _lib():
    if _library_path is not None:
        lib = _loader.load_path(_library_path)
    else:
        lib = _loader.load("vnec_gen")
    if not getattr(lib, "_vnec_typed", False):
        vp = C.c_void_p
        lib.vnec_gen_uniform_k.argtypes = [_i64, _i64, _i32, _f64, _f64, _u64]
        lib.vnec_gen_rmat.argtypes = [_i32, _i64, _f64, _f64, _f64, _f64, _f64, _u64]
        lib.vnec_gen_stencil27.argtypes = [_i32, _u64]
        lib.vnec_gen_lognormal.argtypes = [_i64, _i64, _f64, _f64, _i32, _f64, _f64, _u64]
        lib.vnec_gen_banded.argtypes = [_i64, _i32, _f64, _f64, _u64]
        lib.vnec_gen_blockdiag.argtypes = [_i64, _i32, _f64, _f64, _u64]
        for f in ("uniform_k", "rmat", "stencil27", "lognormal", "banded", "blockdiag"):
            getattr(lib, "vnec_gen_" + f).restype = vp
        lib.vnec_gen_info.argtypes = [vp, C.POINTER(_i64), C.POINTER(_i64)]
        lib.vnec_gen_info.restype = _i64
        lib.vnec_gen_arrays.argtypes = [vp, C.POINTER(C.POINTER(_i64)), C.POINTER(C.POINTER(_i32)),
                                        C.POINTER(C.POINTER(_f64))]
        lib.vnec_gen_arrays.restype = None
        lib.vnec_gen_free.argtypes = [vp]
        lib.vnec_gen_free.restype = None
        lib.vnec_gen_vector.argtypes = [_i64, _f64, _f64, _u64, C.POINTER(_f64)]
        lib.vnec_gen_vector.restype = None
        lib._vnec_typed = True
    return lib


@dataclass
class HostCSR:
    """CSR matrix in host memory: int64 row offsets, int32 columns, float64 values."""

    n_rows: int
    n_cols: int
    row_ptr: np.ndarray
    col: np.ndarray
    val: np.ndarray
    _handle: int | None = None

    @property
    def nnz(self) -> int:
        return int(self.row_ptr[-1])

    def free(self) -> None:
        if self._handle:
            _lib().vnec_gen_free(self._handle)
            self._handle = None

    def __del__(self):  # pragma: no cover - exercised implicitly
        try:
            self.free()
        except Exception:
            pass

    def copy(self) -> "HostCSR":
        """Independent numpy-owned copy (safe to keep after free())."""
        return HostCSR(self.n_rows, self.n_cols, self.row_ptr.copy(), self.col.copy(), self.val.copy())

    def to_dense(self) -> np.ndarray:
        d = np.zeros((self.n_rows, self.n_cols), dtype=self.val.dtype)
        rows = np.repeat(np.arange(self.n_rows), np.diff(self.row_ptr))
        d[rows, self.col[: self.nnz]] = self.val[: self.nnz]
        return d


def _wrap(handle) -> HostCSR:
    if not handle:
        raise ValueError("generator rejected its arguments")
    lib = _lib()
    nr, nc = _i64(), _i64()
    nnz = lib.vnec_gen_info(handle, C.byref(nr), C.byref(nc))
    rp, cp, vp = C.POINTER(_i64)(), C.POINTER(_i32)(), C.POINTER(_f64)()
    lib.vnec_gen_arrays(handle, C.byref(rp), C.byref(cp), C.byref(vp))
    row_ptr = np.ctypeslib.as_array(rp, shape=(nr.value + 1,))
    col = np.ctypeslib.as_array(cp, shape=(max(nnz, 1),))[:nnz]
    val = np.ctypeslib.as_array(vp, shape=(max(nnz, 1),))[:nnz]
    return HostCSR(nr.value, nc.value, row_ptr, col, val, handle)


def uniform_k(n_rows: int, k: int, *, n_cols: int | None = None, lo=-1.0, hi=1.0, seed=0) -> HostCSR:
    """Exactly k distinct, sorted, uniformly random columns per row; values U(lo, hi)."""
    return _wrap(_lib().vnec_gen_uniform_k(n_rows, n_cols or n_rows, k, lo, hi, seed))


def rmat(scale: int, n_edges: int, a=0.57, b=0.19, c=0.19, *, lo=0.0, hi=1.0, seed=1) -> HostCSR:
    """R-MAT graph, 2^scale vertices, n_edges generated edges, duplicates merged."""
    return _wrap(_lib().vnec_gen_rmat(scale, n_edges, a, b, c, lo, hi, seed))


def stencil27(g: int, *, seed=0) -> HostCSR:
    """27-point stencil on g^3; off-diagonals U(-1, 0], diagonal 1 + sum |off|."""
    return _wrap(_lib().vnec_gen_stencil27(g, seed))


def lognormal(n_rows: int, *, n_cols: int | None = None, mu=float(np.log(8.0)), sigma=1.5, cap=4096,
              lo=-1.0, hi=1.0, seed=0) -> HostCSR:
    """Row lengths round(exp(mu + sigma N(0,1))) capped at `cap`; uniform columns."""
    return _wrap(_lib().vnec_gen_lognormal(n_rows, n_cols or n_rows, mu, sigma, cap, lo, hi, seed))


def banded(n: int, bw: int, *, lo=-1.0, hi=1.0, seed=0) -> HostCSR:
    """Dense band of width bw (columns r - bw//2 .. r + bw//2)."""
    return _wrap(_lib().vnec_gen_banded(n, bw, lo, hi, seed))


def blockdiag(n: int, bs: int, *, lo=-1.0, hi=1.0, seed=0) -> HostCSR:
    """Dense bs x bs diagonal blocks."""
    return _wrap(_lib().vnec_gen_blockdiag(n, bs, lo, hi, seed))


def vector(n: int, *, lo=-1.0, hi=1.0, seed=0) -> np.ndarray:
    """Dense float64 vector with entries U(lo, hi)."""
    out = np.empty(n, dtype=np.float64)
    _lib().vnec_gen_vector(n, lo, hi, seed, out.ctypes.data_as(C.POINTER(_f64)))
    return out


def from_arrays(n_rows: int, n_cols: int, row_ptr, col, val) -> HostCSR:
    """Wrap caller arrays (converted to the canonical dtypes) as a HostCSR."""
    return HostCSR(int(n_rows), int(n_cols), np.ascontiguousarray(row_ptr, dtype=np.int64),
                   np.ascontiguousarray(col, dtype=np.int32), np.ascontiguousarray(val, dtype=np.float64))


def kat_values(m: HostCSR) -> tuple[HostCSR, np.ndarray]:
    """The reference harness's known-answer pattern (test_spmv_vnec.cpp:169,185):
    A_ij = i and x_j = j, so y_i = i * sum(cols of row i) is an exact integer in
    FP64 while below 2^53, whatever the summation order."""
    rows = np.repeat(np.arange(m.n_rows, dtype=np.float64), np.diff(m.row_ptr))
    kat = HostCSR(m.n_rows, m.n_cols, m.row_ptr.copy(), m.col.copy(), rows)
    return kat, np.arange(m.n_cols, dtype=np.float64)


def batch_lognormal(n_mats: int, *, rows_lo: int = 1000, rows_hi: int = 200_000, mu=float(np.log(8.0)),
                    sigma=1.5, cap=4096, lo=-1.0, hi=1.0, seed=0) -> list[HostCSR]:
    """Independent square CSR matrices with row counts log-uniform in
    [rows_lo, rows_hi], lognormal row lengths (mu, sigma) capped at `cap`,
    uniformly random distinct sorted columns and values U(lo, hi)."""
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(rows_lo), np.log(rows_hi), size=n_mats)).astype(np.int64)
    sizes = np.maximum(sizes, 1)
    return [lognormal(int(n), n_cols=int(n), mu=mu, sigma=sigma, cap=cap, lo=lo, hi=hi,
                      seed=seed * 1_000_003 + i + 1) for i, n in enumerate(sizes)]
