"""ctypes bindings of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may use this module, and only as the checker or the timed CPU
baseline; the product library never calls it.

* ``liboracle.so`` (``vnec_oracle.c``): the C restatement of the reference's
  VNEC path, parameterised by partition count and lane width.
* ``libvnec_ref.so`` (optional, built from the reference's own sources by
  ``oracle/Makefile`` target ``ref``: the reference's X86_SIMD build on an
  AVX-512 x86 host, its ARM_NEON build on an aarch64 host): used to pin the
  restatement, to generate the golden fixtures and, on the aarch64 GPU host,
  as the timed CPU baseline.  The reference's sources reach a host without
  the reference checkout as a git-ignored staged archive (``make ref-stage``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvnec_ref.so")
REF_TREE = os.path.join(HERE, "_ref", "src-tree")  # the reference's sources unpacked by `make ref`
GEN_SO = os.path.join(HERE, "_build", "libvnec_gen_oracle.so")

# Compile-time constants of the reference builds (src/operation/include/SpB_mxv.h:17-32),
# plus how each build's compiler evaluates the multiply-adds (vnec_oracle.c:
# orc_loop_mode, orc_lane_fused), pinned bit for bit against that build's own
# outputs: tests/golden/*.npz (X86_SIMD build, x86-64 AVX-512) and
# tests/golden/arm/*.npz (ARM_NEON build, aarch64 Neoverse V2).
X86 = dict(nparts=36, nlanes_f64=8, nlanes_f32=16, thr_f64=0.477, thr_f32=0.437,
           loop_modes=(4, 0, 4, 0, 0, 4, 0, 4, 4, 0), lane_fused=1)
ARM = dict(nparts=48, nlanes_f64=2, nlanes_f32=4, thr_f64=0.76, thr_f32=0.543,
           loop_modes=(0, 0, 0, 0, 0, 0, 0, 4, 0, 0), lane_fused=0)

_vp = C.c_void_p
_i64 = C.c_int64
_lib = None
_ref = None


def build() -> None:
    """Builds liboracle.so, the oracle's copy of the generators and, where the
    reference's sources are available (checkout or staged archive) and the
    host has a reference build (AVX-512 x86 or aarch64), the reference library.
    The reference checkout's location comes from the Makefile (REF, or the
    VNEC_REFERENCE environment variable)."""
    subprocess.run(["make", "-s", "-C", HERE, "all", "gen"], check=True)
    subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def reference_tree() -> str | None:
    """Directory of the reference's sources unpacked by ``make ref``, if any."""
    return REF_TREE if os.path.isdir(os.path.join(REF_TREE, "src", "core", "src")) else None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build()
        L = C.CDLL(ORACLE_SO)
        L.orc_spmv_serial_f64.argtypes = [_i64] + [_vp] * 5
        L.orc_spmv_serial_f32.argtypes = [_i64] + [_vp] * 5
        L.orc_spmv_neumaier_f64.argtypes = [_i64] + [_vp] * 6
        L.orc_spmm_neumaier_f64.argtypes = [_i64, _vp, _vp, _vp, C.c_int, _vp, _vp, _vp]
        L.orc_spmv_L_f64.argtypes = [C.c_int, _i64, _i64] + [_vp] * 5
        L.orc_spmv_L_f32.argtypes = [C.c_int, C.c_int, _i64, _i64] + [_vp] * 5
        for f in ("orc_spmv_D_f64", "orc_spmv_S_f64", "orc_spmv_D_f32", "orc_spmv_S_f32"):
            getattr(L, f).argtypes = [C.c_int, C.c_int, _i64, _i64, _i64] + [_vp] * 5 + [C.c_int]
        L.orc_ird.argtypes = [C.c_int, C.c_int, C.c_float, _i64, _i64, _i64, _vp, _vp, _vp]
        L.orc_ird.restype = C.c_int
        L.orc_partition.argtypes = [C.c_int, _i64, _i64, _vp, _vp, _vp, _vp, _vp]
        L.orc_time_L_f64.argtypes = [C.c_int, _i64, _i64] + [_vp] * 5 + [C.c_int, C.c_int]
        L.orc_time_L_f64.restype = C.c_double
        L.orc_time_S_f64.argtypes = [C.c_int, C.c_int, _i64, _i64, _i64] + [_vp] * 5 + [C.c_int, C.c_int]
        L.orc_time_S_f64.restype = C.c_double
        L.orc_num_procs.restype = C.c_int
        _lib = L
    return _lib


def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref_build() -> dict:
    """Constants of the reference build in libvnec_ref.so (X86 or ARM)."""
    return ARM if ref().ref_num_threads() == ARM["nparts"] else X86


def ref() -> C.CDLL:
    global _ref
    if _ref is None:
        R = C.CDLL(REF_SO)
        for f in ("ref_spmv_f64", "ref_spmv_f32"):
            getattr(R, f).argtypes = [C.c_int, _i64, _i64, _i64] + [_vp] * 6
            getattr(R, f).restype = C.c_int
        R.ref_ird.argtypes = [C.c_int, _i64, _i64, _i64, _vp, _vp, _vp, _vp]
        R.ref_ird.restype = C.c_int
        R.ref_time_L_f64.argtypes = [_i64, _i64, _i64] + [_vp] * 4 + [C.c_int, C.c_int]
        R.ref_time_L_f64.restype = C.c_double
        R.ref_time_f64.argtypes = [C.c_int, _i64, _i64, _i64] + [_vp] * 4 + [C.c_int, C.c_int, _vp]
        R.ref_time_f64.restype = C.c_double
        R.ref_num_threads.restype = C.c_int
        _ref = R
    return _ref


def _use(build: dict) -> None:
    """Sets the oracle's multiply-add evaluation to that of `build`'s compiler."""
    L = lib()
    modes = (C.c_int * len(build["loop_modes"])).in_dll(L, "orc_loop_mode")
    for i, v in enumerate(build["loop_modes"]):
        modes[i] = v
    C.c_int.in_dll(L, "orc_lane_fused").value = build["lane_fused"]


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def _csr(m):
    rp = np.ascontiguousarray(m.row_ptr, dtype=np.int64)
    ci = np.ascontiguousarray(m.col, dtype=np.int32)
    return rp, ci


def spmv_serial(m, x, dtype=np.float64, build=X86) -> np.ndarray:
    """SpB_mxv_FP64_serial / _FP32_serial (test_spmv_vnec.hpp:34-79)."""
    _use(build)
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=dtype)
    xx = np.ascontiguousarray(x, dtype=dtype)
    y = np.zeros(m.n_rows, dtype=dtype)
    f = lib().orc_spmv_serial_f64 if dtype == np.float64 else lib().orc_spmv_serial_f32
    f(m.n_rows, _p(rp), _p(ci), _p(v), _p(xx), _p(y))
    return y


def spmv_neumaier(m, x) -> tuple[np.ndarray, np.ndarray]:
    """Compensated FP64 SpMV and the row conditioning sum_j |a_ij x_j|."""
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(m.n_rows)
    cond = np.zeros(m.n_rows)
    lib().orc_spmv_neumaier_f64(m.n_rows, _p(rp), _p(ci), _p(v), _p(xx), _p(y), _p(cond))
    return y, cond


def spmm_neumaier(m, X) -> tuple[np.ndarray, np.ndarray]:
    """Compensated FP64 Y = A X for row-major X (n_cols x k) and the
    conditioning sums, both n_rows x k (the batched path's checker)."""
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=np.float64)
    X = np.ascontiguousarray(X, dtype=np.float64).reshape(m.n_cols, -1)
    k = X.shape[1]
    Y = np.zeros((m.n_rows, k))
    cond = np.zeros((m.n_rows, k))
    lib().orc_spmm_neumaier_f64(m.n_rows, _p(rp), _p(ci), _p(v), k, _p(X), _p(Y), _p(cond))
    return Y, cond


def spmv_vnec(variant: str, m, x, dtype=np.float64, build=X86) -> np.ndarray:
    """The restated reference kernels: variant in {'L', 'D', 'S'}."""
    _use(build)
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=dtype)
    xx = np.ascontiguousarray(x, dtype=dtype)
    y = np.zeros(m.n_rows, dtype=dtype)
    L = lib()
    f64 = dtype == np.float64
    nl = build["nlanes_f64"] if f64 else build["nlanes_f32"]
    if variant == "L":
        if f64:
            L.orc_spmv_L_f64(build["nparts"], m.n_rows, m.nnz, _p(rp), _p(ci), _p(v), _p(xx), _p(y))
        else:
            L.orc_spmv_L_f32(build["nparts"], nl, m.n_rows, m.nnz, _p(rp), _p(ci), _p(v), _p(xx), _p(y))
    else:
        f = getattr(L, f"orc_spmv_{variant}_{'f64' if f64 else 'f32'}")
        f(build["nparts"], nl, m.n_rows, m.n_cols, m.nnz, _p(rp), _p(ci), _p(v), _p(xx), _p(y), 1)
    return y


def ird(m, fp64: bool = True, build=X86) -> tuple[int, float]:
    """IRD_VNEC restated: (SpB_VNEC_D=0 / SpB_VNEC_S=1, ratio)."""
    rp, ci = _csr(m)
    out = np.zeros(1, dtype=np.float32)
    nl = build["nlanes_f64"] if fp64 else build["nlanes_f32"]
    thr = build["thr_f64"] if fp64 else build["thr_f32"]
    t = lib().orc_ird(build["nparts"], nl, C.c_float(thr), m.n_rows, m.n_cols, m.nnz, _p(rp), _p(ci), _p(out))
    return t, float(out[0])


def time_L_f64(m, x, nparts: int, warm: int = 1, reps: int = 40, build=None) -> float:
    """Seconds per SpMV_VNEC_L_FP64 call of the restatement (OpenMP, nparts threads)."""
    _use(build or (ARM if nparts == ARM["nparts"] else X86))
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(m.n_rows)
    return lib().orc_time_L_f64(nparts, m.n_rows, m.nnz, _p(rp), _p(ci), _p(v), _p(xx), _p(y), warm, reps)


def time_S_f64(m, x, build=ARM, warm: int = 1, reps: int = 40) -> float:
    """Seconds per SpMV_VNEC_S_FP64 call of the restatement (format built once)."""
    _use(build)
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    y = np.zeros(m.n_rows)
    return lib().orc_time_S_f64(build["nparts"], build["nlanes_f64"], m.n_rows, m.n_cols, m.nnz, _p(rp), _p(ci),
                                _p(v), _p(xx), _p(y), warm, reps)


def ref_spmv(variant: int, m, x, dtype=np.float64) -> tuple[np.ndarray, int, float]:
    """The reference build itself: variant 0 auto (harness dispatch), 1 D, 2 S, 3 L, 4 serial."""
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=dtype)
    xx = np.ascontiguousarray(x, dtype=dtype)
    y = np.zeros(m.n_rows, dtype=dtype)
    irdv = np.zeros(1, dtype=np.float32)
    f = ref().ref_spmv_f64 if dtype == np.float64 else ref().ref_spmv_f32
    used = f(variant, m.n_rows, m.n_cols, m.nnz, _p(rp), _p(ci), _p(v), _p(xx), _p(y), _p(irdv))
    return y, used, float(irdv[0])


def ref_time_f64(m, x, variant: int = 0, warm: int = 1, reps: int = 40) -> tuple[float, str]:
    """Seconds per call of the reference build's own FP64 SpMV (variant 0: the
    harness's dispatch; 1 D, 2 S, 3 L) and the name of the variant run."""
    rp, ci = _csr(m)
    v = np.ascontiguousarray(m.val, dtype=np.float64)
    xx = np.ascontiguousarray(x, dtype=np.float64)
    used = np.zeros(1, dtype=np.int32)
    secs = ref().ref_time_f64(variant, m.n_rows, m.n_cols, m.nnz, _p(rp), _p(ci), _p(v), _p(xx), warm, reps,
                              _p(used))
    return float(secs), {1: "VNEC-D", 2: "VNEC-S", 3: "VNEC-L"}.get(int(used[0]), "?")


def rowwise_error(y: np.ndarray, y_ref: np.ndarray, cond: np.ndarray) -> np.ndarray:
    """|y_i - yref_i| / sum_j |a_ij x_j| (0 where the row's conditioning sum is 0)."""
    d = np.abs(y.astype(np.float64) - y_ref)
    with np.errstate(divide="ignore", invalid="ignore"):
        e = np.where(cond > 0, d / np.where(cond > 0, cond, 1.0), d)
    return e
