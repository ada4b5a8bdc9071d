"""Python mirror of the OpenSparseBLAS VNEC mxv interface, over the C ABI.

The functions keep the reference's names and argument meaning
(``include/OpenSparseBLAS.h:1951-2073``): ``IRD_VNEC``, ``Build_VNEC_L``,
``SpMV_VNEC_L_FP64``, ``SpB_mxv`` ... operate on :class:`Matrix` and
:class:`Vector`, which own reference-layout objects (``SpB_Matrix_CSC_or_CSR``
with 64-bit ``SpB_Index`` offsets and columns, ``SpB_Vector_Dense``), so the
calls exercise exactly the entry points a C caller of the reference would.
Errors raise :class:`VnecError` carrying the library's last-error message —
the reference exits the process instead (``src/core/src/SpB_Error.c:4-8``).

Everything runs through ``libvnec_gb300.so``; nothing here computes on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _loader

# Enum values of include/vnec_spb_types.h (mirroring include/OpenSparseBLAS.h).
SpB_SUCCESS, SpB_FAILURE = 0, 1
SpB_FP32, SpB_FP64 = 10, 11
SpB_DENSE = 0
SpB_CSC, SpB_CSR = 0, 1
SpB_VNEC_D, SpB_VNEC_S = 0, 1
KERNEL_AUTO, KERNEL_L, KERNEL_D, KERNEL_S, KERNEL_BATCH, KERNEL_HYBRID = 0, 1, 2, 3, 4, 5
KERNEL_LEARNED, KERNEL_SEARCH, KERNEL_RULE, KERNEL_PUSH = 6, 7, 8, 9
CHOSEN_DIRECT, CHOSEN_LEARNED, CHOSEN_SEARCH, CHOSEN_RULE, CHOSEN_FALLBACK = 0, 1, 2, 3, 4
ARITH_AUTO, ARITH_FP64, ARITH_DF32 = 0, 1, 2
PREC_FP64, PREC_FP32, PREC_BF16, PREC_DF32 = 0, 1, 2, 3

_DTYPE = {SpB_FP32: np.float32, SpB_FP64: np.float64}


class VnecError(RuntimeError):
    """A C-ABI call reported failure; the message is the library's last error."""


class _MatrixBase(C.Structure):
    _fields_ = [("element_type", C.c_int), ("format_type", C.c_int), ("row", C.c_uint64),
                ("col", C.c_uint64), ("element_size", C.c_size_t)]


class _CsrStruct(C.Structure):
    _fields_ = [("matrix_base", _MatrixBase), ("val", C.c_void_p), ("indices", C.POINTER(C.c_uint64)),
                ("ptr", C.POINTER(C.c_uint64)), ("ptr_len", C.c_uint64), ("nnz", C.c_uint64),
                ("capacity", C.c_uint64)]


class _VectorBase(C.Structure):
    _fields_ = [("element_type", C.c_int), ("format_type", C.c_int), ("n", C.c_uint64),
                ("element_size", C.c_size_t)]


class _DenseStruct(C.Structure):
    _fields_ = [("vector_base", _VectorBase), ("values", C.c_void_p)]


class Options(C.Structure):
    """SpB_VNEC_options_ext."""

    _fields_ = [("kernel", C.c_int), ("threads_per_block", C.c_int), ("items_per_thread", C.c_int),
                ("pipeline_stages", C.c_int), ("arithmetic", C.c_int), ("window_rows", C.c_int),
                ("long_row_len", C.c_int), ("max_steps", C.c_int), ("cache_hints", C.c_int),
                ("precision", C.c_int), ("hot_columns", C.c_int), ("dense_fill_permille", C.c_int),
                ("transpose", C.c_int), ("host_parts", C.c_int), ("column_deltas", C.c_int),
                ("lane_vectors", C.c_int), ("hot_order", C.c_int), ("offsets64", C.c_int),
                ("shared_patterns", C.c_int), ("l2_prefetch", C.c_int), ("reserved", C.c_int * 4)]


class Info(C.Structure):
    """SpB_VNEC_info_ext."""

    _fields_ = [("kernel", C.c_int), ("value_type", C.c_int), ("n_rows", C.c_int64), ("n_cols", C.c_int64),
                ("nnz", C.c_int64), ("device_bytes", C.c_int64), ("algorithmic_bytes", C.c_int64),
                ("launches_per_call", C.c_int), ("threads_per_block", C.c_int), ("items_per_thread", C.c_int),
                ("num_tiles", C.c_int64), ("pipeline_stages", C.c_int), ("arithmetic", C.c_int),
                ("blocks", C.c_int64), ("precision", C.c_int), ("rhs", C.c_int), ("lanes", C.c_int),
                ("long_row_len", C.c_int)]


class BatchOptions(C.Structure):
    """SpB_VNEC_batch_options_ext."""

    _fields_ = [("precision", C.c_int), ("lanes", C.c_int), ("long_row_len", C.c_int), ("chunk", C.c_int),
                ("warps_per_block", C.c_int), ("autotune", C.c_int), ("no_graph", C.c_int),
                ("window_rows", C.c_int), ("max_steps", C.c_int), ("unroll", C.c_int), ("host_parts", C.c_int),
                ("dispatch", C.c_int), ("k1_layout", C.c_int), ("reserved", C.c_int * 3)]


_vp = C.c_void_p


def lib() -> C.CDLL:
    """The loaded C-ABI library, with argument types declared."""
    L = _loader.load("vnec_gb300")
    if getattr(L, "_vnec_typed", False):
        return L
    L.SpB_mxv.argtypes = [_vp, _vp, _vp, _vp]
    L.SpB_mxv.restype = C.c_int
    L.IRD_VNEC.argtypes = [_vp, C.c_int]
    L.IRD_VNEC.restype = C.c_int
    L.Build_VNEC_L.argtypes = [_vp]
    L.Build_VNEC_L.restype = _vp
    for f in ("SpMV_VNEC_L_FP64", "SpMV_VNEC_L_FP32", "SpMV_VNEC_S_FP64", "SpMV_VNEC_S_FP32",
              "SpMV_VNEC_D_FP64", "SpMV_VNEC_D_FP32"):
        getattr(L, f).argtypes = [_vp, _vp, _vp, _vp]
        getattr(L, f).restype = None
    for f in ("Build_VNEC_S_FP64", "Build_VNEC_S_FP32", "Build_VNEC_D_FP64", "Build_VNEC_D_FP32"):
        getattr(L, f).argtypes = [_vp]
        getattr(L, f).restype = _vp
    for f in ("VNEC_L_free_ext", "VNEC_S_free_fp64", "VNEC_S_free_fp32", "VNEC_D_free_fp64", "VNEC_D_free_fp32"):
        getattr(L, f).argtypes = [_vp]
        getattr(L, f).restype = None
    L.SpB_VNEC_last_error_ext.argtypes = []
    L.SpB_VNEC_last_error_ext.restype = C.c_char_p
    L.SpB_VNEC_plan_ext.argtypes = [C.POINTER(Options), C.c_int, C.c_int64, C.c_int64, _vp, _vp, _vp]
    L.SpB_VNEC_plan_ext.restype = _vp
    L.SpB_VNEC_plan_matrix_ext.argtypes = [C.POINTER(Options), _vp]
    L.SpB_VNEC_plan_matrix_ext.restype = _vp
    L.SpB_VNEC_plan_free_ext.argtypes = [_vp]
    L.SpB_VNEC_plan_free_ext.restype = None
    L.SpB_VNEC_forget_ext.argtypes = [_vp]
    L.SpB_VNEC_forget_ext.restype = None
    L.SpB_mxv_device_ext.argtypes = [_vp, _vp, _vp, _vp]
    L.SpB_mxv_device_ext.restype = C.c_int
    L.SpB_mxv_axpby_ext.argtypes = [_vp, _vp, _vp, C.c_double, C.c_double, _vp, C.c_double, _vp]
    L.SpB_mxv_axpby_ext.restype = C.c_int
    L.SpB_mxv_host_ext.argtypes = [_vp, _vp, _vp]
    L.SpB_mxv_host_ext.restype = C.c_int
    L.SpB_mxv_host_async_ext.argtypes = [_vp, _vp, _vp]
    L.SpB_mxv_host_async_ext.restype = C.c_int
    L.SpB_VNEC_host_wait_ext.argtypes = [_vp]
    L.SpB_VNEC_host_wait_ext.restype = C.c_int
    L.SpB_VNEC_plan_info_ext.argtypes = [_vp, C.POINTER(Info)]
    L.SpB_VNEC_plan_info_ext.restype = C.c_int
    L.SpB_VNEC_set_profiling_ext.argtypes = [_vp, C.c_int]
    L.SpB_VNEC_set_profiling_ext.restype = C.c_int
    L.SpB_VNEC_kernel_ms_ext.argtypes = [_vp, C.POINTER(C.c_float), C.c_int]
    L.SpB_VNEC_kernel_ms_ext.restype = C.c_int
    L.SpB_VNEC_device_status_ext.argtypes = [_vp, _vp]
    L.SpB_VNEC_device_status_ext.restype = C.c_int
    L.SpB_VNEC_wait_polls_ext.argtypes = [_vp, C.c_int64]
    L.SpB_VNEC_wait_polls_ext.restype = C.c_int
    L.SpB_VNEC_f64_to_f32_ext.argtypes = [_vp, _vp, C.c_int64, _vp]
    L.SpB_VNEC_f64_to_f32_ext.restype = C.c_int
    L.SpB_VNEC_spmspv_ext.argtypes = [_vp, C.c_int64, _vp, _vp, _vp, _vp]
    L.SpB_VNEC_spmspv_ext.restype = C.c_int
    L.SpB_VNEC_spmspv_host_ext.argtypes = [_vp, C.c_int64, _vp, _vp, _vp]
    L.SpB_VNEC_spmspv_host_ext.restype = C.c_int
    L.SpB_VNEC_batch_plan_ext.argtypes = [C.c_int, _vp, _vp, _vp, _vp, _vp, C.c_int, C.POINTER(BatchOptions)]
    L.SpB_VNEC_batch_plan_ext.restype = _vp
    L.SpB_VNEC_batch_plan_matrices_ext.argtypes = [C.c_int, _vp, C.c_int, C.POINTER(BatchOptions)]
    L.SpB_VNEC_batch_plan_matrices_ext.restype = _vp
    L.SpB_VNEC_batch_offsets_ext.argtypes = [_vp, _vp, _vp]
    L.SpB_VNEC_batch_offsets_ext.restype = C.c_int
    L.SpB_VNEC_batch_tuning_ext.argtypes = [_vp, _vp, _vp, C.c_int, C.POINTER(C.c_int)]
    L.SpB_VNEC_batch_tuning_ext.restype = C.c_int
    _f = C.POINTER(C.c_float)
    L.SpB_VNEC_tune_configs_ext.argtypes = [_vp, _vp, _vp, C.c_int]
    L.SpB_VNEC_tune_configs_ext.restype = C.c_int
    L.SpB_VNEC_features_ext.argtypes = [C.c_int64, C.c_int64, _vp, _vp, _vp]
    L.SpB_VNEC_features_ext.restype = C.c_int
    L.SpB_VNEC_autotune_ext.argtypes = [C.POINTER(Options), C.c_int, C.c_int64, C.c_int64, _vp, _vp, _vp, C.c_int,
                                        _vp]
    L.SpB_VNEC_autotune_ext.restype = C.c_int
    L.SpB_VNEC_time_configs_ext.argtypes = [C.POINTER(Options), C.c_int, C.c_int64, C.c_int64, _vp, _vp, _vp,
                                            C.c_int, _vp, C.c_int, _vp]
    L.SpB_VNEC_time_configs_ext.restype = C.c_int
    L.SpB_VNEC_stream_gather_ext.argtypes = [_vp, C.c_int64, _vp, _vp, C.c_int64, _vp, _vp]
    L.SpB_VNEC_stream_gather_ext.restype = C.c_int
    L.SpB_mxv_axpbyg_ext.argtypes = [_vp, _vp, _vp, C.c_double, C.c_double, _vp, C.c_double, _vp, C.c_double, _vp]
    L.SpB_mxv_axpbyg_ext.restype = C.c_int
    L.SpB_VNEC_dot_ext.argtypes = [C.c_int64, _vp, _vp, C.c_int, _vp, _vp, _vp]
    L.SpB_VNEC_dot_ext.restype = C.c_int
    L.SpB_VNEC_rule_choice_ext.argtypes = [C.c_int, C.c_int64, C.c_int64, _vp, _vp, _vp]
    L.SpB_VNEC_rule_choice_ext.restype = C.c_int
    L.SpB_VNEC_learned_choice_ext.argtypes = [C.c_int, C.c_int64, C.c_int64, _vp, _vp, _vp, _vp, _vp]
    L.SpB_VNEC_learned_choice_ext.restype = C.c_int
    L.SpB_VNEC_plan_choice_ext.argtypes = [_vp, _vp, _vp]
    L.SpB_VNEC_plan_choice_ext.restype = C.c_int
    L.SpB_VNEC_mlp_create_ext.argtypes = [C.c_uint64]
    L.SpB_VNEC_mlp_create_ext.restype = _vp
    L.SpB_VNEC_mlp_free_ext.argtypes = [_vp]
    L.SpB_VNEC_mlp_free_ext.restype = None
    L.SpB_VNEC_mlp_num_params_ext.argtypes = []
    L.SpB_VNEC_mlp_num_params_ext.restype = C.c_int
    L.SpB_VNEC_mlp_params_ext.argtypes = [_vp, _vp, C.c_int]
    L.SpB_VNEC_mlp_params_ext.restype = C.c_int
    L.SpB_VNEC_mlp_predict_ext.argtypes = [_vp, _vp, C.c_int, _vp]
    L.SpB_VNEC_mlp_predict_ext.restype = C.c_int
    L.SpB_VNEC_mlp_grad_ext.argtypes = [_vp, _vp, _vp, _vp, C.c_int, _f, _vp]
    L.SpB_VNEC_mlp_grad_ext.restype = C.c_int
    L.SpB_VNEC_mlp_train_ext.argtypes = [_vp, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_float, C.c_float,
                                         C.c_uint64, _vp]
    L.SpB_VNEC_mlp_train_ext.restype = C.c_int
    L.SpB_VNEC_builtin_model_ext.argtypes = [_vp, _vp]
    L.SpB_VNEC_builtin_model_ext.restype = C.c_int
    L._vnec_typed = True
    return L


def last_error() -> str:
    return lib().SpB_VNEC_last_error_ext().decode()


def _check(ok: bool, what: str) -> None:
    if not ok:
        raise VnecError(f"{what}: {last_error()}")


class Matrix:
    """A CSR matrix in the reference's object layout (64-bit offsets/columns)."""

    def __init__(self, n_rows: int, n_cols: int, row_ptr, col, val, dtype=np.float64):
        self.ptr = np.ascontiguousarray(row_ptr, dtype=np.uint64)
        self.indices = np.ascontiguousarray(col, dtype=np.uint64)
        self.val = np.ascontiguousarray(val, dtype=dtype)
        if self.ptr.shape != (n_rows + 1,):
            raise ValueError("row_ptr must have n_rows + 1 entries")
        nnz = int(self.ptr[-1]) if n_rows >= 0 else 0
        self.type = SpB_FP64 if self.val.dtype == np.float64 else SpB_FP32
        s = _CsrStruct()
        s.matrix_base.element_type = self.type
        s.matrix_base.format_type = SpB_CSR
        s.matrix_base.row = n_rows
        s.matrix_base.col = n_cols
        s.matrix_base.element_size = self.val.itemsize
        s.val = self.val.ctypes.data
        s.indices = self.indices.ctypes.data_as(C.POINTER(C.c_uint64))
        s.ptr = self.ptr.ctypes.data_as(C.POINTER(C.c_uint64))
        s.ptr_len = n_rows + 1
        s.nnz = nnz
        s.capacity = nnz
        self._s = s
        self.n_rows, self.n_cols, self.nnz = n_rows, n_cols, nnz

    @classmethod
    def from_csr(cls, m, dtype=np.float64) -> "Matrix":
        """From any object with n_rows, n_cols, row_ptr, col, val (e.g. generators.HostCSR)."""
        return cls(m.n_rows, m.n_cols, m.row_ptr, m.col, np.asarray(m.val).astype(dtype, copy=False), dtype=dtype)

    @property
    def handle(self) -> int:
        return C.addressof(self._s)


class Vector:
    """A dense vector in the reference's object layout (host values)."""

    def __init__(self, values=None, n: int | None = None, dtype=np.float64, pinned_buffer=None):
        if pinned_buffer is not None:
            self.values = pinned_buffer
        elif values is not None:
            self.values = np.ascontiguousarray(values, dtype=dtype)
        else:
            self.values = np.zeros(n, dtype=dtype)
        self.type = SpB_FP64 if self.values.dtype == np.float64 else SpB_FP32
        s = _DenseStruct()
        s.vector_base.element_type = self.type
        s.vector_base.format_type = SpB_DENSE
        s.vector_base.n = self.values.shape[0]
        s.vector_base.element_size = self.values.itemsize
        s.values = self.values.ctypes.data
        self._s = s

    @property
    def handle(self) -> int:
        return C.addressof(self._s)


# --- reference entry points -------------------------------------------------

def IRD_VNEC(A: Matrix, type_: int = SpB_FP64) -> int:
    r = lib().IRD_VNEC(A.handle, type_)
    _check(last_error() == "", "IRD_VNEC")
    return r


def Build_VNEC_L(A: Matrix) -> int:
    h = lib().Build_VNEC_L(A.handle)
    _check(bool(h), "Build_VNEC_L")
    return h


def SpMV_VNEC_L_FP64(y: Vector, A: Matrix, x: Vector, h: int) -> None:
    lib().SpMV_VNEC_L_FP64(y.handle, A.handle, x.handle, h)
    _check(last_error() == "", "SpMV_VNEC_L_FP64")


def SpMV_VNEC_L_FP32(y: Vector, A: Matrix, x: Vector, h: int) -> None:
    lib().SpMV_VNEC_L_FP32(y.handle, A.handle, x.handle, h)
    _check(last_error() == "", "SpMV_VNEC_L_FP32")


def VNEC_L_free(h: int) -> None:
    lib().VNEC_L_free_ext(h)


def Build_VNEC_S_FP64(A: Matrix) -> int:
    h = lib().Build_VNEC_S_FP64(A.handle)
    _check(bool(h), "Build_VNEC_S_FP64")
    return h


def Build_VNEC_S_FP32(A: Matrix) -> int:
    h = lib().Build_VNEC_S_FP32(A.handle)
    _check(bool(h), "Build_VNEC_S_FP32")
    return h


def SpMV_VNEC_S_FP64(y: Vector, A: Matrix, x: Vector, h: int) -> None:
    lib().SpMV_VNEC_S_FP64(y.handle, A.handle, x.handle, h)
    _check(last_error() == "", "SpMV_VNEC_S_FP64")


def SpMV_VNEC_S_FP32(y: Vector, A: Matrix, x: Vector, h: int) -> None:
    lib().SpMV_VNEC_S_FP32(y.handle, A.handle, x.handle, h)
    _check(last_error() == "", "SpMV_VNEC_S_FP32")


def Build_VNEC_D_FP64(A: Matrix) -> int:
    h = lib().Build_VNEC_D_FP64(A.handle)
    _check(bool(h), "Build_VNEC_D_FP64")
    return h


def Build_VNEC_D_FP32(A: Matrix) -> int:
    h = lib().Build_VNEC_D_FP32(A.handle)
    _check(bool(h), "Build_VNEC_D_FP32")
    return h


def SpMV_VNEC_D_FP64(y: Vector, A: Matrix, x: Vector, h: int) -> None:
    lib().SpMV_VNEC_D_FP64(y.handle, A.handle, x.handle, h)
    _check(last_error() == "", "SpMV_VNEC_D_FP64")


def SpMV_VNEC_D_FP32(y: Vector, A: Matrix, x: Vector, h: int) -> None:
    lib().SpMV_VNEC_D_FP32(y.handle, A.handle, x.handle, h)
    _check(last_error() == "", "SpMV_VNEC_D_FP32")


def VNEC_D_free_fp64(h: int) -> None:
    lib().VNEC_D_free_fp64(h)


def VNEC_D_free_fp32(h: int) -> None:
    lib().VNEC_D_free_fp32(h)


def VNEC_S_free_fp64(h: int) -> None:
    lib().VNEC_S_free_fp64(h)


def VNEC_S_free_fp32(h: int) -> None:
    lib().VNEC_S_free_fp32(h)


def SpB_mxv(y: Vector, A: Matrix, x: Vector, vnec: int | None = None) -> None:
    _check(lib().SpB_mxv(y.handle, A.handle, x.handle, vnec) == SpB_SUCCESS, "SpB_mxv")


# --- extensions ---------------------------------------------------------------

def options(kernel: int = KERNEL_AUTO, threads_per_block: int = 0, items_per_thread: int = 0,
            pipeline_stages: int = 0, arithmetic: int = ARITH_AUTO, window_rows: int = 0, long_row_len: int = 0,
            max_steps: int = 0, cache_hints: int = 0, precision: int = PREC_FP64, hot_columns: int = 0,
            dense_fill_permille: int = 0, transpose: bool = False, host_parts: int = 0,
            column_deltas: int = 0, lane_vectors: int = 0, hot_order: int = 0, offsets64: int = 0,
            shared_patterns: int = 0, l2_prefetch: int = 0) -> Options:
    o = Options()
    o.kernel, o.threads_per_block, o.items_per_thread = kernel, threads_per_block, items_per_thread
    o.pipeline_stages, o.arithmetic = pipeline_stages, arithmetic
    o.window_rows, o.long_row_len, o.max_steps = window_rows, long_row_len, max_steps
    o.cache_hints, o.precision, o.hot_columns = cache_hints, precision, hot_columns
    o.dense_fill_permille = dense_fill_permille
    o.transpose = int(transpose)
    o.host_parts = host_parts
    o.column_deltas = column_deltas
    o.lane_vectors = lane_vectors
    o.hot_order = hot_order
    o.offsets64 = offsets64
    o.shared_patterns = shared_patterns
    o.l2_prefetch = l2_prefetch
    return o


class Plan:
    """An owned plan (any kernel) built from raw CSR arrays or a Matrix."""

    def __init__(self, csr=None, *, matrix: Matrix | None = None, dtype=np.float64, opts: Options | None = None,
                 **kw):
        o = opts or options(**kw)
        L = lib()
        if matrix is not None:
            h = L.SpB_VNEC_plan_matrix_ext(C.byref(o), matrix.handle)
            self.type = matrix.type
        else:
            rp = np.ascontiguousarray(csr.row_ptr, dtype=np.int64)
            ci = np.ascontiguousarray(csr.col, dtype=np.int32)
            vv = np.ascontiguousarray(csr.val, dtype=dtype)
            self.type = SpB_FP64 if vv.dtype == np.float64 else SpB_FP32
            h = L.SpB_VNEC_plan_ext(C.byref(o), self.type, csr.n_rows, csr.n_cols, rp.ctypes.data,
                                    ci.ctypes.data, vv.ctypes.data)
        _check(bool(h), "plan")
        self.h = h
        self.dtype = _DTYPE[self.type]

    def info(self) -> Info:
        inf = Info()
        _check(lib().SpB_VNEC_plan_info_ext(self.h, C.byref(inf)) == SpB_SUCCESS, "plan_info")
        return inf

    def mxv_device(self, d_x: int, d_y: int, stream: int = 0) -> None:
        """y = A x for device pointers (e.g. torch tensor data_ptr()) on a CUDA stream."""
        _check(lib().SpB_mxv_device_ext(self.h, d_x, d_y, stream or None) == SpB_SUCCESS, "SpB_mxv_device_ext")

    def mxv_axpby(self, d_x: int, d_y: int, alpha: float = 1.0, beta: float = 0.0, d_z: int = 0,
                  gamma: float = 0.0, stream: int = 0) -> None:
        """y = alpha * A x + beta * z + gamma on device pointers (z may be y)."""
        _check(lib().SpB_mxv_axpby_ext(self.h, d_x, d_y, alpha, beta, d_z or None, gamma, stream or None)
               == SpB_SUCCESS, "SpB_mxv_axpby_ext")

    def mxv_axpbyg(self, d_x: int, d_y: int, alpha: float = 1.0, beta: float = 0.0, d_z: int = 0,
                   gamma: float = 0.0, d_g: int = 0, g_scale: float = 0.0, stream: int = 0) -> None:
        """y = alpha * A x + beta * z + gamma + g_scale * (*d_g), d_g a device double."""
        _check(lib().SpB_mxv_axpbyg_ext(self.h, d_x, d_y, alpha, beta, d_z or None, gamma, d_g or None, g_scale,
                                        stream or None) == SpB_SUCCESS, "SpB_mxv_axpbyg_ext")

    def _host_sizes(self) -> tuple[int, int]:
        """Values of x and of y one host-vector call copies (n_cols and n_rows
        times the right-hand sides)."""
        inf = self.info()
        r = max(int(inf.rhs), 1)
        return inf.n_cols * r, inf.n_rows * r

    def _check_y(self, y: np.ndarray, ny: int) -> None:
        if y.dtype != self.dtype or not y.flags.c_contiguous or not y.flags.writeable or y.size != ny:
            raise ValueError(f"y must be a writeable contiguous array of {ny} values of the plan's value type")

    def mxv_host(self, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
        nx, ny = self._host_sizes()
        x = np.ascontiguousarray(x, dtype=self.dtype)
        if x.size != nx:
            raise ValueError(f"x must hold {nx} values")
        if y is None:
            y = np.empty(ny, dtype=self.dtype)
        self._check_y(y, ny)
        _check(lib().SpB_mxv_host_ext(self.h, x.ctypes.data, y.ctypes.data) == SpB_SUCCESS, "SpB_mxv_host_ext")
        return y

    def mxv_host_async(self, x: np.ndarray, y: np.ndarray) -> None:
        """Enqueues y := A x on the pipelined host path (SpB_mxv_host_async_ext);
        x and y are contiguous arrays of the plan's type, left untouched until
        host_wait() returns (the plan holds references to them until then)."""
        nx, ny = self._host_sizes()
        if x.dtype != self.dtype or not x.flags.c_contiguous or x.size != nx:
            raise ValueError(f"x must be a contiguous array of {nx} values of the plan's value type")
        self._check_y(y, ny)
        _check(lib().SpB_mxv_host_async_ext(self.h, x.ctypes.data, y.ctypes.data) == SpB_SUCCESS,
               "SpB_mxv_host_async_ext")
        self.__dict__.setdefault("_in_flight", []).append((x, y))

    def host_wait(self) -> None:
        try:
            _check(lib().SpB_VNEC_host_wait_ext(self.h) == SpB_SUCCESS, "SpB_VNEC_host_wait_ext")
        finally:
            self.__dict__.pop("_in_flight", None)

    def spmspv_host(self, idx: np.ndarray, val: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
        """y = A x for sparse x (push plans): idx int32 positions, val values."""
        idx = np.ascontiguousarray(idx, dtype=np.int32)
        val = np.ascontiguousarray(val, dtype=self.dtype)
        if y is None:
            y = np.empty(self.info().n_rows, dtype=self.dtype)
        _check(lib().SpB_VNEC_spmspv_host_ext(self.h, idx.size, idx.ctypes.data, val.ctypes.data, y.ctypes.data)
               == SpB_SUCCESS, "SpB_VNEC_spmspv_host_ext")
        return y

    def spmspv_device(self, nnz_x: int, d_idx: int, d_val: int, d_y: int, stream: int = 0) -> None:
        _check(lib().SpB_VNEC_spmspv_ext(self.h, nnz_x, d_idx, d_val, d_y, stream or None) == SpB_SUCCESS,
               "SpB_VNEC_spmspv_ext")

    def device_status(self, stream: int = 0) -> None:
        """Raises VnecError if a bounded device wait of this plan timed out."""
        _check(lib().SpB_VNEC_device_status_ext(self.h, stream or None) == SpB_SUCCESS, "device_status")

    def set_wait_polls(self, polls: int = -1) -> None:
        """Poll limit of the plan's bounded device waits (< 0: default; 0: give
        up at the first wait)."""
        _check(lib().SpB_VNEC_wait_polls_ext(self.h, polls) == SpB_SUCCESS, "wait_polls")

    def set_profiling(self, on: bool = True) -> None:
        _check(lib().SpB_VNEC_set_profiling_ext(self.h, int(on)) == SpB_SUCCESS, "set_profiling")

    def kernel_ms(self) -> list[float]:
        buf = (C.c_float * 8)()
        n = lib().SpB_VNEC_kernel_ms_ext(self.h, buf, 8)
        return [buf[i] for i in range(n)]

    def free(self) -> None:
        if self.h:
            lib().SpB_VNEC_plan_free_ext(self.h)  # waits for pipelined calls in flight
            self.h = None
        self.__dict__.pop("_in_flight", None)

    def __del__(self):  # pragma: no cover
        try:
            self.free()
        except Exception:
            pass


def batch_options(precision: int = PREC_FP64, lanes: int = 0, long_row_len: int = 0, chunk: int = 0,
                  warps_per_block: int = 0, autotune: bool = False, graph: bool = True,
                  window_rows: int = 0, max_steps: int = 0, unroll: int = 0, host_parts: int = 0,
                  dispatch: int = 0, k1_layout: int = 0) -> BatchOptions:
    o = BatchOptions()
    o.max_steps, o.unroll, o.host_parts, o.dispatch = max_steps, unroll, host_parts, dispatch
    o.k1_layout = k1_layout
    o.precision, o.lanes, o.long_row_len, o.chunk = precision, lanes, long_row_len, chunk
    o.warps_per_block, o.autotune, o.no_graph, o.window_rows = warps_per_block, int(autotune), int(not graph), \
        window_rows
    return o


class BatchPlan(Plan):
    """Batched multi-right-hand-side plan: Y_m = A_m X_m for a list of FP64 CSR
    matrices (objects with n_rows, n_cols, row_ptr, col, val) or Matrix objects,
    with k right-hand sides; x / y of the calls are the row-major concatenations."""

    def __init__(self, mats, k: int, *, opts: BatchOptions | None = None, **kw):  # noqa: D107
        o = opts or batch_options(**kw)
        L = lib()
        n = len(mats)
        if n and isinstance(mats[0], Matrix):
            arr = (C.c_void_p * n)(*[m.handle for m in mats])
            h = L.SpB_VNEC_batch_plan_matrices_ext(n, arr, k, C.byref(o))
        else:
            keep = []
            nr = np.array([m.n_rows for m in mats], dtype=np.int64)
            nc = np.array([m.n_cols for m in mats], dtype=np.int64)
            rps, cis, vls = (C.c_void_p * n)(), (C.c_void_p * n)(), (C.c_void_p * n)()
            for i, m in enumerate(mats):
                rp = np.ascontiguousarray(m.row_ptr, dtype=np.int64)
                ci = np.ascontiguousarray(m.col, dtype=np.int32)
                vv = np.ascontiguousarray(m.val, dtype=np.float64)
                keep += [rp, ci, vv]
                rps[i], cis[i], vls[i] = rp.ctypes.data, ci.ctypes.data, vv.ctypes.data
            h = L.SpB_VNEC_batch_plan_ext(n, nr.ctypes.data, nc.ctypes.data, rps, cis, vls, k, C.byref(o))
        _check(bool(h), "batch plan")
        self.h = h
        self.type = SpB_FP64
        self.dtype = np.float64
        self.k = k
        self.n_mats = n

    def offsets(self) -> tuple[np.ndarray, np.ndarray]:
        """Row and column offsets of each matrix (n_mats + 1 each, in rows of k values)."""
        ro = np.zeros(self.n_mats + 1, dtype=np.int64)
        co = np.zeros(self.n_mats + 1, dtype=np.int64)
        _check(lib().SpB_VNEC_batch_offsets_ext(self.h, ro.ctypes.data, co.ctypes.data) == SpB_SUCCESS,
               "batch_offsets")
        return ro, co

    def mxv_host(self, x: np.ndarray, y: np.ndarray | None = None) -> np.ndarray:
        inf = self.info()
        x = np.ascontiguousarray(x, dtype=np.float64)
        if x.size != inf.n_cols * self.k:
            raise ValueError("x must hold n_cols * k values")
        if y is None:
            y = np.empty((inf.n_rows, self.k), dtype=np.float64)
        self._check_y(y, inf.n_rows * self.k)
        _check(lib().SpB_mxv_host_ext(self.h, x.ctypes.data, y.ctypes.data) == SpB_SUCCESS, "SpB_mxv_host_ext")
        return y

    def tuning(self) -> tuple[list[tuple[int, int, int, int]], list[float], int]:
        """Autotuner record: candidates (lanes, long_row_len, warps_per_block, deep unroll), median ms, chosen index."""
        cap = 256
        cfg = (C.c_int * (4 * cap))()
        ms = (C.c_float * cap)()
        best = C.c_int(-1)
        n = lib().SpB_VNEC_batch_tuning_ext(self.h, cfg, ms, cap, C.byref(best))
        _check(n >= 0, "batch_tuning")
        n = min(n, cap)
        return ([(cfg[4 * i], cfg[4 * i + 1], cfg[4 * i + 2], cfg[4 * i + 3]) for i in range(n)],
                [ms[i] for i in range(n)], best.value)


# --- kernel selection ---------------------------------------------------------

NUM_FEATURES = 16


def tune_configs() -> list[tuple[int, int, int]]:
    """(kernel, chunk, dense-fill permille) of every tuner configuration."""
    n = lib().SpB_VNEC_tune_configs_ext(None, None, None, 0)
    k, c, p = (C.c_int * n)(), (C.c_int * n)(), (C.c_int * n)()
    lib().SpB_VNEC_tune_configs_ext(k, c, p, n)
    return [(k[i], c[i], p[i]) for i in range(n)]


def _csr_args(csr):
    rp = np.ascontiguousarray(csr.row_ptr, dtype=np.int64)
    ci = np.ascontiguousarray(csr.col, dtype=np.int32)
    vv = np.ascontiguousarray(csr.val, dtype=np.float64)
    return rp, ci, vv


def features(csr) -> np.ndarray:
    """The 16 selection features of a CSR matrix, computed on the GPU."""
    rp, ci, _ = _csr_args(csr)
    out = np.zeros(NUM_FEATURES, dtype=np.float32)
    _check(lib().SpB_VNEC_features_ext(csr.n_rows, csr.n_cols, rp.ctypes.data, ci.ctypes.data, out.ctypes.data)
           == SpB_SUCCESS, "SpB_VNEC_features_ext")
    return out


def autotune(csr, reps: int = 5, opts: Options | None = None) -> tuple[np.ndarray, int]:
    """Exhaustive autotune: median ms of every configuration (inf where unavailable), best index."""
    rp, ci, vv = _csr_args(csr)
    n = len(tune_configs())
    ms = np.zeros(n, dtype=np.float32)
    o = opts or options()
    best = lib().SpB_VNEC_autotune_ext(C.byref(o), SpB_FP64, csr.n_rows, csr.n_cols, rp.ctypes.data, ci.ctypes.data,
                                       vv.ctypes.data, reps, ms.ctypes.data)
    _check(best >= 0, "SpB_VNEC_autotune_ext")
    ms = ms.astype(np.float64)
    ms[ms >= np.finfo(np.float32).max] = np.inf
    return ms, best


def time_configs(csr, configs, reps: int = 5, opts: Options | None = None) -> np.ndarray:
    """Median ms of the listed configurations only (inf where unavailable), same protocol as `autotune`."""
    rp, ci, vv = _csr_args(csr)
    cfg = np.ascontiguousarray(configs, dtype=np.int32)
    ms = np.zeros(len(cfg), dtype=np.float32)
    o = opts or options()
    rc = lib().SpB_VNEC_time_configs_ext(C.byref(o), SpB_FP64, csr.n_rows, csr.n_cols, rp.ctypes.data,
                                         ci.ctypes.data, vv.ctypes.data, reps, cfg.ctypes.data, len(cfg),
                                         ms.ctypes.data)
    _check(rc == 0, "SpB_VNEC_time_configs_ext")
    ms = ms.astype(np.float64)
    ms[ms >= np.finfo(np.float32).max] = np.inf
    return ms


DOT_BLOCKS = 1024  # SPB_VNEC_DOT_BLOCKS


def dot(n: int, d_a: int, d_b: int, mode: int, d_partial: int, d_out: int, stream: int = 0) -> None:
    """d_out[0] = sum a*b (mode 0) or sum |a - b| (mode 1) over n device doubles,
    in a fixed order; d_partial holds DOT_BLOCKS doubles of scratch."""
    _check(lib().SpB_VNEC_dot_ext(n, d_a, d_b, mode, d_partial, d_out, stream or None) == SpB_SUCCESS,
           "SpB_VNEC_dot_ext")


STREAM_GATHER_BLOCKS = 4096  # SPB_VNEC_STREAM_GATHER_BLOCKS


def stream_gather(d_x: int, n_x: int, d_col: int, d_val: int, n: int, d_out: int, stream: int = 0) -> None:
    """The measurement kernel: sum of val[i] * x[col[i]] over n items, as
    STREAM_GATHER_BLOCKS partial sums in d_out (device pointers)."""
    _check(lib().SpB_VNEC_stream_gather_ext(d_x, n_x, d_col, d_val, n, d_out, stream or None) == SpB_SUCCESS,
           "SpB_VNEC_stream_gather_ext")


def rule_choice(csr) -> int:
    rp, ci, vv = _csr_args(csr)
    c = lib().SpB_VNEC_rule_choice_ext(SpB_FP64, csr.n_rows, csr.n_cols, rp.ctypes.data, ci.ctypes.data,
                                       vv.ctypes.data)
    _check(c >= 0, "SpB_VNEC_rule_choice_ext")
    return c


def learned_choice(csr) -> tuple[int, np.ndarray, bool]:
    """Built-in model's choice, its predicted relative costs and the out-of-range flag."""
    rp, ci, vv = _csr_args(csr)
    n = len(tune_configs())
    pred = np.zeros(n, dtype=np.float32)
    ood = C.c_int(0)
    c = lib().SpB_VNEC_learned_choice_ext(SpB_FP64, csr.n_rows, csr.n_cols, rp.ctypes.data, ci.ctypes.data,
                                          vv.ctypes.data, pred.ctypes.data, C.byref(ood))
    _check(c >= 0, "SpB_VNEC_learned_choice_ext")
    return c, pred, bool(ood.value)


def plan_choice(plan: "Plan") -> tuple[int, int]:
    cfg, how = C.c_int(-1), C.c_int(0)
    _check(lib().SpB_VNEC_plan_choice_ext(plan.h, C.byref(cfg), C.byref(how)) == SpB_SUCCESS, "plan_choice")
    return cfg.value, how.value


def builtin_model() -> tuple[np.ndarray, np.ndarray] | None:
    n = lib().SpB_VNEC_mlp_num_params_ext()
    p = np.zeros(n, dtype=np.float32)
    r = np.zeros(2 * NUM_FEATURES, dtype=np.float32)
    if not lib().SpB_VNEC_builtin_model_ext(p.ctypes.data, r.ctypes.data):
        return None
    return p, r.reshape(NUM_FEATURES, 2)


class Mlp:
    """The selection MLP, trained and evaluated by the library's CUDA kernels."""

    def __init__(self, seed: int = 0):
        self.h = lib().SpB_VNEC_mlp_create_ext(seed)
        _check(bool(self.h), "SpB_VNEC_mlp_create_ext")
        self.n_params = lib().SpB_VNEC_mlp_num_params_ext()
        self.n_out = len(tune_configs())

    @property
    def params(self) -> np.ndarray:
        p = np.zeros(self.n_params, dtype=np.float32)
        _check(lib().SpB_VNEC_mlp_params_ext(self.h, p.ctypes.data, 0) == SpB_SUCCESS, "mlp_params")
        return p

    @params.setter
    def params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.n_params
        _check(lib().SpB_VNEC_mlp_params_ext(self.h, p.ctypes.data, 1) == SpB_SUCCESS, "mlp_params")

    def predict(self, X: np.ndarray) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        out = np.zeros((X.shape[0], self.n_out), dtype=np.float32)
        _check(lib().SpB_VNEC_mlp_predict_ext(self.h, X.ctypes.data, X.shape[0], out.ctypes.data) == SpB_SUCCESS,
               "mlp_predict")
        return out

    def loss_grad(self, X, T, M) -> tuple[float, np.ndarray]:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        M = np.ascontiguousarray(M, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = C.c_float(0)
        _check(lib().SpB_VNEC_mlp_grad_ext(self.h, X.ctypes.data, T.ctypes.data, M.ctypes.data, X.shape[0],
                                           C.byref(loss), g.ctypes.data) == SpB_SUCCESS, "mlp_grad")
        return loss.value, g

    def train(self, X, T, M, epochs=300, batch=64, lr=2e-3, weight_decay=1e-4, seed=1) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32)
        T = np.ascontiguousarray(T, dtype=np.float32)
        M = np.ascontiguousarray(M, dtype=np.float32)
        curve = np.zeros(epochs, dtype=np.float32)
        _check(lib().SpB_VNEC_mlp_train_ext(self.h, X.ctypes.data, T.ctypes.data, M.ctypes.data, X.shape[0], epochs,
                                            batch, lr, weight_decay, seed, curve.ctypes.data) == SpB_SUCCESS,
               "mlp_train")
        return curve

    def free(self) -> None:
        if self.h:
            lib().SpB_VNEC_mlp_free_ext(self.h)
            self.h = None

    def __del__(self):  # pragma: no cover
        try:
            self.free()
        except Exception:
            pass
