/*
 * vnec_gb300 — GB300 (sm_103a) implementation of the OpenSparseBLAS VNEC mxv
 * (sparse matrix x dense vector) path, behind the reference's own C API.
 *
 * Drop-in use: link libvnec_gb300.so in place of the reference's operation
 * module; the reference's core objects (SpB_Matrix in CSR, dense SpB_Vector)
 * are read in place.  Each entry point below names the reference declaration
 * it replaces.  Functions with the _ext suffix are additions of this library.
 *
 * Semantics shared by all SpMV entry points: y := A x (overwrite, no
 * accumulate), as in the reference kernels (spmv_vnec_L_for_mxv.c:145,
 * spmv_vnec_D_for_mxv.c:452).  A handle is built once from A and uploads A to
 * the GPU; the host-vector entry points copy x to the device and y back on
 * every call.  Errors never exit the process: functions returning SpB_Info
 * report SpB_FAILURE, void functions of the reference signature record the
 * error, and SpB_VNEC_last_error_ext() returns the message of the calling
 * thread's last failure.
 */
#ifndef VNEC_GB300_H
#define VNEC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifndef VNEC_HAVE_OPENSPARSEBLAS_H
#include "vnec_spb_types.h"
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ------------------------------------------------------------------------ */
/* Reference entry points                                                    */
/* ------------------------------------------------------------------------ */

/* include/OpenSparseBLAS.h:1951 (declared there, body commented out in
 * src/operation/src/SpB_mxv.c:28-35).  y := A x.  VNEC is a handle returned by
 * any Build_VNEC_* or SpB_VNEC_plan_ext of this library, or NULL: then a plan
 * for A is built with the automatic selection and cached against A (the cache
 * is keyed by A and its array pointers; call SpB_VNEC_forget_ext(A) after
 * changing A in place). */
SpB_Info SpB_mxv(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, void *VNEC);

/* include/OpenSparseBLAS.h:1983 (ird_calc.c:2-122).  Returns SpB_VNEC_D when
 * nnz / (blocks * nLanes) >= threshold, else SpB_VNEC_S, computed exactly as
 * the reference's x86 build does (36 merge-path partitions, nLanes 8/16 and
 * thresholds 0.477/0.437 for FP64/FP32, SpB_mxv.h:25-32).  Does not print.
 * Like the reference (ird_calc.c:103, `int _nnz_ = v_row_ptr[n] * nLanes`),
 * the denominator blocks x nLanes is a 32-bit int: past 2^31 - 1 (about
 * 2.7e8 blocks at nLanes 8 — the 27-point stencil on 256^3 has more) it
 * wraps as the reference's does, so the ratio, and the choice, of such a
 * matrix is the reference's wrapped one, not a meaningful IRD.  The
 * reference's harness never asks for it there (it sends every matrix of
 * 3e6 rows or more to VNEC-L). */
SpB_VNEC_type IRD_VNEC(const SpB_Matrix A, SpB_Type type);

/* include/OpenSparseBLAS.h:2023 (spmv_vnec_L_for_mxv.c:2-35).  Merge-path plan
 * for A (FP64 or FP32 values) below 2^26 nonzeros; from 2^26 nonzeros on, the
 * plan of the automatic selection (the one SpB_mxv builds for a NULL handle),
 * because the reference's harness sends every matrix of 3e6 rows or more to
 * VNEC-L and the merge-path kernel is the slower plan at those sizes (R-MAT
 * 2^24: 2.30 vs 0.92 ms).  Either way SpMV_VNEC_L_* computes y := A x within
 * the same error bound; SpB_VNEC_plan_ext with kernel SpB_VNEC_KERNEL_L gives
 * a merge-path plan of any size.  The public fields num_merge_items and
 * items_per_thread are filled; the pointer fields are NULL.  Release with
 * VNEC_L_free_ext (or the harness's field-by-field free, which leaks the
 * device plan). */
struct VNEC_L *Build_VNEC_L(const SpB_Matrix A);

/* include/OpenSparseBLAS.h:2024 and :2073 (spmv_vnec_L_for_mxv.c:36-165). */
void SpMV_VNEC_L_FP32(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, VNEC_L *mat_thd);
void SpMV_VNEC_L_FP64(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, VNEC_L *mat_thd);

/* include/OpenSparseBLAS.h:2071 and :2012 (spmv_vnec_S_for_mxv.c:336-588,
 * :3-334).  Sliced row-group plan: rows bucketed by length into interleaved
 * groups of 32 lanes (the reference's equal-length cross-row groups, re-derived
 * for warps), long rows split into chunks.  Pointer fields of the public
 * struct are NULL.  Release with VNEC_S_free_fp64 / VNEC_S_free_fp32. */
struct VNEC_S_FP64 *Build_VNEC_S_FP64(const SpB_Matrix A);
struct VNEC_S_FP32 *Build_VNEC_S_FP32(const SpB_Matrix A);

/* include/OpenSparseBLAS.h:2066 and :2007 (spmv_vnec_S_for_mxv.c:589-660, :255-334). */
void SpMV_VNEC_S_FP64(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, VNEC_S_FP64 *mat_thd);
void SpMV_VNEC_S_FP32(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, VNEC_S_FP32 *mat_thd);

/* include/OpenSparseBLAS.h:2043 and :1982 (spmv_vnec_D_for_mxv.c:242-398,
 * :2-241).  Dense-block plan: each row cut into zero-padded blocks of 4
 * consecutive columns by the reference's grouping rule (applied to global
 * columns), laid out as warp tasks like the sliced format.  Rows must have
 * strictly increasing columns.  Release with VNEC_D_free_fp64 / _fp32. */
struct VNEC_D_FP64 *Build_VNEC_D_FP64(const SpB_Matrix A);
struct VNEC_D_FP32 *Build_VNEC_D_FP32(const SpB_Matrix A);

/* include/OpenSparseBLAS.h:2038 and :1977 (spmv_vnec_D_for_mxv.c:400-485, :185-241). */
void SpMV_VNEC_D_FP64(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, VNEC_D_FP64 *mat_thd);
void SpMV_VNEC_D_FP32(SpB_Vector y, const SpB_Matrix A, const SpB_Vector x, VNEC_D_FP32 *mat_thd);

/* ------------------------------------------------------------------------ */
/* Handle release (the reference frees handles field by field in its test    */
/* code, src/operation/test/test_spmv_vnec.hpp:81-176 and                     */
/* test_spmv_vnec.cpp:248-253; these library functions replace that).        */
/* ------------------------------------------------------------------------ */
void VNEC_L_free_ext(VNEC_L *mat_thd);
void VNEC_S_free_fp64(VNEC_S_FP64 *mat_thd);
void VNEC_S_free_fp32(VNEC_S_FP32 *mat_thd);
void VNEC_D_free_fp64(VNEC_D_FP64 *mat_thd);
void VNEC_D_free_fp32(VNEC_D_FP32 *mat_thd);

/* ------------------------------------------------------------------------ */
/* Extensions                                                                */
/* ------------------------------------------------------------------------ */

/* Message of the calling thread's last failure ("" if none). */
const char *SpB_VNEC_last_error_ext(void);

/* Plan construction options (zero-initialise for defaults). */
typedef enum {
  SpB_VNEC_KERNEL_AUTO = 0, /* LEARNED when the library carries a trained model, else RULE */
  SpB_VNEC_KERNEL_L = 1, /* merge-path CSR */
  SpB_VNEC_KERNEL_D = 2, /* windowed dense blocks */
  SpB_VNEC_KERNEL_S = 3, /* windowed sliced rows */
  SpB_VNEC_KERNEL_BATCH = 4, /* batched multi-right-hand-side plans (SpB_VNEC_batch_plan_ext) */
  SpB_VNEC_KERNEL_HYBRID = 5, /* rows split by dense-block fill: dense blocks (D) / sliced rows (S) */
  SpB_VNEC_KERNEL_LEARNED = 6, /* configuration predicted by the built-in MLP from matrix features;
                                  exhaustive search for matrices outside its training range */
  SpB_VNEC_KERNEL_SEARCH = 7,  /* exhaustive autotune: every configuration built and timed */
  SpB_VNEC_KERNEL_RULE = 8,    /* the reference harness's rule: L for >= 3e6 rows, else IRD_VNEC's D or S */
  SpB_VNEC_KERNEL_PUSH = 9     /* push-side SpMSpV plan: A held as CSC (SpB_VNEC_spmspv_ext) */
} SpB_VNEC_kernel_ext;

/* How a tuned plan's configuration was chosen (SpB_VNEC_plan_choice_ext). */
typedef enum {
  SpB_VNEC_CHOSEN_DIRECT = 0,   /* built with an explicit kernel */
  SpB_VNEC_CHOSEN_LEARNED = 1,  /* the MLP's prediction */
  SpB_VNEC_CHOSEN_SEARCH = 2,   /* exhaustive autotune (requested) */
  SpB_VNEC_CHOSEN_RULE = 3,     /* the reference's rule */
  SpB_VNEC_CHOSEN_FALLBACK = 4  /* exhaustive autotune after the learned choice declined */
} SpB_VNEC_chosen_ext;

/* Arithmetic of the FP64 merge-path kernel. */
typedef enum {
  SpB_VNEC_ARITH_AUTO = 0, /* DF32 when A's values allow it, else FP64 */
  SpB_VNEC_ARITH_FP64 = 1, /* one FP64 FMA per nonzero */
  SpB_VNEC_ARITH_DF32 = 2  /* double-float on the FP32 pipe: products and sums
                              with ~2^-46 relative error, needs |a|,|x| in
                              [2^-40, 2^41) or 0, else the call runs in FP64 */
} SpB_VNEC_arith_ext;

typedef struct {
  int kernel;            /* SpB_VNEC_kernel_ext */
  int threads_per_block; /* 0: default */
  int items_per_thread;  /* 0: default; sliced plans: load steps in flight 4/8/12/16,
                            0 or -1: each timed on the matrix at plan build (y is
                            the same at every value) */
  int pipeline_stages;   /* merge-path: 0 default (2), 1 unpipelined kernel, 2-3 stages */
  int arithmetic;        /* SpB_VNEC_arith_ext (FP64 values) */
  int window_rows;       /* sliced: rows sorted within windows of this size (0: 65536) */
  int long_row_len;      /* sliced: rows longer than this are chunked (0: 1024) */
  int max_steps;         /* sliced: max 32-wide loads per lane for a row group (0: 32) */
  int cache_hints;       /* sliced: 0 default (streaming loads), 2 explicit L1/L2 evict policies */
  int precision;         /* sliced, FP64 matrices: SpB_VNEC_precision_ext */
  int hot_columns;       /* sliced: hot-column window — the N most used columns get
                            dense slots whose x values each call gathers once
                            (0: library default, -1: off, N > 0: at most N) */
  int dense_fill_permille; /* hybrid: rows whose dense-block fill (nnz / (4 x blocks))
                              is at least this / 1000 use dense blocks (0: 500) */
  int transpose;         /* 1: the plan computes y := A^T x (the reference's SpB_TRAN0
                            descriptor, OpenSparseBLAS.h:62-72): x has n_rows entries,
                            y n_cols; any kernel, built on A's transpose */
  int host_parts;        /* sliced FP64 plans: host-vector calls run in this many parts so
                            that y copies overlap the SpMV (0: 8, 1: one part) */
  int column_deltas;     /* sliced: store the columns of one-row-per-lane groups as 16-bit
                            deltas where the gaps allow (0: on unless a hot-column window
                            is used, -1: off) */
  int lane_vectors;      /* sliced FP32 / BF16 forms: each lane's entries stored in runs of 4 /
                            8 consecutive steps, read as 16-byte vectors (0: where most
                            entries use 16-bit column deltas, except FP32 plans whose
                            entries sit mostly in shared-pattern tasks; 1: on, -1: off;
                            the sums are the same either way) */
  int hot_order;         /* sliced plans with a hot-column window: 0 (default) stores each
                            row's hot-window entries first, hottest first, and groups rows
                            of equal length by their hottest column, so the lanes of one
                            gather step share x lines (the row sums change order: FP64
                            results agree to rounding); -1 keeps CSR order within rows
                            (bit-identical to the plan without a window) */
  int offsets64;         /* merge-path plans: 1 stores row ends and merge coordinates as 64-bit
                            integers (always done from 2^31 - 1 rows + nonzeros on) */
  int shared_patterns;   /* sliced precision forms: groups of rows with equal length and the
                            same column gaps (stencils, banded rows) read one copy of the gaps
                            per group (0: on, -1: off; the sums are the same either way) */
  int l2_prefetch;       /* sliced plans: each warp has the L2 prefetch the stored entries (values
                            and columns) this many entries past its own task's, and the task
                            metadata the same distance ahead, so that the tasks' loads meet
                            L2 instead of HBM (0: 262,144 where most nonzeros sit in 16-bit-delta
                            row groups, i.e. local columns, off for gather-bound layouts; -1:
                            off; > 0: the distance, rounded down to a multiple of 32; the sums
                            are the same either way) */
  int reserved[4];
} SpB_VNEC_options_ext;

/* Precision forms of the sliced kernel for an FP64 matrix (x and y stay
 * FP64).  Products are accumulated in FP32 per lane; row reductions, the
 * BF16 row scale and the long-row fix-up are FP64. */
typedef enum {
  SpB_VNEC_PREC_FP64 = 0, /* plain: FP64 values, FP64 FMA */
  SpB_VNEC_PREC_FP32 = 1, /* FP32 values (4 B), x rounded to FP32 per call */
  SpB_VNEC_PREC_BF16 = 2, /* BF16 values (2 B) scaled per row by a power of two */
  SpB_VNEC_PREC_DF32 = 3  /* FP32 hi+lo split of FP64 values and x, double-float
                             sums: FP64-level error on the FP32 pipe */
} SpB_VNEC_precision_ext;

/* Plan from raw host CSR arrays: int64 row offsets (n_rows + 1), int32
 * columns and FP64/FP32 values (nnz = row_ptr[n_rows]).  The arrays are
 * copied; the caller keeps ownership.  Returns NULL on failure. */
void *SpB_VNEC_plan_ext(const SpB_VNEC_options_ext *opts, SpB_Type type, int64_t n_rows, int64_t n_cols,
                        const int64_t *row_ptr, const int32_t *col, const void *val);

/* Plan from a reference SpB_Matrix with explicit options. */
void *SpB_VNEC_plan_matrix_ext(const SpB_VNEC_options_ext *opts, const SpB_Matrix A);

/* Releases any plan or handle of this library (including Build_VNEC_*). */
void SpB_VNEC_plan_free_ext(void *plan);

/* Drops the plan SpB_mxv cached for A (no-op if none). */
void SpB_VNEC_forget_ext(const SpB_Matrix A);

/* y := A x with x and y in device memory, enqueued on `stream` (a
 * cudaStream_t; NULL = legacy default stream) without synchronising.  Value
 * type of x and y is the plan's (FP64 or FP32). */
SpB_Info SpB_mxv_device_ext(void *plan, const void *d_x, void *d_y, void *stream);

/* y := alpha * (A x) + beta * z + gamma on device vectors (iterative
 * solvers and graph analytics keep x and y on the GPU; the output transform
 * is fused into the sliced kernel's stores, an elementwise pass elsewhere).
 * z may be NULL (beta ignored) or equal to d_y (y := alpha A x + beta y). */
SpB_Info SpB_mxv_axpby_ext(void *plan, const void *d_x, void *d_y, double alpha, double beta, const void *d_z,
                           double gamma, void *stream);

/* As SpB_mxv_axpby_ext with one more additive term read on the device:
 * y := alpha * (A x) + beta * z + gamma + g_scale * (*d_g), where d_g points
 * to one double in device memory written by an earlier launch on the stream
 * (for example SpB_VNEC_dot_ext), so a power iteration needs no host round
 * trip for a data-dependent shift.  g_scale == 0 ignores d_g. */
SpB_Info SpB_mxv_axpbyg_ext(void *plan, const void *d_x, void *d_y, double alpha, double beta, const void *d_z,
                            double gamma, const double *d_g, double g_scale, void *stream);

/* Deterministic device reduction over n FP64 values, for chains of calls that
 * stay on the GPU: mode 0 writes sum_i a[i] * b[i], mode 1 sum_i |a[i] - b[i]|
 * to d_out[0].  d_partial holds SPB_VNEC_DOT_BLOCKS doubles of scratch owned
 * by the caller; the sum runs in a fixed order (identical bits run to run).
 * Enqueued on `stream`. */
#define SPB_VNEC_DOT_BLOCKS 1024
SpB_Info SpB_VNEC_dot_ext(int64_t n, const double *d_a, const double *d_b, int mode, double *d_partial,
                          double *d_out, void *stream);

/* y := A x with host x and y (the SpB_mxv data path without SpB_Vector). */
SpB_Info SpB_mxv_host_ext(void *plan, const void *h_x, void *h_y);

/* Pipelined host-vector calls for a stream of independent right-hand sides:
 * enqueues y := A x (copy x in, SpMV, copy y out) and returns without waiting.
 * Each call uses one of two device buffer slots; its x copy overlaps the
 * previous call's SpMV and its y copy the next call's, so a sequence of
 * calls runs at the rate of its slowest stage.  h_x must not change and h_y
 * must not be read until SpB_VNEC_host_wait_ext returns; page-locked host
 * buffers are needed for the copies to overlap.  Works with every plan kind.
 * A synchronous host call on the plan (SpB_mxv_host_ext, SpB_mxv) first waits
 * for the pipelined SpMVs in flight; device-pointer calls on the plan go after
 * SpB_VNEC_host_wait_ext. */
SpB_Info SpB_mxv_host_async_ext(void *plan, const void *h_x, void *h_y);
/* Waits for every enqueued pipelined call of the plan and reports device-side
 * errors (as SpB_VNEC_device_status_ext). */
SpB_Info SpB_VNEC_host_wait_ext(void *plan);

/* Plan description. */
typedef struct {
  int kernel;              /* SpB_VNEC_kernel_ext actually built */
  int value_type;          /* SpB_Type of x / y */
  int64_t n_rows, n_cols, nnz;
  int64_t device_bytes;    /* device memory held by the plan */
  int64_t algorithmic_bytes; /* bytes one SpMV must move at minimum */
  int launches_per_call;   /* kernels launched by one SpMV */
  int threads_per_block;
  int items_per_thread;
  int64_t num_tiles;
  int pipeline_stages;     /* 0 for the unpipelined kernel */
  int arithmetic;          /* SpB_VNEC_arith_ext in use */
  int64_t blocks;          /* dense-block plans: blocks of 4 columns (fill = nnz / (4 * blocks)) */
  int precision;           /* SpB_VNEC_precision_ext of a sliced or batch plan */
  int rhs;                 /* right-hand sides k (1 for single-vector plans) */
  int lanes;               /* batch plans: lanes per row (items_per_thread = k / lanes per lane);
                              0 for a k = 1 batch run as one sliced plan (items_per_thread is then
                              its unroll) */
  int long_row_len;        /* sliced and batch plans: rows longer than this are chunked */
} SpB_VNEC_info_ext;

/* Device-side error status of the plan's last calls: waits for the plan's
 * work on `stream`, returns SpB_FAILURE (with a message) if a bounded
 * pipeline wait timed out, and clears the status. */
SpB_Info SpB_VNEC_device_status_ext(void *plan, void *stream);

/* Poll limit of a plan's bounded device waits (no counterpart in the
 * reference, whose waits are OpenMP barriers).  The pipelined merge-path
 * kernel polls each pipeline stage's mbarrier at most this many times before
 * it raises the plan's device error flag, finishes the copies it has in
 * flight and exits; SpB_VNEC_device_status_ext then reports the timeout.
 * polls < 0 restores the default (2^24 polls, seconds of wall time); 0 gives
 * up at the first wait, which is how the timeout path is tested.  Plans
 * whose kernels never wait accept and ignore it.  Takes effect from the next
 * call; do not change it while a call of the plan is in flight. */
SpB_Info SpB_VNEC_wait_polls_ext(void *plan, int64_t polls);

/* Rounds n FP64 values to FP32 (round to nearest even) on `stream`; used for
 * the FP32/BF16 precision forms, exposed for callers keeping x in FP32. */
SpB_Info SpB_VNEC_f64_to_f32_ext(const double *d_in, float *d_out, int64_t n, void *stream);

/* Measurement kernel (no counterpart in the reference; no SpMV path uses it).
 * For i in [0, n) it reads d_val[i] and d_col[i] with coalesced loads,
 * gathers d_x[d_col[i]] (columns must lie in [0, n_x)) and accumulates the
 * FP64 product: the memory traffic of n CSR nonzeros without the row
 * structure.  d_out receives SPB_VNEC_STREAM_GATHER_BLOCKS partial sums.
 * Its rate on a matrix's own column stream, and on uniform random columns
 * over windows of chosen size, is the device's ceiling for kernels that
 * gather x once per nonzero (bench.py reports it beside the SpMV). */
#define SPB_VNEC_STREAM_GATHER_BLOCKS 4096
SpB_Info SpB_VNEC_stream_gather_ext(const double *d_x, int64_t n_x, const int32_t *d_col, const double *d_val,
                                    int64_t n, double *d_out, void *stream);

/* Allocation-free y := A x (no counterpart in the reference).
 *
 * For callers that cannot let a library allocate device memory: hosts whose
 * device memory is handed out entirely by their own pool allocator, and
 * latency-critical loops where a cudaMalloc/cudaFree (and the device
 * synchronisation it implies) is not acceptable.  The caller passes the CSR
 * matrix already in device memory — int32 row offsets d_row_ptr[n_rows + 1]
 * with d_row_ptr[0] == 0, non-decreasing, and d_row_ptr[n_rows] == nnz;
 * int32 columns in [0, n_cols); FP64 values — and FP64 x and y; the product
 * is enqueued on `stream` (a cudaStream_t, NULL = legacy default stream) with
 * the FP64 merge-path kernel.  Unlike a plan, this call cannot inspect the
 * device arrays: offsets that break those rules give wrong y (the kernel's
 * reads stay inside d_col[0, nnz) and d_val[0, nnz)), and a column outside
 * [0, n_cols) reads outside x.  Nothing is allocated: the kernel's scratch
 * (tile coordinates and carries) lives in a fixed 5 MiB array that every
 * device holds from library load until process exit.  Limit: n_rows, nnz and
 * n_rows + nnz each <= 469,762,048 (262,144 tiles of 1,792 merge items), and
 * n_cols <= INT32_MAX; larger inputs return SpB_FAILURE with a message.  The
 * first call in each CUDA context looks up that context's scratch address
 * (cudaGetSymbolAddress) and caches it under the context's id, so a device
 * reset or a caller's own driver context gets its own lookup; make a first
 * call in each context before any stream capture.  All calls on a device
 * share the one scratch array: calls that can overlap on the GPU (different
 * streams without ordering) race and must be serialised by the caller. */
SpB_Info SpB_mxv_csr_noalloc_ext(int64_t n_rows, int64_t n_cols, int64_t nnz, const int32_t *d_row_ptr,
                                 const int32_t *d_col, const double *d_val, const double *d_x, double *d_y,
                                 void *stream);

SpB_Info SpB_VNEC_plan_info_ext(const void *plan, SpB_VNEC_info_ext *info);

/* Push-side sparse x sparse-vector product (SpMSpV): y := A x for a sparse x
 * of nnz_x (index, value) pairs, on a plan built with kernel
 * SpB_VNEC_KERNEL_PUSH (A held as its CSC).  Replaces the reference's
 * declared-only SpB_vxm (OpenSparseBLAS.h:1940) for the push side of
 * push/pull traversal: only the columns x selects are read.  y (n_rows
 * values of the plan's type) is overwritten; additions into one y entry run
 * as atomics, so results agree with the FP64 oracle to rounding but are not
 * bit-reproducible.  An index outside [0, n_cols) is skipped and reported by
 * SpB_VNEC_device_status_ext (the host variant reports it directly).  On a
 * push plan, SpB_mxv_device_ext / SpB_mxv_host_ext take a dense x. */
SpB_Info SpB_VNEC_spmspv_ext(void *plan, int64_t nnz_x, const int32_t *d_idx, const void *d_val, void *d_y,
                             void *stream);
SpB_Info SpB_VNEC_spmspv_host_ext(void *plan, int64_t nnz_x, const int32_t *idx, const void *val, void *y);

/* ---- Kernel selection (no counterpart in the reference, which fixes the
 * choice in its test harness, test_spmv_vnec.cpp:197-245) ----
 *
 * Configuration space: SpB_VNEC_tune_configs_ext lists, per index, the kernel
 * (L or HYBRID), its chunk (L: items per thread of a 256-thread merge-path
 * tile; HYBRID: long-row chunk length) and the dense-block fill threshold in
 * permille (HYBRID; 1 = every row dense, 1001 = every row sliced).  Returns
 * the number of configurations (writes at most `cap`). */
int SpB_VNEC_tune_configs_ext(int *kernel, int *chunk, int *permille, int cap);

/* The 16 matrix features the learned choice reads, computed on the GPU from
 * host CSR arrays (int64 offsets, int32 columns). */
SpB_Info SpB_VNEC_features_ext(int64_t n_rows, int64_t n_cols, const int64_t *row_ptr, const int32_t *col,
                               float *features);

/* Exhaustive autotune: builds and times (median of `reps` calls, L2 flushed
 * before each) every configuration; ms[i] = FLT_MAX where one cannot be
 * built.  Returns the fastest index, -1 on failure.  `base` supplies the
 * other options (precision, ...), may be NULL. */
int SpB_VNEC_autotune_ext(const SpB_VNEC_options_ext *base, SpB_Type type, int64_t n_rows, int64_t n_cols,
                          const int64_t *row_ptr, const int32_t *col, const void *val, int reps, float *ms);

/* Times only the listed configurations, with the protocol of
 * SpB_VNEC_autotune_ext (the median of `reps` calls, L2 flushed before
 * each); ms[i] is the time of configs[i] (FLT_MAX where it cannot be built).
 * Used to refresh stored timings of the configurations whose kernels changed.
 * Returns 0, or -1 on invalid arguments. */
int SpB_VNEC_time_configs_ext(const SpB_VNEC_options_ext *base, SpB_Type type, int64_t n_rows, int64_t n_cols,
                              const int64_t *row_ptr, const int32_t *col, const void *val, int reps,
                              const int *configs, int n_configs, float *ms);

/* Configuration index the reference's rule and the built-in model choose
 * (the latter also writes the predicted relative costs, log2 units, and
 * whether a feature lies outside its training range).  -1 on failure or,
 * for the learned choice, when no model is built in. */
int SpB_VNEC_rule_choice_ext(SpB_Type type, int64_t n_rows, int64_t n_cols, const int64_t *row_ptr,
                             const int32_t *col, const void *val);
int SpB_VNEC_learned_choice_ext(SpB_Type type, int64_t n_rows, int64_t n_cols, const int64_t *row_ptr,
                                const int32_t *col, const void *val, float *predicted, int *out_of_range);

/* Configuration index and SpB_VNEC_chosen_ext of a plan built with kernel
 * LEARNED / SEARCH / RULE (-1 / DIRECT otherwise). */
SpB_Info SpB_VNEC_plan_choice_ext(const void *plan, int *config, int *how);

/* The selection MLP: FP32, 16 -> 64 -> 64 -> one output per configuration
 * (predicted log2 of its time over the fastest's), ReLU, trained with Adam on
 * masked squared error by the library's own CUDA kernels.  Parameters as one
 * array of SpB_VNEC_mlp_num_params_ext() floats: W1[64x16] b1 W2[64x64] b2
 * W3[Cx64] b3 (row-major, out x in). */
void *SpB_VNEC_mlp_create_ext(uint64_t seed);
void SpB_VNEC_mlp_free_ext(void *model);
int SpB_VNEC_mlp_num_params_ext(void);
SpB_Info SpB_VNEC_mlp_params_ext(void *model, float *params, int set); /* set = 0: read, 1: write */
SpB_Info SpB_VNEC_mlp_predict_ext(void *model, const float *X, int n, float *out);
/* Loss and gradient (no update) of one batch: X n x 16, targets T and mask M n x C. */
SpB_Info SpB_VNEC_mlp_grad_ext(void *model, const float *X, const float *T, const float *M, int n, float *loss,
                               float *grad);
SpB_Info SpB_VNEC_mlp_train_ext(void *model, const float *X, const float *T, const float *M, int n, int epochs,
                                int batch, float lr, float weight_decay, uint64_t seed, float *loss_curve);
/* The built-in model: returns 1 and copies its parameters and feature range
 * (min, max per feature) when the library carries one, else 0. */
int SpB_VNEC_builtin_model_ext(float *params, float *feature_range);

/* Batched multi-right-hand-side mxv (no counterpart in the reference, whose
 * SpB_mxv multiplies one matrix by one vector).
 *
 * Y_m := A_m X_m for n_mats independent FP64 CSR matrices of any sizes and k
 * right-hand sides (k = 1, 2, 4, 8, 16 or 32).  X_m is dense row-major
 * n_cols[m] x k, Y_m is n_rows[m] x k.  A plan's x and y are the
 * concatenations of the X_m and Y_m in matrix order (offsets from
 * SpB_VNEC_batch_offsets_ext, in rows of k values), so one
 * SpB_mxv_device_ext / SpB_mxv_host_ext call runs the whole batch: one
 * persistent kernel (the FP32 form adds one launch that rounds X), or for
 * k = 1 the kernels of one sliced plan of the concatenation (k1_layout),
 * replayed from a CUDA graph captured on the first call with a given (x, y)
 * pair.
 * Device x and y must be 16-byte aligned when k / lanes >= 2.  Calls on one
 * batch plan must not overlap on the GPU (they share the plan's long-row
 * scratch). */
typedef struct {
  int precision;       /* SpB_VNEC_PREC_FP64 (0), SpB_VNEC_PREC_FP32 (FP32 values and products) or
                          SpB_VNEC_PREC_DF32 (values and X as FP32 hi+lo pairs, double-float products
                          and sums on the FP32 pipe: FP64-level error; needs |a| in [2^-40, 2^41) or 0,
                          a call whose X leaves that range computes in FP64) */
  int lanes;           /* lanes per row (divides 32 and k, k / lanes in {1,2,4,8}); 0: tuned or default */
  int long_row_len;    /* rows longer than this are cut into chunks; 0: tuned or 1024 */
  int chunk;           /* entries per chunk; 0: long_row_len */
  int warps_per_block; /* 4 or 8; 0: tuned or 8 */
  int autotune;        /* 1: time candidate layouts on a sample of the batch and keep the fastest */
  int no_graph;        /* 1: launch the kernels directly on each call */
  int window_rows;     /* rows sorted by length within windows of this size (0: 65536) */
  int max_steps;       /* a row group spreads over enough slots to take at most this many steps (0: 32) */
  int unroll;          /* kernel mode: 1 normal load steps in flight per lane, 2 doubled, 3 each
                          task's columns and values read in bulk (128 per round) and passed to
                          the slots by shuffles; 0: tuned or normal */
  int host_parts;      /* host-vector calls run in this many parts so that X and Y copies overlap the
                          compute (0: 8, 1: one part) */
  int dispatch;        /* 0: default, 1: persistent warps striding the task list, 2: one warp per task
                          (blocks dispatched in task order, so the tasks in flight stay a compact window) */
  int k1_layout;       /* k = 1 only.  0 (default): the batch runs as one sliced row-group plan (the
                          SpB_VNEC_KERNEL_S layout, unroll timed at build) of the block-diagonal
                          concatenation, in the same precision form: at one right-hand side the batch
                          is one sparse matrix, and that layout's 16-bit deltas, hot-column window and
                          long-row fix-up serve it best (512 uneven matrices: FP64 2.15 -> 1.83 ms);
                          lanes, long_row_len, chunk, warps_per_block, unroll and dispatch do not apply,
                          and the plan reports lanes = 0.  -1: the batch kernel. */
  int reserved[3];
} SpB_VNEC_batch_options_ext;

/* Plan from host CSR arrays per matrix: int64 row offsets (n_rows[m] + 1),
 * int32 columns, FP64 values.  The arrays are copied.  NULL on failure. */
void *SpB_VNEC_batch_plan_ext(int n_mats, const int64_t *n_rows, const int64_t *n_cols,
                              const int64_t *const *row_ptr, const int32_t *const *col, const double *const *val,
                              int k, const SpB_VNEC_batch_options_ext *opts);

/* Plan from reference FP64 SpB_Matrix objects. */
void *SpB_VNEC_batch_plan_matrices_ext(int n_mats, const SpB_Matrix *A, int k,
                                       const SpB_VNEC_batch_options_ext *opts);

/* Row and column offsets of each matrix in the concatenation (n_mats + 1
 * entries each, in rows; multiply by k for element offsets). */
SpB_Info SpB_VNEC_batch_offsets_ext(const void *plan, int64_t *row_offset, int64_t *col_offset);

/* Autotuner result of a batch plan: candidates timed (0 if not tuned) and,
 * per candidate, {lanes, long_row_len, warps_per_block, kernel mode 0/1/2 (unroll - 1)}
 * and its median milliseconds on the sample (up to `cap` entries); *best =
 * chosen index. */
int SpB_VNEC_batch_tuning_ext(const void *plan, int *configs, float *ms, int cap, int *best);

/* Per-kernel timing: when enabled, each SpMV of the plan records CUDA events
 * around each of its kernels on the launching stream;
 * SpB_VNEC_kernel_ms_ext waits for the last call and writes up to `cap`
 * durations in milliseconds (the main kernel first).  Returns the count. */
SpB_Info SpB_VNEC_set_profiling_ext(void *plan, int enable);
int SpB_VNEC_kernel_ms_ext(const void *plan, float *ms, int cap);

#ifdef __cplusplus
}
#endif

#endif /* VNEC_GB300_H */
