// Batched multi-right-hand-side SpMV: many CSR matrices of uneven size,
// Y_m = A_m X_m for k right-hand sides (row-major X_m: n_cols x k, Y_m:
// n_rows x k), in one persistent launch over one task list.
//
// The batch is the block-diagonal concatenation of its matrices: global row
// r = row_offset[m] + local row, global column c = col_offset[m] + local
// column, so X and Y are the matrices' blocks concatenated.  Tasks follow the
// sliced layout idea (rows sorted by length, interleaved groups): L lanes
// share one (value, column) slot and each owns k/L consecutive right-hand
// sides, so a warp holds S = 32/L slots per step; a row spreads over V slots (V = 1..S chosen
// per group of rows so that a row takes at most max_steps steps) and entry j
// of group row g sits at base + (j / V) * S + g * V + j % V.
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

#include "sliced.h"

namespace vnec {

struct BatchMatrix {
  int64_t n_rows = 0, n_cols = 0, nnz = 0, entries = 0;  // of the concatenation
  int k = 1;          // right-hand sides
  int lanes = 1;      // lanes per row L (k % L == 0, 32 % L == 0)
  int64_t num_tasks = 0, num_long = 0, num_chunks = 0;
  const SlicedTask* tasks = nullptr;
  const void* val = nullptr;       // entries: double (FP64), float (FP32) or float2 hi/lo (DF32)
  const int32_t* col = nullptr;    // global columns
  const int32_t* rowid = nullptr;  // global rows
  const int32_t* long_row = nullptr;
  const int32_t* long_first = nullptr;  // num_long + 1 chunk offsets
  const int32_t* chunk_long = nullptr;  // chunk -> long row index
  double* chunk_sum = nullptr;          // num_chunks * k partial sums
  int* chunk_count = nullptr;           // num_long arrival counters, 0 between calls
  int grid = 0;                         // persistent CTAs
  bool per_task = false;                // one warp per task (blocks dispatched in task order) instead of persistent warps
  int warps_per_block = 8;
  int mode = 0;                         // 0: U steps in flight, 1: 2U, 2: entries staged in registers
  int precision = 0;                    // kPrecFP64, kPrecFP32 or kPrecDF32 (SlicedPrecision)
  void* xbuf = nullptr;                 // FP32 / DF32: n_cols * k converted X
  int* flag = nullptr;                  // DF32: X outside the split range this call
};

struct BatchParams {
  int lanes = 0;          // 0: min(k, 32) (one right-hand side per lane)
  int long_len = 1024;    // rows longer than this become chunks
  int chunk = 1024;       // entries per chunk
  int window_rows = 1 << 16;
  int max_steps = 32;     // slots per row chosen so that a row takes at most this many steps
};

struct BatchHost;
// mats: n matrices given as (n_rows, n_cols, int64 row_ptr, int32 col, FP64 val).
BatchHost* batch_build(int n, const int64_t* n_rows, const int64_t* n_cols, const int64_t* const* row_ptr,
                       const int32_t* const* col, const double* const* val, int k, const BatchParams& prm);
void batch_free(BatchHost* h);
struct BatchHostView {
  int64_t n_rows, n_cols, nnz, entries, num_tasks, num_long, num_chunks, n_rowid;
  const SlicedTask* tasks;
  const double* val;
  const int32_t* col;
  const int32_t* rowid;
  const int32_t* long_row;
  const int32_t* long_first;
  const int32_t* chunk_long;
  int lanes;
  int64_t num_windows;      // windows of window_rows global rows
  const int64_t* win_task;  // first task of each window (num_windows + 1)
  const int64_t* win_entry; // first entry of each window (num_windows + 1)
};
BatchHostView batch_view(const BatchHost* h);

// k in {1, 2, 4, ..., 32}, lanes a divisor of 32 with k / lanes in {1, 2, 4, 8}.
bool batch_supported(int k, int lanes);
// Persistent CTAs for the kernel of (precision, k / lanes, warps_per_block, mode).
int batch_grid(int precision, int rhs_per_lane, int warps_per_block, int mode);
// Y = A X for the whole batch: one persistent kernel (the FP32 form first
// rounds X into xbuf).  Long rows are finished inside the kernel by the last
// of their chunks to arrive.
bool batch_spmm(const BatchMatrix& m, const double* X, double* Y, cudaStream_t s);
// One part of a call: converts X columns [c0, c1) (FP32 / DF32 forms; `first`
// clears the DF32 range flag) and runs tasks [t0, t1).  Parts of whole windows
// write disjoint Y rows; a long row's chunks never straddle two windows.
bool batch_spmm_range(const BatchMatrix& m, const double* X, double* Y, cudaStream_t s, int64_t t0, int64_t t1,
                      int64_t c0, int64_t c1, bool first);
inline int batch_launches(const BatchMatrix& m) { return m.precision == kPrecFP64 ? 1 : 2; }

}  // namespace vnec
