// Sliced row-group format (VNEC-S counterpart) shared by the host builder
// (sliced_build.cpp) and the kernels (sliced_kernels.cu).
#pragma once

#include <cstdint>

#include <cuda_runtime.h>

namespace vnec {

// One warp task = one 16-byte descriptor.
//   kind ROWS : G = 32 >> vw_log2 rows of one group, each padded to `steps * VW`
//               entries; entry j of group row g sits at
//               base + (j / VW) * 32 + g * VW + (j % VW).  y[rowid[row_base+g]] = sum.
//   kind CHUNK: a 32*steps-entry piece of a long row (VW = 32, G = 1); the sum
//               goes to chunk_sum[row_base] and a fix-up adds the pieces.
//   kind ZERO : `nrows` empty rows, y[rowid[row_base + lane]] = 0.
enum SlicedKind : int { kSlicedRows = 0, kSlicedChunk = 1, kSlicedZero = 2 };
// meta flag of a ROWS task with VW = 1 whose columns are stored as 16-bit
// deltas: lane g starts at first[row_base + g] and adds col16[entry] at each
// step (0 on padding), so the column stream costs 2 bytes per entry instead of 4.
constexpr int kSlicedDelta = 1 << 16;
// meta flag of a delta task whose rows all have `steps` entries with the same
// deltas (stencils, banded rows): the deltas are also stored once for the task,
// step k at pat16[base / 32 + k] (step 0: 0), for kernels that read the task's
// columns as first[row_base + g] plus a per-step offset shared by all lanes.
constexpr int kSlicedShared = 1 << 17;

struct SlicedTask {
  int32_t base;      // first entry (element index into vals / cols)
  int32_t row_base;  // index into rowid (ROWS, ZERO) or chunk id (CHUNK)
  int32_t steps;     // warp-wide load steps (32 entries each)
  int32_t meta;      // kind | vw_log2 << 4 | nrows << 8
};

// The long-row fix-up sums a row of at most this many chunks in one thread
// and a longer row with a whole warp.
constexpr int kHeavyChunks = 16;
// Blocks of `threads` for the fix-up launch: one thread per long row, then
// one warp per heavy row.
struct FixupGrid {
  unsigned light, total;
};

// L2 prefetch distance of a plan (prefetch.cuh): a warp prefetches the entries
// `entries` past its task's, and the task descriptor, row slots and shared
// pattern the same distance ahead, expressed in tasks and row slots.
struct SlicedPrefetch {
  long long entries = 0;  // 0: off
  long long tasks = 0, rows = 0;
  long long n_entries = 0, n_tasks = 0, n_rows = 0;  // array bounds
};

struct SlicedMatrix {
  int64_t n_rows = 0, n_cols = 0, nnz = 0, entries = 0;  // entries include padding
  int64_t num_tasks = 0, num_long = 0, num_chunks = 0;
  const SlicedTask* tasks = nullptr;
  const void* val = nullptr;        // entries x vpe values (double or float), padding = 0
  const int32_t* col = nullptr;     // entries, padding = a valid column
  const int32_t* rowid = nullptr;   // group row slots
  const int32_t* long_row = nullptr;    // num_long rows
  const int32_t* long_first = nullptr;  // num_long + 1 chunk offsets
  // Long rows of more than kHeavyChunks chunks (indices into long_row, minus
  // heavy_sub): the fix-up sums each with a warp instead of one thread.
  const int32_t* long_heavy = nullptr;
  int64_t num_heavy = 0, heavy_sub = 0;
  void* chunk_sum = nullptr;            // num_chunks scratch (value type)
  int cache_hints = 0;                  // load cache-hint variant (sliced_kernels.cu), 0 default
  int unroll = 8;                       // load steps in flight per lane: 4, 8, 12 or 16
  int vpe = 1;                          // values per entry: 1 (nonzeros) or 4 (dense blocks)
  // Hot-column window: the `hot` most frequently used columns are relabelled
  // n_cols + slot in `col`, and each call gathers their x values into a dense
  // array (xhot for the FP64 kernel, the tail of the converted x for the
  // precision forms), so the hottest part of x occupies consecutive sectors.
  int hot = 0;
  const int32_t* hot_cols = nullptr;  // original column of each slot
  void* xhot = nullptr;               // FP64 kernel: hot x values
  bool hot_ready = false;             // xhot already gathered for this call (later parts of a split call)
  const uint16_t* col16 = nullptr;    // delta tasks (kSlicedDelta): 16-bit column deltas
  const int32_t* first = nullptr;     // delta tasks: first column of each row slot
  const uint16_t* pat16 = nullptr;    // shared-pattern tasks (kSlicedShared): one delta per step
  SlicedPrefetch pf;                  // L2 prefetch ahead of the running tasks (prefetch.cuh), off by default
  // FP32 / BF16 forms: 0, or P when val / col / col16 hold each lane's entries
  // in runs of P consecutive steps.  Steps [P*b, P*b + P) of a task's lane l
  // sit at base + b*32*P + l*P + (step - P*b), so a lane reads a run with one
  // 16-byte vector load; the last steps % P steps keep the stride-32 layout
  // (entry base + step*32 + l).
  int lane_run = 0;
};

struct SlicedParams {
  int window_rows = 1 << 16;  // rows sorted / grouped within windows of this size
  int long_len = 1024;        // rows longer than this are split into chunks
  int chunk = 1024;           // entries per chunk (multiple of 32)
  int max_steps = 32;         // target load steps per lane for grouped rows
  int hot = 0;                // hot-column window size (0: none)
  bool delta16 = false;       // 16-bit column deltas for VW = 1 groups whose rows allow it
  bool shared = false;        // delta16 layouts: also mark shared-pattern tasks (kSlicedShared)
  // Optional secondary key of the row sort (rows of equal length in a window
  // are grouped in ascending key order), n_rows values, or null.
  const int32_t* row_key = nullptr;
};

// Host-side arrays of a built sliced matrix.
struct SlicedHost;
// `vpe` values per entry: 1 for the sliced format (one nonzero per entry),
// the block width for the dense-block format (entry = block start column +
// that many consecutive zero-padded values).
// `keep` (optional, n_rows flags): rows with keep[r] == 0 get no task at all
// (another plan writes their y).
SlicedHost* sliced_build(int64_t n_rows, int64_t n_cols, const int64_t* row_ptr_or_null,
                         const uint64_t* row_ptr64_or_null, const int32_t* col_or_null,
                         const uint64_t* col64_or_null, const void* val, int value_bytes, const SlicedParams& prm,
                         int vpe = 1, const uint8_t* keep = nullptr);
void sliced_free(SlicedHost* h);
// Uploads a built matrix; device buffers are owned by the caller-provided allocator.
struct SlicedHostView {
  int64_t entries, num_tasks, num_long, num_chunks, n_rowid;
  const SlicedTask* tasks;
  const void* val;
  const int32_t* col;
  const int32_t* rowid;
  const int32_t* long_row;
  const int32_t* long_first;
  int vpe;
  const uint16_t* col16;  // delta tasks' column deltas (entries), or null
  const int32_t* first;   // first column of each row slot (n_rowid), or null
  // Windows of window_rows rows in row order: tasks, long rows and entries of
  // window w start at win_task[w], win_long[w], win_entry[w].
  int64_t num_windows;
  const int64_t* win_task;
  const int64_t* win_long;
  const int64_t* win_entry;
  int64_t delta_nnz, delta_rows;  // nonzeros and rows stored with 16-bit column deltas
  const uint16_t* pat16;          // shared-pattern deltas (entries / 32 + 64), or null
  int64_t shared_nnz, shared_steps;  // nonzeros and steps of shared-pattern tasks
};
SlicedHostView sliced_view(const SlicedHost* h);

// Fused output transform: y := alpha * (A x) + beta * z + gamma (z may be
// null, or alias y: each y entry is read and written by one thread).
struct SlicedEpilogue {
  double alpha = 1.0, beta = 0.0, gamma = 0.0;
  const void* z = nullptr;
  // Optional device scalar: gamma + gamma_dev_scale * *gamma_dev, read by the
  // kernel (a value an earlier launch on the stream computed).
  const double* gamma_dev = nullptr;
  double gamma_dev_scale = 0.0;
};

bool sliced_spmv(const SlicedMatrix& m, bool fp64, const void* x, void* y, cudaStream_t s,
                 cudaEvent_t* events = nullptr, const SlicedEpilogue* epi = nullptr);
// Gathers the hot-column window's x values of a call (the first step of the
// sliced kernel when hot_ready is false).
bool sliced_gather_hot(const SlicedMatrix& m, bool fp64, const void* x, cudaStream_t s);
// y[0..n) := alpha * y + beta * z + gamma (the unfused form of the epilogue).
bool apply_epilogue(void* y, long long n, bool fp64, const SlicedEpilogue& e, cudaStream_t s);

// Precision forms of the sliced format (sliced_mixed.cu).
enum SlicedPrecision : int { kPrecFP64 = 0, kPrecFP32 = 1, kPrecBF16 = 2, kPrecDF32 = 3 };
struct SlicedMixed {
  int precision = kPrecFP64;
  void* xbuf = nullptr;                    // n_cols converted x: float (FP32/BF16) or float2 (DF32)
  int* flag = nullptr;                     // DF32: x outside the split range this call
  const signed char* row_scale = nullptr;  // BF16: power-of-two exponent per row slot
  const signed char* chunk_scale = nullptr;  // BF16: exponent per chunk
  const float2* val_split = nullptr;         // DF32: values as FP32 (hi, lo) truncation-split pairs
};
bool sliced_mixed_spmv(const SlicedMatrix& m, const SlicedMixed& mx, const double* x, double* y, cudaStream_t s,
                       cudaEvent_t* events = nullptr);
// FP64 sliced kernel that only runs when *flag != 0 (DF32 fallback).
bool sliced_guard_f64(const SlicedMatrix& m, const double* x, double* y, const int* flag, cudaStream_t s);
// FP64 -> FP32 round-to-nearest-even of n values on stream s (one launch).
bool round_to_f32(const double* x, float* x32, long long n, cudaStream_t s);
// Truncation split of n FP64 values into FP32 (hi, lo) pairs; sets *flag when a
// nonzero value lies outside [2^-40, 2^41) (the caller clears it).
bool split_to_df32(const double* x, float2* xs, long long n, int* flag, cudaStream_t s);
inline int sliced_mixed_launches(const SlicedMatrix& m, int precision) {
  return 2 + (precision == kPrecDF32 ? 1 : 0) + (m.num_long > 0 || precision == kPrecDF32 ? 1 : 0) +
         (precision == kPrecDF32 && m.hot > 0 ? 1 : 0);
}
inline FixupGrid fixup_grid(const SlicedMatrix& m, int threads) {
  const int64_t light = (m.num_long + threads - 1) / threads;
  const int64_t heavy = (m.num_heavy * 32 + threads - 1) / threads;
  return FixupGrid{(unsigned)light, (unsigned)(light + heavy)};
}
inline int sliced_launches(const SlicedMatrix& m) { return (m.num_long > 0 ? 2 : 1) + (m.hot > 0 ? 1 : 0); }

}  // namespace vnec
