// Host-side plan machinery shared by the C-ABI translation units.
#pragma once

#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "common.h"
#include "sliced.h"
#include "vnec_gb300.h"

namespace vnec {

// A CSR matrix as handed in by a caller: either the reference's
// SpB_Matrix_CSC_or_CSR (64-bit offsets and columns) or raw arrays (int64
// offsets, int32 columns).
struct CsrView {
  SpB_Type type = SpB_FP64;
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  const SpB_Index* ptr64 = nullptr;  // reference layout
  const SpB_Index* idx64 = nullptr;
  const int64_t* ptr = nullptr;      // raw layout
  const int32_t* idx = nullptr;
  const void* val = nullptr;
  int64_t row_begin(int64_t r) const { return ptr64 ? (int64_t)ptr64[r] : ptr[r]; }
  int64_t col_at(int64_t p) const { return idx64 ? (int64_t)idx64[p] : idx[p]; }
  size_t value_bytes() const { return type == SpB_FP64 ? 8 : 4; }
};

bool view_from_matrix(const SpB_Matrix A, CsrView* v);
bool view_from_arrays(SpB_Type type, int64_t n_rows, int64_t n_cols, const int64_t* row_ptr, const int32_t* col,
                      const void* val, CsrView* v);
// Checks ptr[0]==0, monotone offsets, ptr[n]==nnz, 0<=col<n_cols (and, when
// `need_sorted`, strictly increasing columns per row).
bool validate_csr(const CsrView& v, bool need_sorted);
// CSR of the transpose (rows = the input's columns, each row's columns in
// increasing order) with a view over its arrays.
struct CsrTranspose {
  std::vector<int64_t> row_ptr;
  std::vector<int32_t> col;
  std::vector<unsigned char> val;
  CsrView view;
};
bool transpose_csr(const CsrView& v, CsrTranspose* t);
// Row ends (row_ptr[1..n]) as int32 or int64 and int32 columns.
void convert_row_end(const CsrView& v, bool wide, void* out);
void convert_cols(const CsrView& v, int32_t* out);

// Kinds of plans this library builds.
enum class PlanKind : int {
  kMergePath = 1, kWindowDense = 2, kWindowSliced = 3, kMixed = 4, kBatch = 5, kHybrid = 6, kPush = 7
};

// Base of every plan.  The reference-typed public struct handed to callers is
// a separate calloc'd block registered against the plan (see registry below).
struct Plan {
  PlanKind kind;
  SpB_Type type = SpB_FP64;  // value type of x and y
  int64_t n_rows = 0, n_cols = 0, nnz = 0;
  int rhs = 1;  // right-hand sides: x is n_cols x rhs, y is n_rows x rhs (row-major)
  int tune_config = -1;  // configuration index chosen by the tuner (tuner.h), -1 if built directly
  int tune_how = 0;      // SpB_VNEC_chosen_ext
  bool transposed = false;  // the plan computes y = A^T x (built from A's transpose)
  int device = 0;
  cudaStream_t own_stream = nullptr;
  DeviceBuffer dx, dy;  // staging for host-vector calls
  // The public handle carries NULL-filled per-partition pointer arrays
  // (Build_VNEC_S_* / Build_VNEC_D_*) that the release must free.
  bool pub_part_arrays = false;
  // Per-kernel timing of the most recent call (SpB_VNEC_set_profiling_ext).
  bool profiling = false;
  cudaEvent_t events[4] = {nullptr, nullptr, nullptr, nullptr};
  bool ensure_events();
  explicit Plan(PlanKind k) : kind(k) {}
  virtual ~Plan();
  virtual bool run(const void* d_x, void* d_y, cudaStream_t s) = 0;
  // y := alpha * (A x) + beta * z + gamma.  Default: the SpMV, then an
  // elementwise pass (z aliasing y is copied first); plans with a fused
  // epilogue override it.
  virtual bool run_epilogue(const void* d_x, void* d_y, const SlicedEpilogue& e, cudaStream_t s);
  DeviceBuffer epi_scratch;
  virtual int launches_per_call() const = 0;
  virtual int64_t device_bytes() const = 0;
  // Algorithmic bytes moved by one call (roofline numerator).
  virtual int64_t algorithmic_bytes() const = 0;
  // Kernel-specific fields of SpB_VNEC_info_ext.
  virtual void describe(SpB_VNEC_info_ext* info) const = 0;
  // Milliseconds of each kernel of the last profiled call (main kernel first).
  virtual int kernel_ms(float* ms, int cap) const = 0;
  // Waits for the plan's work on `s` and reports device-side errors.
  virtual bool device_status(cudaStream_t s) { return VNEC_CUDA(cudaStreamSynchronize(s)); }
  // Poll limit of the plan's bounded device waits (polls < 0: the default);
  // plans whose kernels never wait ignore it.
  virtual void set_wait_polls(int64_t polls) { (void)polls; }
  // y := A x with host vectors: copy x in, SpMV, copy y out, synchronise.
  virtual bool run_host(const void* h_x, void* h_y);
  std::mutex host_mu;  // serialises host-vector calls (they share dx, dy and own_stream)
  // Pipelined host-vector calls: enqueue returns at once; call i copies x in
  // on one stream, computes on a second and copies y out on a third, using
  // buffer slot i % 2, so call i+1's x copy and call i-1's y copy overlap
  // call i's SpMV.  host_wait() waits for every enqueued call.
  bool run_host_async(const void* h_x, void* h_y);
  bool host_wait();
  // Waits for the SpMVs of pipelined calls still in flight (they share the
  // plan's scratch with a synchronous host call); caller holds host_mu.
  bool drain_pipe() { return !pipe || VNEC_CUDA(cudaStreamSynchronize(pipe->comp)); }
  // The SpMV of one pipelined call (slot 0 or 1); default run().
  virtual bool run_slot(int slot, const void* d_x, void* d_y, cudaStream_t s) {
    (void)slot;
    return run(d_x, d_y, s);
  }
  struct HostPipe {
    cudaStream_t in = nullptr, comp = nullptr, out = nullptr;
    DeviceBuffer x[2], y[2];
    cudaEvent_t x_ready[2] = {nullptr, nullptr}, comp_done[2] = {nullptr, nullptr}, out_done[2] = {nullptr, nullptr};
    bool used[2] = {false, false};
    long long calls = 0;
    bool init(size_t xb, size_t yb);
    ~HostPipe();
  };
  std::unique_ptr<HostPipe> pipe;
};

// Registry: public handle pointer -> plan.
void register_plan(const void* handle, std::unique_ptr<Plan> plan);
Plan* find_plan(const void* handle);
std::unique_ptr<Plan> take_plan(const void* handle);

// Plan builders.
std::unique_ptr<Plan> build_merge_path(const CsrView& v, const SpB_VNEC_options_ext* opts);
// `keep` (optional): only rows with keep[r] != 0 are computed (the others' y is left alone).
std::unique_ptr<Plan> build_sliced(const CsrView& v, const SpB_VNEC_options_ext* opts, const uint8_t* keep = nullptr);
std::unique_ptr<Plan> build_dense(const CsrView& v, const SpB_VNEC_options_ext* opts, const uint8_t* keep = nullptr);
// Row-level dense/sparse split between the two (options: dense_fill_permille).
std::unique_ptr<Plan> build_hybrid(const CsrView& v, const SpB_VNEC_options_ext* opts);
// Plans of kernel LEARNED / SEARCH / RULE (tuner.cpp).
std::unique_ptr<Plan> build_tuned(const CsrView& v, const SpB_VNEC_options_ext* opts);
// Push plans (SpMSpV, push_plan.cpp) and their sparse-x calls.
std::unique_ptr<Plan> build_push(const CsrView& v, const SpB_VNEC_options_ext* opts);
bool push_run_sparse(Plan* p, long long nx, const int32_t* d_idx, const void* d_val, void* d_y, cudaStream_t s);
bool push_run_sparse_host(Plan* p, long long nx, const int32_t* idx, const void* val, void* y);
// Batched multi-right-hand-side plan over n CSR matrices (all FP64).
std::unique_ptr<Plan> build_batch(int n, const CsrView* mats, int k, const SpB_VNEC_batch_options_ext* opts);
// Row and column offsets of each matrix in a batch plan's concatenation (n + 1 each).
bool batch_offsets(const Plan* p, int64_t* row_off, int64_t* col_off);
int batch_size(const Plan* p);
// Autotuner record of a batch plan (see SpB_VNEC_batch_tuning_ext); -1 if p is not a batch plan.
int batch_tuning(const Plan* p, int* configs, float* ms, int cap, int* best);

// Reference partition count and lane width constants used by IRD_VNEC.
struct IrdParams {
  int nparts;
  int nlanes;
  float threshold;
};
IrdParams ird_params(SpB_Type type);
// IRD = nnz / (blocks * nlanes) as IRD_VNEC computes it (ird_calc.c:2-122).
float ird_ratio(const CsrView& v, const IrdParams& p);

}  // namespace vnec
